"""GPU NMH build against the oracle: topology bit-exact, deterministic."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes
from helpers import load_golden

pytestmark = pytest.mark.gpu


def _gpu_build(ctx, V):
    import torch
    Vd = torch.from_numpy(np.ascontiguousarray(V, np.float32).reshape(-1)).cuda()
    nmh = api.Nmh(ctx, Vd, count=V.shape[0])
    perm, verts = nmh.export()
    count, levels = nmh.info()
    return nmh, perm, verts, levels


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 33, 34, 100, 1001, 2047, 2048, 2049, 2050, 3071, 4096, 4099,
                               8191, 65537, 300000])
def test_build_matches_oracle(ctx, n):
    V = scenes.random_soup(n, seed=n)
    nmh, perm, verts, levels = _gpu_build(ctx, V)
    operm, olv = oracle.nmh_build(V)
    assert levels == olv
    assert np.array_equal(perm, operm)
    assert np.array_equal(verts, oracle.gather9(oracle.pad_even(V), operm))


@pytest.mark.parametrize("maker", ["cornell", "cornell_sphere", "terrain64", "spheres"])
def test_build_with_key_ties(ctx, maker):
    sd = {"cornell": scenes.cornell, "cornell_sphere": scenes.cornell_sphere,
          "terrain64": lambda: scenes.terrain(res=64, seed=2), "spheres": lambda: scenes.sphere_scene(3)}[maker]()
    _, perm, _, _ = _gpu_build(ctx, sd.vertices)
    assert np.array_equal(perm, oracle.nmh_build(sd.vertices)[0])


@pytest.mark.parametrize("name", ["soup2048", "cornell"])
def test_build_matches_golden(ctx, name):
    g = load_golden(name)
    _, perm, _, levels = _gpu_build(ctx, g["vertices"])
    assert np.array_equal(perm, g["perm"]) and levels == int(g["levels"])


def test_build_is_deterministic(ctx):
    V = scenes.random_soup(200000, seed=77)
    V[1000:2000] = V[0]                 # many exact duplicates -> key ties everywhere
    _, p1, _, _ = _gpu_build(ctx, V)
    _, p2, _, _ = _gpu_build(ctx, V)
    assert np.array_equal(p1, p2)
    assert np.array_equal(p1, oracle.nmh_build(V)[0])


def test_empty_build(ctx):
    nmh, perm, verts, levels = _gpu_build(ctx, np.zeros((0, 9), np.float32))
    assert levels == 0 and perm.size == 0


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_non_finite_vertices_are_refused(ctx, bad):
    """The reference's float sorts have no order for NaN: a soup with a NaN or
    infinite coordinate is refused (AUR_ERR_INVALID), and the context then
    builds a finite soup normally."""
    import torch
    V = scenes.random_soup(5001, seed=6)
    V[4321, 4] = bad
    Vd = torch.from_numpy(np.ascontiguousarray(V, np.float32).reshape(-1)).cuda()
    with pytest.raises(api.AuroraError) as e:
        api.Nmh(ctx, Vd, count=V.shape[0])
    assert e.value.status == 1 and "NaN or infinite" in str(e.value)
    V[4321, 4] = 0.5
    _, perm, _, _ = _gpu_build(ctx, V)
    assert np.array_equal(perm, oracle.nmh_build(V)[0])
