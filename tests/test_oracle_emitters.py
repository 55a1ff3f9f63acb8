"""Known answers for the oracle's emitter table (cudaCreateEmitters)."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import scenes, types as T


def _scene(V, emissions):
    n = V.shape[0]
    sh = np.stack([T.lambert((0.5, 0.5, 0.5)) for _ in emissions])
    sh["emission"] = emissions
    sh["emission_color"] = np.stack([np.full(3, k + 1, np.float32) for k in range(len(emissions))])
    sids = (np.arange(n) % len(emissions) + 1).astype(np.uint16)
    return scenes.SceneData("t", V, np.zeros_like(V), sids, sh, np.zeros(0, T.light_dtype), scenes.cornell_camera())


def test_right_triangles_areas_and_cdf():
    # triangles (0,0,0) (s,0,0) (0,s,0): area s^2 / 2
    s = np.array([1.0, 2.0, 0.5, 3.0], np.float32)
    p1 = np.zeros((4, 3), np.float32)
    p2 = np.stack([s, 0 * s, 0 * s], 1)
    p3 = np.stack([0 * s, s, 0 * s], 1)
    sd = _scene(scenes.tris_to_soa(p1, p2, p3), [1.0, 0.0, 3.0, 0.0])   # triangles 0 and 2 emit
    ns = oracle.NmhScene(sd, perm=np.arange(4, dtype=np.uint32))
    e = oracle.emitters(ns)
    assert list(e["triangle_id"]) == [0, 2]
    assert np.allclose(e["area"], [0.5, 0.125]) and np.allclose(e["pdf"], [2.0, 8.0])
    assert np.allclose(e["cdf"], [0.25, 1.0])
    assert np.array_equal(e["power"][:, 0], [1.0, 3.0])


def test_cdf_is_monotone_and_ends_at_one():
    V = scenes.random_soup(5000, seed=4)
    sd = _scene(V, list(np.random.default_rng(1).uniform(0, 2, size=37) * (np.arange(37) % 3 > 0)))
    e = oracle.emitters(oracle.NmhScene(sd))
    assert len(e) > 1000 and np.all(np.diff(e["cdf"]) >= 0) and e["cdf"][-1] == np.float32(1.0)


def test_areas_match_the_reference_primitive_area():
    """The emitter table's areas are Primitive3::area (primitive.cuh:74-85),
    compiled from the reference's own header: bit for bit, on a random soup
    and on degenerate triangles."""
    if oracle.ref_lib() is None:
        pytest.skip("the reference sources are not on this machine")
    V = scenes.random_soup(3000, seed=9)
    V[:5] = V[5]                                               # duplicates
    V[10, 0:3] = V[10, 0]                                      # zero extent in x
    V[11] = 0.0                                                # a point
    sh = np.stack([T.lambert((0.5, 0.5, 0.5))])
    sh["emission"] = 1.0
    sd = scenes.SceneData("t", V, np.zeros_like(V), np.ones(V.shape[0], np.uint16), sh, np.zeros(0, T.light_dtype),
                          scenes.cornell_camera())
    ns = oracle.NmhScene(sd)
    e = oracle.emitters(ns)
    ref = oracle.ref_triangle_areas(ns.V)
    assert np.array_equal(e["area"].view(np.uint32), ref[e["triangle_id"]].view(np.uint32))
