"""aur_scene_emitters (cudaCreateEmitters) on the GPU against the oracle:
ids, areas, pdfs and powers bit for bit; the CDF within float rounding
(both sum in double, in different orders)."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu


def _emissive_soup(n, n_shaders, seed):
    rng = np.random.default_rng(seed)
    V = scenes.random_soup(n, seed=seed)
    sh = np.stack([T.lambert(tuple(rng.uniform(0.2, 0.8, 3))) for _ in range(n_shaders)])
    sh["emission"] = np.where(rng.random(n_shaders) < 0.3, rng.uniform(0.1, 5.0, n_shaders), 0.0)
    sh["emission_color"] = rng.uniform(0, 4, size=(n_shaders, 3))
    sids = rng.integers(0, n_shaders + 1, size=n).astype(np.uint16)      # 0 selects shader 0
    return scenes.SceneData("soup", V, np.zeros_like(V), sids, sh, np.zeros(0, T.light_dtype),
                            scenes.cornell_camera())


@pytest.mark.parametrize("n,n_shaders", [(1, 1), (3001, 7), (100000, 200), (2_500_000, 1000)])
def test_emitters_match_oracle(ctx, n, n_shaders):
    sd = _emissive_soup(n, n_shaders, seed=n)
    sc = api.Scene(ctx, sd)
    perm, _ = sc.nmh.export()
    got = sc.emitters()
    ref = oracle.emitters(oracle.NmhScene(sd, perm=perm))
    assert got.shape == ref.shape
    for f in ("triangle_id", "area", "pdf", "power"):
        assert np.array_equal(got[f].view(np.uint32), ref[f].view(np.uint32)), f
    if len(ref):
        assert np.allclose(got["cdf"], ref["cdf"], rtol=2 ** -22, atol=0)
        assert got["cdf"][-1] == np.float32(1.0)


def test_no_emitters(ctx):
    sc = api.Scene(ctx, scenes.cornell())
    assert sc.emitters().shape == (0,)
