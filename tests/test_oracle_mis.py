"""The oracle's AUR_MODE_PATH_MIS estimator: its light-selection table, and
unbiasedness of both strategies against independent estimates (pure BSDF
sampling through path mode, and quadrature of the area-light integral)."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import scenes, types as T


def _means(ns, mode, depth, seeds, W=16, spp=1024):
    out = []
    for seed in range(seeds):
        img, _ = oracle.render(ns, T.render_params(W, W, spp, depth, seed=seed, mode=mode))
        out.append(img[..., :3].mean())
    return np.array(out)


def _z(a, b):
    """z-score of the difference of two sets of independent estimates."""
    se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    return abs(a.mean() - b.mean()) / se


def test_table_excludes_the_padding_copy_and_normalises():
    sd = scenes.cornell_emissive()
    assert sd.count % 2 == 1                                # the padding duplicates the last emitter
    ns = oracle.NmhScene(sd)
    tri, cdf, pa = oracle.mis_table(ns)
    assert len(tri) == 15                                   # 2 lamp + 12 block + 1 wall triangles
    assert np.all(ns.perm[tri] < sd.count)                  # the copy (perm == count) is left out
    assert np.all(np.diff(tri.astype(np.int64)) > 0)        # NMH order
    assert np.all(np.diff(cdf) >= 0) and cdf[-1] == np.float32(1.0)
    V = ns.V[tri]
    v1, v2, v3 = V[:, 0::3], V[:, 1::3], V[:, 2::3]
    area = 0.5 * np.linalg.norm(np.cross(v2 - v1, v3 - v1), axis=1)
    assert abs(float(np.sum(pa[tri] * area)) - 1.0) < 1e-5  # probabilities sum to one
    assert np.count_nonzero(pa) == len(tri)
    # selection follows emission * area: the lamp (weight 1) against the block (weight 0.5)
    psel = np.diff(np.concatenate([[0.0], cdf]))
    w = ns.shaders["emission"][ns.S[tri].astype(np.int64) - 1] * area
    assert np.allclose(psel, w / w.sum(), rtol=1e-5)


def test_table_of_a_scene_without_emitters_is_empty():
    tri, cdf, pa = oracle.mis_table(oracle.NmhScene(scenes.cornell()))
    assert len(tri) == 0 and not np.any(pa)


def test_emitter_sampling_matches_bsdf_sampling():
    """Emissive geometry only: MIS at depth d sees the paths path mode sees
    at depth d + 1 (its last hit samples the emitters with full weight), so
    their expectations agree; d = 0 compares pure emitter sampling with pure
    BSDF sampling."""
    ns = oracle.NmhScene(scenes.cornell_emissive())
    for d in (0, 1):
        mis = _means(ns, T.MODE_PATH_MIS, d, 8)
        path = _means(ns, T.MODE_PATH, d + 1, 8)
        assert _z(mis, path) < 4.0, (d, mis.mean(), path.mean())
        assert mis.std() < 0.5 * path.std()                  # the point of the exercise


def test_area_light_matches_quadrature():
    """A floor under a 0.5 x 0.5 area light at height 0.4, seen from above
    (depth 0, one camera ray per pixel, 4096 samples per strategy): each
    pixel against the midpoint-rule integral
    (rho / pi) I h^3 / r^5 dA of the reference's emission model."""
    h, I, rho = 0.4, 2.0, 0.6
    p1, p2, p3 = scenes._quad((-2, 0, -2), (3, 0, -2), (3, 0, 3), (-2, 0, 3), (0, 1, 0))
    fn = scenes.face_normals(p1, p2, p3)
    light = T.area_light((0.25, h, 0.25), (0.5, 0.0, 0.0), (0.0, 0.0, 0.5), (0.0, -1.0, 0.0), intensity=I,
                         samples=4096)
    cam = scenes.make_camera((0.5, 1.6, -0.6), (0.0, -1.6, 1.1), 0.6, 0.6)
    sd = scenes.SceneData("floor", scenes.tris_to_soa(p1, p2, p3), scenes.normals_to_aos(fn, fn, fn),
                          np.ones(2, np.uint16), np.stack([T.lambert((rho, rho, rho))]), np.stack([light]), cam)
    W = 12
    img, _ = oracle.render(oracle.NmhScene(sd), T.render_params(W, W, 1, 0, seed=5, mode=T.MODE_PATH_MIS))
    rays = oracle.generate_rays(cam, W, W, 0, 1)
    o = rays["pos"].reshape(-1, 3).astype(np.float64)
    d = rays["dir"].reshape(-1, 3).astype(np.float64)
    x = o + d * (-o[:, 1:2] / d[:, 1:2])
    g = (np.arange(400) + 0.5) / 400 * 0.5
    lx, lz = np.meshgrid(0.25 + g, 0.25 + g, indexing="ij")
    r2 = (lx.ravel()[None, :] - x[:, 0:1]) ** 2 + h * h + (lz.ravel()[None, :] - x[:, 2:3]) ** 2
    ref = rho / np.pi * I * np.sum(h ** 3 / r2 ** 2.5, axis=1) * (0.5 / 400) ** 2
    got = img.reshape(-1, 4)[:, 0]
    assert np.all(img.reshape(-1, 4)[:, 3] == 1.0)
    assert np.ptp(x[:, 0]) > 0.5 and np.ptp(x[:, 2]) > 0.5        # the view spans the lit region
    rel = got / ref - 1.0
    assert abs(rel.mean()) < 0.003 and np.max(np.abs(rel)) < 0.05, (rel.mean(), np.abs(rel).max())


def test_reference_and_path_modes_are_unchanged_by_the_table():
    """A scene with emitters renders the same in the other two modes whether
    or not MIS rendered it before (the table is MIS-only state)."""
    ns = oracle.NmhScene(scenes.cornell_emissive(area_light=True))
    for mode in (T.MODE_REFERENCE, T.MODE_PATH):
        p = T.render_params(8, 8, 4, 2, seed=3, mode=mode)
        a, _ = oracle.render(ns, p)
        oracle.render(ns, T.render_params(8, 8, 4, 2, seed=3, mode=T.MODE_PATH_MIS))
        b, _ = oracle.render(ns, p)
        assert np.array_equal(a, b)
