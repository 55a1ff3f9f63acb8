"""Pins the pieces of the MIS mode that the reference has to the
reference's own code, compiled as host C++ (oracle/ref_shim/ref_shade.cpp):
BSDF::samplef at real hits with the tangent frames of cudaGenerateTB (path
mode's bounce; directions to a few ulp, the disk mapping's sin / cos being
this build's own; the MIS mode samples in an orthonormal frame instead and
is checked for its density), powerHeuristic (the same weight,
written so that it cannot overflow), and Light::visibleArea's ray / quad
test (the same hits and distances where the reference sees the quad). The solid-angle
light density is the one the reference leaves commented out in
Light::pdf (light.cuh:87)."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import scenes, types as T


def _need_reference():
    if oracle.ref_lib() is None:
        pytest.skip("the reference sources are not on this machine")


def _hits(W=40, H=36):
    sd = scenes.cornell_sphere(seed=4, slices=24, stacks=12)
    ns = oracle.NmhScene(sd)
    pr = oracle.generate_rays(ns.camera, W, H, 0, 1)
    rays = np.zeros(W * H, T.ray_dtype)
    rays["ox"], rays["oy"], rays["oz"] = pr["pos"][:, 0], pr["pos"][:, 1], pr["pos"][:, 2]
    rays["dx"], rays["dy"], rays["dz"] = pr["dir"][:, 0], pr["dir"][:, 1], pr["dir"][:, 2]
    rays["tmax"] = pr["t"]
    tuv, ids = oracle.ref_trace_closest(ns.V, rays)
    assert (ids >= 0).mean() > 0.9
    return ns, rays.view(np.float32).reshape(-1, 8), ids, tuv


def test_path_bounce_matches_the_reference_samplef():
    """Path mode's diffuse bounce is BSDF::samplef in the reference's own
    (interpolated, not orthonormal) tangent frame."""
    _need_reference()
    ns, r8, ids, tuv = _hits()
    n = r8.shape[0]
    tg, bt = oracle.generate_tb(ns.N)
    rng = np.random.default_rng(3)
    u = rng.uniform(0.0, 1.0, size=(n, 2)).astype(np.float32)
    u[:4] = [[1.0, 1.0], [0.5, 0.5], [1.0, 0.5], [2.0 ** -24, 1.0]]     # edge draws of (0, 1]
    probes = np.zeros((n, 3), np.float32)
    mine = oracle.bsdf_hits(ns, r8, ids, tuv, u, probes)
    # the reference draws samplef's two uniforms in the order its compiler
    # evaluates the arguments (probed on Light::sampleL)
    ru = u[:, ::-1] if oracle.ref_uniform_order() == 1 else u
    ref = oracle.bsdf_hits(ns, r8, ids, tuv, np.ascontiguousarray(ru), probes, tg, bt, reference=True)
    hit = ids >= 0
    # the disk mapping's sin / cos are this build's own (the reference calls
    # the device's or the C library's sinf / cosf): directions agree to a few
    # ulp, most of them bit for bit
    assert np.max(np.abs(mine[hit, :3] - ref[hit, :3])) <= 2e-6
    assert np.mean(np.all(mine[hit, :3] == ref[hit, :3], axis=1)) > 0.5
    assert np.max(np.abs(mine[hit, 3] - ref[hit, 3])) <= 2e-6     # near-grazing samples amplify the ulp
    # that frame is not orthonormal on the sphere: samplef's density differs
    # from the density of the direction it returns, by up to a few percent
    assert np.max(np.abs(ref[hit, 3] - ref[hit, 4])) > 1e-3


def test_mis_sampling_is_consistent():
    """The MIS mode samples in an orthonormal frame about N: unit directions,
    the returned density is exactly bsdf_pdf of the returned direction, and
    over many samples cos(theta) has the cosine law's mean 2/3 and
    second moment 1/2."""
    ns, r8, ids, tuv = _hits()
    n = r8.shape[0]
    rng = np.random.default_rng(4)
    u = rng.uniform(0.0, 1.0, size=(n, 2)).astype(np.float32)
    got = oracle.bsdf_hits(ns, r8, ids, tuv, u, np.zeros((n, 3), np.float32), mis=True)
    hit = ids >= 0
    assert np.max(np.abs(np.linalg.norm(got[hit, :3], axis=1) - 1.0)) < 1e-6
    assert np.array_equal(got[hit, 3], got[hit, 4]) and np.all(got[hit, 3] > 0)
    # one curved-surface hit, 20000 samples
    k = int(np.flatnonzero(hit & (tuv[:, 0] > 0))[n // 3 % hit.sum()])
    m = 20000
    u = rng.uniform(0.0, 1.0, size=(m, 2)).astype(np.float32)
    rep = lambda a: np.repeat(a[k:k + 1], m, axis=0)
    g = oracle.bsdf_hits(ns, rep(r8), rep(ids), rep(tuv), u, np.zeros((m, 3), np.float32), mis=True)
    cos = g[:, 3] * np.pi                                                # |cos| against N
    assert abs(cos.mean() - 2.0 / 3.0) < 0.01 and abs((cos ** 2).mean() - 0.5) < 0.01


def test_power_heuristic_matches_the_reference():
    _need_reference()
    rng = np.random.default_rng(5)
    a = np.exp(rng.uniform(-20, 20, 2000)).astype(np.float32)
    b = np.exp(rng.uniform(-20, 20, 2000)).astype(np.float32)
    for x, y in zip(a, b):
        m, r = oracle.mis_weight(float(x), float(y)), oracle.mis_weight(float(x), float(y), reference=True)
        assert abs(m - r) <= 2e-7 + 2e-6 * r, (x, y, m, r)
    assert oracle.mis_weight(1.0, 0.0) == 1.0 and oracle.mis_weight(1e30, 1e-30) == 1.0
    assert oracle.mis_weight(1e-30, 1e30) == 0.0                        # no inf / inf


def test_quad_hit_matches_visible_area():
    """visibleArea tests the quad as two triangles with the culled
    Moller-Trumbore: from the emitting side it sees only the triangle
    (position, position + e1, position + e2), whose winding faces that way,
    and misses the other half (a + b > 1), which faces the other way. The
    MIS mode's quad test takes both halves from either side (the emitting
    side is chosen by cos_l > 0); where the reference sees the quad, both
    give the same hit and distance."""
    _need_reference()
    rng = np.random.default_rng(7)
    L = T.area_light((0.2, 0.9, 0.3), (0.5, 0.0, 0.1), (-0.1, 0.0, 0.4), (0.0, -1.0, 0.0), samples=1)
    p0, e1, e2 = (np.asarray(L[k], np.float64) for k in ("position", "e1", "e2"))
    seen = {"same": 0, "far half": 0, "outside": 0}
    for _ in range(3000):
        a, b = rng.uniform(-0.3, 1.3, 2)
        if min(abs(a), abs(a - 1), abs(b), abs(b - 1), abs(a + b - 1)) < 1e-4:
            continue                                                    # on an edge: rounding decides
        target = p0 + a * e1 + b * e2
        pos = rng.uniform(0.0, 1.0, 3) * [1.0, 0.85, 1.0]                 # below the light: its lit side
        d = target - pos
        d /= np.linalg.norm(d)
        hm, tm = oracle.area_hit(L, pos, d)
        hr, tr = oracle.area_hit(L, pos, d, reference=True)
        inside = 0 <= a <= 1 and 0 <= b <= 1
        assert hm == inside, (a, b)
        if not inside:
            assert not hr
            seen["outside"] += 1
        elif a + b < 1:
            assert hr and abs(tm - tr) <= 1e-6 * tr, (a, b, tm, tr)
            seen["same"] += 1
        else:
            assert not hr                                               # the reference's culled half
            seen["far half"] += 1
    assert min(seen.values()) > 300, seen
