"""Subtree-box pruning leaves every traversal result unchanged.

The GPU traversal skips children whose padded subtree box the ray misses;
the oracle walks the NMH exactly as intersect()/intersectAny() (no boxes).
Hits, distances and occluders must agree bit for bit, including on the cases
that stress a box test: zero direction components, rays starting on box
faces and triangle vertices, flat (axis-aligned) triangles, coordinates far
from the origin and grazing rays."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu


def _check(ctx, V, rays):
    import torch
    Vd = torch.from_numpy(np.ascontiguousarray(V, np.float32).reshape(-1)).cuda()
    nmh = api.Nmh(ctx, Vd, count=V.shape[0])
    perm, verts = nmh.export()
    rd = api.rays_tensor(rays)
    hits = api.hits_to_numpy(api.trace_closest(ctx, nmh, rd))
    occ = api.trace_any(ctx, nmh, rd).cpu().numpy().view(np.uint32)
    ohits, _, otot = oracle.trace_closest(verts, perm, rays)
    oocc, _, atot = oracle.trace_any(verts, perm, rays)
    assert np.array_equal(hits.view(np.uint32), ohits.view(np.uint32))
    assert np.array_equal(occ, oocc)
    work = api.trace_stats(ctx, nmh, rd)
    assert work["closest"]["node_fetches"] <= otot and work["any"]["node_fetches"] <= atot
    for w in work.values():
        assert w["box_loads"] <= w["slab_crossings"] <= w["node_fetches"]
    return hits, work, otot


def _rays(o, d, tmax=1.0e6):
    r = np.zeros(o.shape[0], T.ray_dtype)
    r["ox"], r["oy"], r["oz"] = o[:, 0], o[:, 1], o[:, 2]
    r["dx"], r["dy"], r["dz"] = d[:, 0], d[:, 1], d[:, 2]
    r["tmax"] = tmax
    return r


def test_microbench_sample_matches_oracle(ctx):
    """1M triangles and 2^18 rays drawn from the 2^24-ray microbench."""
    V = scenes.random_soup(1_000_000, seed=0)
    rays = scenes.microbench_rays(1 << 24, seed=1)
    sel = np.sort(np.random.default_rng(11).choice(rays.shape[0], 1 << 18, replace=False))
    hits, work, otot = _check(ctx, V, rays[sel])
    assert (hits["prim"] != T.NO_HIT).mean() > 0.5
    assert work["closest"]["node_fetches"] < 0.6 * otot        # the pruning does prune


def test_axis_aligned_rays_and_flat_triangles(ctx):
    rng = np.random.default_rng(3)
    n = 20000
    c = rng.integers(0, 64, size=(n, 3)).astype(np.float32) / 64.0      # lattice: many shared planes
    e = (rng.integers(1, 4, size=(n, 2)) / 256.0).astype(np.float32)
    flat = rng.integers(0, 3, size=n)
    p1, p2, p3 = c.copy(), c.copy(), c.copy()
    for i in range(n):                     # triangles in x=, y= or z= planes
        a, b = [q for q in range(3) if q != flat[i]]
        p2[i, a] += e[i, 0]
        p3[i, b] += e[i, 1]
    V = scenes.tris_to_soa(p1, p2, p3)
    m = 1 << 15
    o = rng.integers(-8, 72, size=(m, 3)).astype(np.float32) / 64.0       # on the lattice planes
    o[: m // 4] = p1[rng.integers(0, n, m // 4)]                          # from triangle vertices
    axis = rng.integers(0, 3, size=m)
    d = np.zeros((m, 3), np.float32)
    d[np.arange(m), axis] = np.where(rng.random(m) < 0.5, -1.0, 1.0)
    d[m // 2:] = rng.normal(size=(m - m // 2, 3)).astype(np.float32)     # half random
    d[m // 2: 3 * m // 4, rng.integers(0, 3)] = 0.0                       # ... with one zero component
    d = np.where(d == 0.0, np.float32(0.0), d)
    d[m // 2:] /= np.linalg.norm(d[m // 2:], axis=1, keepdims=True)
    d[-64:] = np.array([0.0, -0.0, 1.0], np.float32)                      # negative zero
    _check(ctx, V, _rays(o, d))


def test_far_from_origin_and_grazing(ctx):
    rng = np.random.default_rng(5)
    V = scenes.random_soup(50000, seed=7).reshape(-1, 3, 3)
    V = (V + np.array([1000.0, -2000.0, 500.0], np.float32)[:, None]).reshape(-1, 9).astype(np.float32)
    tri = V.reshape(-1, 3, 3)
    m = 1 << 15
    k = rng.integers(0, tri.shape[0], m)
    a, b = rng.random((2, m)).astype(np.float32)
    sw = a + b > 1
    a[sw], b[sw] = 1 - a[sw], 1 - b[sw]
    v1 = tri[k, :, 0]
    e1 = tri[k, :, 1] - v1
    e2 = tri[k, :, 2] - v1
    target = v1 + a[:, None] * e1 + b[:, None] * e2
    nrm = np.cross(e1, e2)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    inplane = e1 / np.linalg.norm(e1, axis=1, keepdims=True)
    mix = rng.uniform(1e-4, 0.05, size=(m, 1)).astype(np.float32)           # grazing angles
    d = (inplane + mix * nrm).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = (target - d * rng.uniform(0.001, 3.0, size=(m, 1)).astype(np.float32)).astype(np.float32)
    _check(ctx, V, _rays(o, d))
