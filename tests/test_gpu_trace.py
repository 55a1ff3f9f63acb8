"""GPU closest-hit / any-hit traversal against the oracle and the reference goldens."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes, types as T
from helpers import closest_vs_reference, hits_equal, load_golden

pytestmark = pytest.mark.gpu


def _setup(ctx, V):
    import torch
    Vd = torch.from_numpy(np.ascontiguousarray(V, np.float32).reshape(-1)).cuda()
    nmh = api.Nmh(ctx, Vd, count=V.shape[0])
    perm, verts = nmh.export()
    return nmh, perm, verts


def _gpu_trace(ctx, nmh, rays):
    rd = api.rays_tensor(rays)
    hits = api.hits_to_numpy(api.trace_closest(ctx, nmh, rd))
    occ = api.trace_any(ctx, nmh, rd).cpu().numpy().view(np.uint32)
    return hits, occ


@pytest.mark.parametrize("name", ["soup2048", "cornell"])
def test_trace_matches_reference_golden(ctx, name):
    g = load_golden(name)
    nmh, perm, verts = _setup(ctx, g["vertices"])
    hits, occ = _gpu_trace(ctx, nmh, g["rays"])
    closest_vs_reference(hits, g["ref_tuv"], g["ref_prim"])
    assert np.array_equal(occ, g["ref_any"])
    ohits, _, _ = oracle.trace_closest(verts, perm, g["rays"])
    assert hits_equal(hits, ohits)


@pytest.mark.parametrize("n_tris,n_rays", [(1000, 1 << 14), (100000, 1 << 16), (1000000, 1 << 15)])
def test_trace_matches_oracle(ctx, n_tris, n_rays):
    V = scenes.random_soup(n_tris, seed=n_tris)
    nmh, perm, verts = _setup(ctx, V)
    rays = scenes.microbench_rays(n_rays, seed=3)
    hits, occ = _gpu_trace(ctx, nmh, rays)
    ohits, ovis, otot = oracle.trace_closest(verts, perm, rays)
    oocc, avis, atot = oracle.trace_any(verts, perm, rays)
    assert hits_equal(hits, ohits)
    assert np.array_equal(occ, oocc)
    assert (hits["prim"] != T.NO_HIT).mean() > (0.2 if n_tris >= 100000 else 0.005)
    assert api.count_visits(ctx, nmh, api.rays_tensor(rays)) == (otot, atot)


@pytest.mark.parametrize("n_tris", [3000, 1000000])
def test_trace_texture_and_plain_loads_agree(ctx, n_tris):
    """The traversal entry points read part of each node through the records'
    texture; an NMH without one (too large for a texture) is read with plain
    loads. Both give the same hits, bit for bit, in closest and any hit."""
    V = scenes.random_soup(n_tris, seed=n_tris + 7)
    nmh, perm, verts = _setup(ctx, V)
    rays = scenes.microbench_rays(1 << 16, seed=5)
    hits_tex, occ_tex = _gpu_trace(ctx, nmh, rays)
    api.check(api.lib().aur_debug_nmh_drop_texture(nmh.handle))
    hits_plain, occ_plain = _gpu_trace(ctx, nmh, rays)
    assert hits_equal(hits_tex, hits_plain)
    assert np.array_equal(occ_tex, occ_plain)
    ohits, _, _ = oracle.trace_closest(verts, perm, rays)
    assert hits_equal(hits_plain, ohits)


def test_trace_tie_rule_on_duplicates(ctx):
    V = scenes.random_soup(4000, seed=5)
    V[3000:3100] = V[100:200]           # coincident copies: exact ties in t
    nmh, perm, verts = _setup(ctx, V)
    rng = np.random.default_rng(0)
    tri = np.concatenate([np.arange(100, 200), np.arange(3000, 3100)])
    c = np.stack([V[tri, 0:3].mean(1), V[tri, 3:6].mean(1), V[tri, 6:9].mean(1)], 1)
    o = c + rng.normal(size=c.shape) * 0.2
    d = c - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(len(tri), T.ray_dtype)
    rays["ox"], rays["oy"], rays["oz"] = o.T
    rays["dx"], rays["dy"], rays["dz"] = d.T
    rays["tmax"] = 1e6
    hits, _ = _gpu_trace(ctx, nmh, rays)
    ohits, _, _ = oracle.trace_closest(verts, perm, rays)
    assert hits_equal(hits, ohits)
    # a ray that hits a coincident pair reports the lower id of the two
    assert not np.any((hits["prim"] >= 3000) & (hits["prim"] < 3100))
    assert np.isin(hits["prim"], np.arange(100, 200)).sum() > 50


def test_trace_host_buffers_match_device(ctx):
    V = scenes.random_soup(50000, seed=9)
    nmh, perm, verts = _setup(ctx, V)
    # three pipeline chunks (2M, 4M + 12345, 2M): both launch streams, and slot 0 reused
    rays = scenes.microbench_rays((2 << 22) + 12345, seed=4)
    hits_d, occ_d = _gpu_trace(ctx, nmh, rays)
    hits_h = np.zeros(rays.shape[0], T.hit_dtype)
    occ_h = np.zeros(rays.shape[0], np.uint32)
    api.trace_closest_host(ctx, nmh, rays, hits_h)
    api.trace_any_host(ctx, nmh, rays, occ_h)
    assert hits_equal(hits_h, hits_d) and np.array_equal(occ_h, occ_d)


def test_trace_edge_cases(ctx):
    import torch
    V = scenes.random_soup(3, seed=1)                 # odd count -> padded
    nmh, perm, verts = _setup(ctx, V)
    rays = scenes.microbench_rays(64, seed=2)
    rays["tmax"][:8] = 1e-9                            # nothing closer than Epsilon
    hits, occ = _gpu_trace(ctx, nmh, rays)
    ohits, _, _ = oracle.trace_closest(verts, perm, rays)
    assert hits_equal(hits, ohits)
    assert np.all(hits["prim"][:8] == T.NO_HIT)
    empty = api.Nmh(ctx, torch.zeros(0, device="cuda"), count=0)
    h2, o2 = _gpu_trace(ctx, empty, rays)
    assert np.all(h2["prim"] == T.NO_HIT) and np.all(o2 == T.NO_HIT)
    assert np.array_equal(h2["t"], rays["tmax"])
    z = api.trace_closest(ctx, nmh, api.rays_tensor(rays[:0]))
    assert z.shape[0] == 0


def test_trace_non_finite_rays(ctx):
    """Rays with a NaN or infinite origin or direction component hit nothing,
    as the reference's arithmetic gives (NaN fails every t test), and do not
    disturb the other rays of the launch."""
    V = scenes.random_soup(20000, seed=8)
    nmh, perm, verts = _setup(ctx, V)
    rays = scenes.microbench_rays(4096, seed=9)
    bad = np.arange(0, 4096, 7)
    for j, k in enumerate(bad):
        field = ("ox", "oy", "oz", "dx", "dy", "dz")[j % 6]
        rays[field][k] = (np.nan, np.inf, -np.inf)[j % 3]
    hits, occ = _gpu_trace(ctx, nmh, rays)
    ohits, _, _ = oracle.trace_closest(verts, perm, rays)
    oocc, _, _ = oracle.trace_any(verts, perm, rays)
    assert hits_equal(hits, ohits) and np.array_equal(occ, oocc)
    nan_rays = bad[np.arange(len(bad)) % 3 == 0]
    assert np.all(hits["prim"][nan_rays] == T.NO_HIT)
    good = np.setdiff1d(np.arange(4096), bad)
    assert (hits["prim"][good] != T.NO_HIT).mean() > 0.05


def _octant_rays(n, seed, octant_of_chunk, spread=1.0):
    """Random directions whose signs are set per chunk of 32 rays by
    octant_of_chunk(chunk index) (bit a: dir[a] < 0); origins at a random
    point of the unit cube per chunk, plus U[0, spread)^3 per ray."""
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, T.ray_dtype)
    centre = np.repeat(rng.random(((n + 31) // 32, 3)), 32, axis=0)[:n]
    o = (centre * (1.0 - spread) + rng.random((n, 3)) * spread).astype(np.float32)
    d = np.abs(rng.normal(size=(n, 3)))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    oct_ = np.array([octant_of_chunk(i // 32) for i in range(n)])
    for a in range(3):
        d[:, a] = np.where((oct_ >> a) & 1, -d[:, a], d[:, a])
    rays["ox"], rays["oy"], rays["oz"] = o.T
    rays["dx"], rays["dy"], rays["dz"] = d.astype(np.float32).T
    rays["tmax"] = 1e6
    return rays


def _check_against_oracle(ctx, nmh, perm, verts, rays):
    hits, occ = _gpu_trace(ctx, nmh, rays)
    ohits, _, _ = oracle.trace_closest(verts, perm, rays)
    oocc, _, _ = oracle.trace_any(verts, perm, rays)
    assert hits_equal(hits, ohits)
    assert np.array_equal(occ, oocc)
    return hits


def test_packets_of_one_octant_match_oracle(ctx):
    """Chunks of rays from nearby origins with random directions of one
    octant (a different one per chunk) run as warp packets whose lanes' node
    sets differ widely; the last chunk is partial. The same directions from
    origins spread over the soup go one ray per lane (the packet test also
    asks for nearby origins). Closest and any hit equal the oracle."""
    V = scenes.random_soup(100000, seed=21)
    nmh, perm, verts = _setup(ctx, V)
    n = 32 * 700 + 13
    rays = _octant_rays(n, 4, lambda c: c % 8, spread=0.004)
    hits = _check_against_oracle(ctx, nmh, perm, verts, rays)
    assert api.trace_deferred(ctx) == 0
    assert (hits["prim"] != T.NO_HIT).mean() > 0.5
    spread = _octant_rays(n, 4, lambda c: c % 8)
    _check_against_oracle(ctx, nmh, perm, verts, spread)
    assert api.trace_deferred(ctx) == (n + 31) // 32


def test_packets_and_deferred_chunks_mixed(ctx):
    """Uniform and mixed-octant chunks in one launch, a partial mixed last
    chunk (its missing rays trace the last ray again), and packets of
    axis-parallel rays with +0 and -0 direction components (-0 is not
    negative: the same near child as +0, in packets and per lane)."""
    V = scenes.random_soup(20000, seed=22)
    nmh, perm, verts = _setup(ctx, V)
    n = 32 * 64 + 20
    rays = _octant_rays(n, 5, lambda c: (c * 5) % 8, spread=0.004)
    rng = np.random.default_rng(6)
    mixed = sorted({c for c in range(65) if c % 3 == 1} | {64})
    for c in mixed:                                   # flip one lane's x sign
        j = min(32 * c + 7, n - 1)
        rays["dx"][j] = -rays["dx"][j]
    ax = np.arange(32 * 3, 32 * 4)                    # a uniform chunk of axis-parallel rays
    rays["dx"][ax], rays["dy"][ax] = np.where(np.arange(32) % 2, -0.0, 0.0), 0.0
    rays["dz"][ax] = 1.0
    rays["ox"][ax], rays["oy"][ax] = 0.3 + 0.004 * rng.random(32), 0.6 + 0.004 * rng.random(32)
    rays["oz"][ax] = -1.0
    _check_against_oracle(ctx, nmh, perm, verts, rays)
    assert 3 not in mixed and 64 in mixed
    assert api.trace_deferred(ctx) == len(mixed)


def test_camera_rays_run_as_packets(ctx):
    """The microbench's pinhole half (rows of 4096 rays, no chunk across the
    image's centre column) is all packets; its random half all deferred."""
    V = scenes.random_soup(50000, seed=23)
    nmh, perm, verts = _setup(ctx, V)
    rays = scenes.microbench_rays(1 << 15, seed=7)
    _check_against_oracle(ctx, nmh, perm, verts, rays)
    deferred = api.trace_deferred(ctx)
    assert deferred <= (1 << 14) // 32 and deferred > (1 << 14) // 32 - 8
