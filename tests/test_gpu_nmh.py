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


def test_build_matches_oracle_on_the_traversal_benchmark_soup(ctx):
    """The 1,000,000-triangle soup the traversal benchmark builds and traces
    (random_soup(1_000_000, seed=0)), with its 19 levels: topology and the
    NMH-ordered vertices equal the oracle's."""
    V = scenes.random_soup(1_000_000, seed=0)
    nmh, perm, verts, levels = _gpu_build(ctx, V)
    operm, olv = oracle.nmh_build(V)
    assert levels == olv == 19
    assert np.array_equal(perm, operm)
    assert np.array_equal(verts.view(np.uint32), oracle.gather9(V, operm).view(np.uint32))


@pytest.mark.parametrize("maker", ["cornell", "cornell_sphere", "terrain64", "spheres"])
def test_build_with_key_ties(ctx, maker):
    sd = {"cornell": scenes.cornell, "cornell_sphere": scenes.cornell_sphere,
          "terrain64": lambda: scenes.terrain(res=64, seed=2), "spheres": lambda: scenes.sphere_scene(3)}[maker]()
    _, perm, _, _ = _gpu_build(ctx, sd.vertices)
    assert np.array_equal(perm, oracle.nmh_build(sd.vertices)[0])


@pytest.mark.parametrize("n", [4097, 100001])
def test_build_of_identical_triangles(ctx, n):
    """Every key tied on every axis: the order comes from the prim ids alone,
    through the global levels and the per-subtree finish."""
    V = np.tile(scenes.random_soup(1, seed=5), (n, 1))
    _, perm, _, _ = _gpu_build(ctx, V)
    assert np.array_equal(perm, oracle.nmh_build(V)[0])


def _subtree_extremes(verts, levels):
    """Per node: the pair's min of the triangles' minima and max of their
    maxima on each axis, and the same over the node's whole subtree
    (bottom-up, one vectorised pass per level)."""
    mn = np.stack([verts[:, 3 * a:3 * a + 3].min(1) for a in range(3)], 1)
    mx = np.stack([verts[:, 3 * a:3 * a + 3].max(1) for a in range(3)], 1)
    pmn, pmx = np.minimum(mn[0::2], mn[1::2]), np.maximum(mx[0::2], mx[1::2])
    n = pmn.shape[0]
    smn, smx = pmn.copy(), pmx.copy()
    for lv in range(levels - 2, -1, -1):
        k = np.arange((1 << lv) - 1, min((2 << lv) - 1, n))
        for c in (2 * k + 1, 2 * k + 2):
            ok = c < n
            smn[k[ok]] = np.minimum(smn[k[ok]], smn[c[ok]])
            smx[k[ok]] = np.maximum(smx[k[ok]], smx[c[ok]])
    return pmn, pmx, smn, smx


def test_build_and_trace_beyond_the_largest_workload(ctx):
    """2^24 + 3 triangles, twice the 8.4M-triangle terrain (the oracle's build
    would take minutes here, so the tree is checked by its properties): the
    NMH-ordered soup is the padded input gathered by a permutation; every
    node's pair holds the extremes of its subtree on the node's axis (the
    property that makes the pair's slab a bound of the subtree, over all 24
    levels); and closest and any hits of 2^13 microbench rays equal the
    oracle's traversal of the exported tree bit for bit."""
    V = scenes.random_soup((1 << 24) + 3, seed=24)
    nmh, perm, verts, levels = _gpu_build(ctx, V)
    N = V.shape[0] + 1
    n = N // 2
    assert perm.size == N and levels == n.bit_length()
    assert np.array_equal(np.bincount(perm, minlength=N), np.ones(N, np.int64))
    assert np.array_equal(verts, oracle.pad_even(V)[perm])
    pmn, pmx, smn, smx = _subtree_extremes(verts, levels)
    axis = np.zeros(n, np.int64)
    for lv in range(levels):
        axis[(1 << lv) - 1:min((2 << lv) - 1, n)] = lv % 3
    k = np.arange(n)
    assert np.array_equal(pmn[k, axis], smn[k, axis]) and np.array_equal(pmx[k, axis], smx[k, axis])
    rays = scenes.microbench_rays(1 << 13, seed=25)
    hits = api.hits_to_numpy(api.trace_closest(ctx, nmh, api.rays_tensor(rays)))
    ohits, _, _ = oracle.trace_closest(verts, perm, rays)
    assert np.array_equal(hits.view(np.uint32), ohits.view(np.uint32))
    assert (ohits["prim"] != 0xFFFFFFFF).mean() > 0.3
    occ = api.trace_any(ctx, nmh, api.rays_tensor(rays)).cpu().numpy().view(np.uint32)
    assert np.array_equal(occ, oracle.trace_any(verts, perm, rays)[0])


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


def test_build_graph_reuse(ctx):
    """The context's build cache: the first build of a size launches
    directly, the second records the size's launch graph, later ones replay
    it with the new vertex and output buffers patched in; up to four sizes
    keep a graph. Every build, through each of the three ways and across
    evictions, equals the oracle's tree."""
    soups = {("a", 30001): scenes.random_soup(30001, seed=31), ("b", 30001): scenes.random_soup(30001, seed=32)}
    for i, n in enumerate((777, 1500, 2049, 4100, 9001)):
        soups[("s", n)] = scenes.random_soup(n, seed=40 + i)
    want = {k: oracle.nmh_build(V)[0] for k, V in soups.items()}
    order = [("a", 30001), ("b", 30001), ("a", 30001), ("s", 777), ("b", 30001)]
    sizes = [("s", n) for n in (777, 1500, 2049, 4100, 9001)]
    order += sizes + sizes + sizes[:2] + [("a", 30001)]
    for k in order:
        V = soups[k]
        _, perm, verts, _ = _gpu_build(ctx, V)
        assert np.array_equal(perm, want[k]), k
        assert np.array_equal(verts, oracle.gather9(oracle.pad_even(V), want[k])), k


def test_build_cache_across_streams(ctx):
    """Builds of one size from the context's cache on different launch
    streams: each waits for the previous one's use of the shared scratch."""
    import torch
    V = scenes.random_soup(20001, seed=51)
    want = oracle.nmh_build(V)[0]
    Vd = torch.from_numpy(V.reshape(-1)).cuda()
    streams = [torch.cuda.Stream() for _ in range(3)]
    try:
        for i in range(6):
            with torch.cuda.stream(streams[i % 3]):
                ctx.use_torch_stream()
                nmh = api.Nmh(ctx, Vd, count=V.shape[0])
                assert np.array_equal(nmh.export()[0], want), i
    finally:
        ctx.use_torch_stream()


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
