"""The oracle (CPU restatement) against the reference's own code and known answers."""
import math

import numpy as np
import pytest

import oracle
from oracle import nmh_literal
from aurora_gb300 import scenes, types as T
from helpers import closest_vs_reference, load_golden


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    assert [hex(x) for x in oracle.philox([0, 0, 0, 0], [0, 0])] == \
        ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(x) for x in oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                                          [0xA4093822, 0x299F31D0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_sincos_accuracy():
    x = np.linspace(-math.pi / 4 - 0.01, 7 * math.pi / 4 + 0.01, 200001).astype(np.float32)
    s, c = oracle.sincos(x)
    x64 = x.astype(np.float64)
    assert np.abs(s - np.sin(x64)).max() < 2e-7
    assert np.abs(c - np.cos(x64)).max() < 2e-7


def _subtree(k, n):
    s, f, w = 0, k, 1
    while f < n:
        s += min(w, n - f)
        f, w = 2 * f + 1, 2 * w
    return s


def test_calc_partition_matches_heap_subtrees():
    for n in range(2, 1200):
        for k in range(n):
            if _subtree(k, n) > 1:
                L, R = oracle.calc_partition(2 * _subtree(k, n))
                assert L == 2 * _subtree(2 * k + 1, n) and R == 2 * _subtree(2 * k + 2, n)


@pytest.mark.parametrize("n", [2, 4, 6, 10, 34, 66, 130, 1000, 2050, 4096])
def test_canonical_build_equals_literal_rebuilder(n):
    for seed in range(50):
        V = scenes.random_soup(n, seed=seed + 17 * n)
        if not nmh_literal.has_key_ties(V):
            break
    assert np.array_equal(oracle.nmh_build(V)[0], nmh_literal.rebuild_nmh(V))


def test_build_invariants_with_ties():
    """On the Cornell box (heavy key ties) every node's slab bounds its subtree."""
    sc = scenes.cornell()
    perm, levels = oracle.nmh_build(sc.vertices)
    assert sorted(perm.tolist()) == list(range(sc.count))
    V = sc.vertices[perm]
    n = sc.count // 2
    mn = [V[:, 3 * a:3 * a + 3].min(1) for a in range(3)]
    mx = [V[:, 3 * a:3 * a + 3].max(1) for a in range(3)]

    def sub(k):
        out, stack = [], [k]
        while stack:
            q = stack.pop()
            if q < n:
                out += [2 * q, 2 * q + 1]
                stack += [2 * q + 1, 2 * q + 2]
        return out
    for k in range(n):
        a = ((k + 1).bit_length() - 1) % 3
        s = sub(k)
        assert min(mn[a][2 * k], mn[a][2 * k + 1]) == min(mn[a][i] for i in s)
        assert max(mx[a][2 * k], mx[a][2 * k + 1]) == max(mx[a][i] for i in s)


def test_build_edge_sizes():
    assert oracle.nmh_build(np.zeros((0, 9), np.float32))[1] == 0
    one = scenes.random_soup(1, seed=3)
    perm, lv = oracle.nmh_build(one)           # padded to 2
    assert lv == 1 and sorted(perm.tolist()) == [0, 1]
    perm, lv = oracle.nmh_build(scenes.random_soup(7, seed=4))
    assert lv == 3 and sorted(perm.tolist()) == list(range(8))


@pytest.mark.parametrize("name", ["soup2048", "cornell"])
def test_oracle_topology_matches_golden(name):
    g = load_golden(name)
    perm, levels = oracle.nmh_build(g["vertices"])
    assert np.array_equal(perm, g["perm"]) and levels == int(g["levels"])


@pytest.mark.parametrize("name", ["soup2048", "cornell"])
def test_oracle_traversal_matches_reference_golden(name):
    g = load_golden(name)
    Vn = oracle.gather9(g["vertices"], g["perm"])
    hits, _, _ = oracle.trace_closest(Vn, g["perm"], g["rays"])
    closest_vs_reference(hits, g["ref_tuv"], g["ref_prim"])
    occ, _, _ = oracle.trace_any(Vn, g["perm"], g["rays"])
    assert np.array_equal(occ, g["ref_any"])
    assert (hits["prim"] != T.NO_HIT).mean() > 0.3


def test_oracle_traversal_matches_live_reference():
    if oracle.ref_lib() is None:
        pytest.skip("reference source tree not present")
    V = scenes.random_soup(30000, seed=21)
    perm, _ = oracle.nmh_build(V)
    Vn = oracle.gather9(V, perm)
    rays = scenes.microbench_rays(1 << 13, seed=22)
    hits, _, _ = oracle.trace_closest(Vn, perm, rays)
    tuv, ids = oracle.ref_trace_closest(Vn, rays)
    ref_prim = np.where(ids >= 0, perm[np.maximum(ids, 0)], T.NO_HIT).astype(np.uint32)
    closest_vs_reference(hits, tuv, ref_prim)
    occ, _, _ = oracle.trace_any(Vn, perm, rays)
    aid = oracle.ref_trace_any(Vn, rays)
    assert np.array_equal(occ, np.where(aid >= 0, perm[np.maximum(aid, 0)], T.NO_HIT).astype(np.uint32))


def test_traversal_matches_brute_force():
    V = scenes.random_soup(5000, seed=8)
    perm, _ = oracle.nmh_build(V)
    Vn = oracle.gather9(V, perm)
    rays = scenes.microbench_rays(1 << 12, seed=9)
    hits, _, _ = oracle.trace_closest(Vn, perm, rays)
    bf = oracle.brute_closest(V, rays)
    assert np.array_equal(hits["prim"], bf["prim"]) and np.array_equal(hits["t"], bf["t"])


def test_render_golden_regression():
    g = load_golden("cornell")
    sc = scenes.cornell()
    ns = oracle.NmhScene(sc)
    for mode in (T.MODE_REFERENCE, T.MODE_PATH):
        img, _ = oracle.render(ns, T.render_params(32, 32, 4, 4, seed=0, mode=mode))
        assert np.array_equal(img, g["image_mode%d" % mode])


def test_render_sample_ranges_add_up():
    ns = oracle.NmhScene(scenes.cornell())
    full, _ = oracle.render(ns, T.render_params(16, 16, 4, 3, seed=5))
    part, _ = oracle.render(ns, T.render_params(16, 16, 4, 3, seed=5, sample_begin=0, sample_end=2))
    part, _ = oracle.render(ns, T.render_params(16, 16, 4, 3, seed=5, sample_begin=2, sample_end=4), accum=part)
    assert np.array_equal(full, part)


def test_render_counted_counts_fetches_and_shading_points():
    """The path-sampling roofline's units: the counted render gives the same
    image; in reference mode without specular shaders every sample is shaded
    exactly once per camera hit, and path mode adds one shading point per
    bounce that hits."""
    from aurora_gb300 import scenes, types as T
    ns = oracle.NmhScene(scenes.cornell())
    p = T.render_params(16, 16, 4, 3, seed=2, mode=T.MODE_REFERENCE)
    img, fetches, shaded = oracle.render_counted(ns, p)
    ref, fetches2 = oracle.render(ns, p)
    assert np.array_equal(img, ref) and fetches == fetches2
    hits = int(round(img[..., 3].sum() * 4))                       # alpha: 1/spp per hitting sample
    assert shaded == hits
    pp = T.render_params(16, 16, 4, 3, seed=2, mode=T.MODE_PATH)
    _, _, shaded_path = oracle.render_counted(ns, pp)
    assert hits < shaded_path <= 4 * hits
