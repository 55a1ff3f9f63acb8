"""The allocation-free NMH build entry point (aur_nmh_build_noalloc).

It serves callers that cannot allocate device memory themselves, such as a
plug-in whose host application owns the GPU memory budget, or a render loop
that must avoid cudaMalloc/cudaFree. It must give exactly what aur_nmh_build
gives, also when called twice in a row (its shared scratch array still holds
the previous call's data), and must refuse soups above its fixed limit.
This file is collected last so that a failure here stops a -x run only after
every other test has run.
"""
import ctypes

import numpy as np
import pytest

from aurora_gb300 import api, scenes

pytestmark = pytest.mark.gpu

LIMIT = 1 << 16


def _stream_arg():
    import torch
    h = torch.cuda.current_stream().cuda_stream
    return ctypes.c_void_p(h if h else 0)      # NULL selects the legacy default stream


def _noalloc_build(V):
    """Builds through the C ABI into buffers allocated here, by the caller."""
    import torch
    count = V.shape[0]
    N = count + (count & 1)
    Vd = torch.from_numpy(np.ascontiguousarray(V, np.float32).reshape(-1)).cuda()
    recs = torch.full((max(N // 2, 1) * 32,), float("nan"), dtype=torch.float32, device="cuda")
    perm = torch.full((max(N, 1),), -1, dtype=torch.int32, device="cuda")
    verts = torch.full((max(N, 1) * 9,), float("nan"), dtype=torch.float32, device="cuda")
    levels = ctypes.c_uint32(0)
    api.check(api.lib().aur_nmh_build_noalloc(api._ptr(Vd), count, _stream_arg(), api._ptr(recs), api._ptr(perm),
                                              api._ptr(verts), ctypes.byref(levels)))
    return (recs.cpu().numpy()[:N // 2 * 32].reshape(-1, 32), perm.cpu().numpy()[:N].view(np.uint32),
            verts.cpu().numpy()[:N * 9].reshape(-1, 9), levels.value)


def _expected_records(verts):
    """Node records from the NMH-ordered soup: slab of the pair on the node's
    axis, each triangle as v1, v2 - v1, v3 - v1, then the padded subtree boxes
    of the two children (empty box (1, -1) where a child does not exist)."""
    n = verts.shape[0] // 2
    recs = np.zeros((n, 32), np.float32)
    box = np.zeros((n, 6), np.float32)
    for k in range(n):
        a = ((k + 1).bit_length() - 1) % 3
        t0, t1 = verts[2 * k], verts[2 * k + 1]
        for ax in range(3):
            box[k, ax] = min(t0[3 * ax:3 * ax + 3].min(), t1[3 * ax:3 * ax + 3].min())
            box[k, 3 + ax] = max(t0[3 * ax:3 * ax + 3].max(), t1[3 * ax:3 * ax + 3].max())
        recs[k, 0] = box[k, a]
        recs[k, 1] = box[k, 3 + a]
        for i, t in enumerate((t0, t1)):
            v1 = np.array([t[0], t[3], t[6]], np.float32)
            v2 = np.array([t[1], t[4], t[7]], np.float32)
            v3 = np.array([t[2], t[5], t[8]], np.float32)
            recs[k, 2 + 9 * i:11 + 9 * i] = np.concatenate([v1, v2 - v1, v3 - v1])
    for k in range(n - 1, -1, -1):              # children have higher indices: bottom-up
        for j, c in enumerate((2 * k + 1, 2 * k + 2)):
            cb = np.array([1, 1, 1, -1, -1, -1], np.float32)
            if c < n:
                box[k, :3] = np.minimum(box[k, :3], box[c, :3])
                box[k, 3:] = np.maximum(box[k, 3:], box[c, 3:])
                pad = np.float32(1e-5) * (np.abs(box[c, :3]) + np.abs(box[c, 3:])) + np.float32(1e-30)
                cb = np.concatenate([box[c, :3] - pad, box[c, 3:] + pad]).astype(np.float32)
            recs[k, 20 + 6 * j:26 + 6 * j] = cb
    return recs


def _regular_build(ctx, V):
    import torch
    Vd = torch.from_numpy(np.ascontiguousarray(V, np.float32).reshape(-1)).cuda()
    nmh = api.Nmh(ctx, Vd, count=V.shape[0])
    perm, verts = nmh.export()
    return perm, verts, nmh.info()[1]


def test_noalloc_build_matches_regular_build_twice_in_a_row(ctx):
    first = scenes.random_soup(40000, seed=1)
    second = scenes.random_soup(3001, seed=2)       # smaller, odd: the first call's data is still in the scratch
    for V in (first, second):
        recs, perm, verts, levels = _noalloc_build(V)
        rperm, rverts, rlevels = _regular_build(ctx, V)
        assert levels == rlevels
        assert np.array_equal(perm, rperm)
        assert np.array_equal(verts.view(np.uint32), rverts.view(np.uint32))
        exp = _expected_records(rverts)
        assert np.array_equal(recs.view(np.uint32), exp.view(np.uint32))


@pytest.mark.parametrize("count", [LIMIT, LIMIT - 1])
def test_noalloc_build_at_its_limit(ctx, count):
    """65,536 triangles, and 65,535 (which pads to 65,536): the scratch layout
    then ends exactly at the end of the fixed array."""
    V = scenes.random_soup(count, seed=3)
    recs, perm, verts, levels = _noalloc_build(V)
    rperm, rverts, rlevels = _regular_build(ctx, V)
    assert levels == rlevels
    assert np.array_equal(perm, rperm)
    assert np.array_equal(verts.view(np.uint32), rverts.view(np.uint32))
    exp = _expected_records(rverts)
    assert np.array_equal(recs.view(np.uint32), exp.view(np.uint32))


def test_noalloc_build_allocates_nothing(ctx):
    """Every device or pinned allocation the library makes goes through one
    helper, which the fault injector can make fail; armed to fail the very
    next allocation, the allocation-free build must still succeed."""
    V = scenes.random_soup(5000, seed=4)
    _noalloc_build(V)                            # device set-up (the array's address) done beforehand
    lib = api.lib()
    try:
        lib.aur_debug_fail_allocation(1)
        recs, perm, verts, levels = _noalloc_build(V)
    finally:
        lib.aur_debug_fail_allocation(0)
    rperm, rverts, _ = _regular_build(ctx, V)
    assert np.array_equal(perm, rperm)
    assert np.array_equal(verts.view(np.uint32), rverts.view(np.uint32))


def test_noalloc_build_rejects_soups_above_its_limit(ctx):
    import torch
    V = torch.zeros(9 * (LIMIT + 1), dtype=torch.float32, device="cuda")
    out = torch.zeros(9 * (LIMIT + 2), dtype=torch.float32, device="cuda")
    perm = torch.zeros(LIMIT + 2, dtype=torch.int32, device="cuda")
    st = api.lib().aur_nmh_build_noalloc(api._ptr(V), LIMIT + 1, _stream_arg(), api._ptr(out), api._ptr(perm),
                                         api._ptr(out), None)
    assert st == 1
    assert "65536" in api.lib().aur_last_error().decode()
