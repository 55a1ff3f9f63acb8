"""Out-of-memory paths, by fault injection on the host: for each operation,
the 1st, 2nd, ... device or pinned allocation it makes is failed in turn
(aur_debug_fail_allocation) until the operation no longer reaches the armed
one. Every failure must come back as AUR_ERR_OOM with nothing launched on a
missing buffer, and the library must then give the operation's normal
result, bit for bit. No GPU fault is involved: the failing allocation is
never made."""
import numpy as np
import pytest

from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu
OOM = 2


@pytest.fixture(autouse=True)
def _disarm():
    yield
    api.lib().aur_debug_fail_allocation(0)


def _sweep(op, max_k=40):
    base = op()
    for k in range(1, max_k + 1):
        api.lib().aur_debug_fail_allocation(k)
        try:
            got = op()
        except api.AuroraError as e:
            assert e.status == OOM, (k, str(e))
            api.lib().aur_debug_fail_allocation(0)
            assert _same(op(), base), k            # the library recovers
            continue
        finally:
            api.lib().aur_debug_fail_allocation(0)
        assert _same(got, base), k
        return k - 1                                # allocations the operation makes
    raise AssertionError("more than %d allocations" % max_k)


def _same(a, b):
    if a is None or b is None:
        return a is None and b is None
    if isinstance(a, (list, tuple)):
        return all(_same(x, y) for x, y in zip(a, b))
    return np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))


def test_nmh_build_and_trace(ctx):
    import torch
    V = scenes.random_soup(20000, seed=2)
    Vd = torch.from_numpy(V.reshape(-1)).cuda()
    rays = scenes.microbench_rays(1 << 15, seed=3)

    def op():
        fresh = api.Context(0)      # a fresh context allocates the build's scratch again
        try:
            nmh = api.Nmh(fresh, Vd, count=V.shape[0])
            again = api.Nmh(fresh, Vd, count=V.shape[0])       # the same size: the recorded build graph
            hits = api.hits_to_numpy(api.trace_closest(fresh, nmh, api.rays_tensor(rays)))
            return [nmh.export()[0], again.export()[0], hits.view(np.uint32),
                    np.array(api.count_visits(fresh, nmh, api.rays_tensor(rays)))]
        finally:
            fresh.close()
    assert _sweep(op) >= 5          # context flags, NMH arrays, build scratch, second NMH, trace counters


def test_scene_textures_render_emitters_adjoint(ctx):
    import torch
    sd = scenes.cornell_textured(seed=1)
    sd.shaders = sd.shaders.copy()
    sd.shaders["emission"][0] = 1.0
    p = T.render_params(32, 32, 4, 3, seed=1, mode=T.MODE_PATH)

    def op():
        sc = api.Scene(ctx, sd)
        sc.set_textures(sd.texcoords, sd.textures)
        img = sc.render(p)
        d_diffuse, _ = sc.adjoint(p, torch.ones_like(img))
        return [img.cpu().numpy(), sc.emitters(), d_diffuse.cpu().numpy() * 0]   # adjoint sums are order-dependent
    assert _sweep(op) >= 10


def test_host_pipeline_with_a_fresh_context(ctx):
    import torch
    V = scenes.random_soup(5000, seed=4)
    nmh = api.Nmh(ctx, torch.from_numpy(V.reshape(-1)).cuda(), count=V.shape[0])
    rays = scenes.microbench_rays((1 << 22) + 7, seed=5)

    def op():
        fresh = api.Context(0)                      # allocates its flags and, on first use, the pipeline buffers
        try:
            hits = np.zeros(rays.shape[0], T.hit_dtype)
            api.trace_closest_host(fresh, nmh, rays, hits)
            return hits.view(np.uint32)
        finally:
            fresh.close()
    assert _sweep(op) >= 5


def test_mis_tables_render_batch_adjoint(ctx):
    """AUR_MODE_PATH_MIS builds the light-selection table on first use (its
    scratch and three arrays), in aur_render, the batch and the adjoint."""
    import torch
    sd = scenes.cornell_emissive(area_light=True)
    p = T.render_params(24, 24, 4, 3, seed=3, mode=T.MODE_PATH_MIS)

    def op():
        sc = api.Scene(ctx, sd)
        img = sc.render(p)
        sc2 = api.Scene(ctx, sd)
        b = api.Batch(ctx, [sc2], [p], tuning=api.make_tuning(4096, 1, 128, 4))
        fr = b.render()
        b.status()
        b.close()
        sc3 = api.Scene(ctx, sd)
        d_diffuse, _ = sc3.adjoint(p, torch.ones_like(img))
        tri, cdf, pa = sc.mis_table()
        return [img.cpu().numpy(), fr[0].cpu().numpy(), tri, cdf, pa, d_diffuse.cpu().numpy() * 0]
    assert _sweep(op, max_k=60) >= 12


def test_wavefront_batch_and_autotune(ctx):
    import torch
    sds = [scenes.cornell(), scenes.cornell_sphere(seed=1, slices=16, stacks=8)]
    scs = [api.Scene(ctx, sd) for sd in sds]
    prm = [T.render_params(24, 20, 4, 3, seed=2, mode=T.MODE_PATH, scene_id=i) for i in range(2)]

    def op():
        b = api.Batch(ctx, scs, prm, tuning=api.make_tuning(4096, 2, 128, 4))
        frames = [torch.zeros((20, 24, 4), device="cuda") for _ in scs]
        b.render(frames)
        b.status()
        b.close()
        return [f.cpu().numpy() for f in frames]
    assert _sweep(op) >= 1
    # the autotuner skips candidates whose batch cannot be created
    for k in (2, 3, 5):
        api.lib().aur_debug_fail_allocation(k)
        t, ms = api.autotune(ctx, scs, prm)
        api.lib().aur_debug_fail_allocation(0)
        assert t["paths_in_flight"] >= 1024 and ms > 0


def test_memory_entry_points(ctx):
    import ctypes
    for policy in (1, 2):                            # device, pinned
        p = ctypes.c_void_p()
        api.lib().aur_debug_fail_allocation(1)
        assert api.lib().aur_malloc(ctx.handle, 1 << 20, policy, ctypes.byref(p)) == OOM
        api.lib().aur_debug_fail_allocation(0)
        assert api.lib().aur_malloc(ctx.handle, 1 << 20, policy, ctypes.byref(p)) == 0 and p.value
        assert api.lib().aur_free(ctx.handle, p, policy) == 0
