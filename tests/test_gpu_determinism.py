"""Determinism in place of a race detector (compute-sanitizer is not
available): the NMH build, traversal, renders, the wavefront batch and the
emitter table give identical bytes when run twice. (The adjoint's gradient
sums use float atomics and are reproducible only to rounding.)"""
import numpy as np
import pytest

from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu


def test_build_trace_render_batch_twice(ctx):
    import torch
    V = scenes.random_soup(300000, seed=11)
    Vd = torch.from_numpy(V.reshape(-1)).cuda()
    rays = api.rays_tensor(scenes.microbench_rays(1 << 18, seed=12))
    out = []
    for _ in range(2):
        nmh = api.Nmh(ctx, Vd, count=V.shape[0])
        perm, verts = nmh.export()
        hits = api.hits_to_numpy(api.trace_closest(ctx, nmh, rays)).view(np.uint32)
        occ = api.trace_any(ctx, nmh, rays).cpu().numpy()
        out.append([perm, verts.view(np.uint32), hits, occ])
    for a, b in zip(*out):
        assert np.array_equal(a, b)
    sd = scenes.cornell_sphere(seed=2)
    sd.shaders = sd.shaders.copy()
    sd.shaders["emission"][::7] = 0.5
    imgs, frames, ems = [], [], []
    for _ in range(2):
        sc = api.Scene(ctx, sd)
        p = T.render_params(64, 48, 8, 4, seed=3, mode=T.MODE_PATH)
        imgs.append(sc.render(p).cpu().numpy())
        b = api.Batch(ctx, [sc], [p], tuning=api.make_tuning(1 << 14, 2, 128, 4))
        f = [torch.zeros((48, 64, 4), device="cuda")]
        b.render(f)
        b.status()
        frames.append(f[0].cpu().numpy())
        ems.append(sc.emitters())
    assert np.array_equal(imgs[0], imgs[1]) and np.array_equal(frames[0], frames[1])
    assert np.array_equal(ems[0].view(np.uint8), ems[1].view(np.uint8))
