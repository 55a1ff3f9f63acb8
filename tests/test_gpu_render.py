"""GPU integrator against the oracle: same counter RNG streams, per-pixel agreement."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes, types as T
from helpers import load_golden

pytestmark = pytest.mark.gpu

REL = 1e-4   # per-pixel relative tolerance


def _close(a, b):
    return np.all(np.abs(a - b) <= REL * np.abs(b) + 1e-7)


@pytest.mark.parametrize("mode", [T.MODE_REFERENCE, T.MODE_PATH])
def test_cornell_render_matches_oracle(ctx, mode):
    sd = scenes.cornell()
    sc = api.Scene(ctx, sd)
    p = T.render_params(64, 64, 16, 4, seed=0, mode=mode)
    img = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd), p)
    assert _close(img, ref)
    assert np.array_equal(img, ref)      # same arithmetic, same order: bit-exact


@pytest.mark.parametrize("mode", [T.MODE_REFERENCE, T.MODE_PATH])
def test_cornell_full_frame_matches_oracle(ctx, mode):
    """The Cornell workload at its stated size: 256x256, 16 spp, depth 4, seed 0."""
    sd = scenes.cornell()
    sc = api.Scene(ctx, sd)
    p = T.render_params(256, 256, 16, 4, seed=0, mode=mode)
    img = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd), p)
    assert _close(img, ref)
    assert np.array_equal(img, ref)


def test_cornell_sphere_render_matches_oracle(ctx):
    sd = scenes.cornell_sphere(seed=1)
    sc = api.Scene(ctx, sd)
    p = T.render_params(48, 48, 4, 4, seed=3, mode=T.MODE_PATH)
    img = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd), p)
    assert _close(img, ref)


def test_render_golden_regression(ctx):
    g = load_golden("cornell")
    sc = api.Scene(ctx, scenes.cornell())
    for mode in (T.MODE_REFERENCE, T.MODE_PATH):
        img = sc.render(T.render_params(32, 32, 4, 4, seed=0, mode=mode)).cpu().numpy()
        assert _close(img, g["image_mode%d" % mode])


def test_helper_entry_points_match_fused_render(ctx):
    import torch
    sd = scenes.cornell()
    sc = api.Scene(ctx, sd)
    W = H = 40
    spp = 4
    p = T.render_params(W, H, spp, 4, seed=2, mode=T.MODE_PATH)
    fused = sc.render(p).cpu().numpy()
    rays = torch.zeros((W * H, 9), dtype=torch.float32, device="cuda")
    hits = torch.zeros((W * H, 12), dtype=torch.float32, device="cuda")
    accum = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    api.clear_pixels(ctx, W, H, accum)
    for s in range(spp):
        api.generate_rays(ctx, W, H, s, spp, sd.camera, rays, hits)
        for off in range(0, W * H, 512):                  # tiles, as the reference renders
            api.raytrace_monte_carlo(ctx, sc, p, s, off, min(512, W * H - off), rays, hits)
        api.draw_pixels(ctx, W, H, 1.0 / spp, hits, accum)
    assert np.array_equal(accum.cpu().numpy(), fused)
    prays = rays.cpu().numpy().view(T.path_ray_dtype).reshape(-1)
    orays = oracle.generate_rays(sd.camera, W, H, spp - 1, spp)
    assert np.array_equal(prays.view(np.uint32), orays.view(np.uint32))


def test_sample_ranges_add_up(ctx):
    sc = api.Scene(ctx, scenes.cornell())
    full = sc.render(T.render_params(24, 24, 9, 3, seed=4)).cpu().numpy()
    acc = sc.render(T.render_params(24, 24, 9, 3, seed=4, sample_begin=0, sample_end=5))
    acc = sc.render(T.render_params(24, 24, 9, 3, seed=4, sample_begin=5, sample_end=9), accum=acc)
    assert np.array_equal(acc.cpu().numpy(), full)


def test_invalid_arguments_raise(ctx):
    sd = scenes.cornell()
    sc = api.Scene(ctx, sd)
    with pytest.raises(api.AuroraError):
        sc.render(T.render_params(8, 8, 0, 4))
    with pytest.raises(api.AuroraError):
        sc.render(T.render_params(8, 8, 4, 99))
    bad = sd.shaders.copy()
    bad["texture"][0] = 1               # names texture 1, but the scene has none
    sc.set_shaders(bad)
    with pytest.raises(api.AuroraError) as e:
        sc.render(T.render_params(8, 8, 1, 4))
    assert e.value.status == 1 and "texture" in str(e.value)
    bad["type"][0] = 7
    with pytest.raises(api.AuroraError):
        sc.set_shaders(bad)


@pytest.mark.parametrize("mode", [T.MODE_REFERENCE, T.MODE_PATH])
def test_specular_render_matches_oracle(ctx, mode):
    """Reflective and refractive shaders exercise the reference's ray stack
    (monteCarloRaytracer.cu:54-85)."""
    sd = scenes.cornell()
    sh = np.concatenate([sd.shaders, np.stack([T.lambert((0.9, 0.9, 0.9)), T.lambert((0.8, 0.9, 1.0))])])
    sh["reflectivity"][3] = 0.6
    sh["translucence"][4] = 0.7
    sh["refractive_index"][4] = 1.5
    sids = sd.shader_ids.copy()
    sids[10:22] = 4          # short block: mirror-like
    sids[22:34] = 5          # tall block: glass-like
    sd2 = scenes.SceneData("cornell_specular", sd.vertices, sd.normals, sids, sh, sd.lights, sd.camera)
    sc = api.Scene(ctx, sd2)
    p = T.render_params(48, 48, 4, 5, seed=11, mode=mode)
    img = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd2), p)
    assert np.array_equal(img, ref)


@pytest.mark.parametrize("W,H,spp,depth,mode", [(1, 1, 1, 0, T.MODE_REFERENCE), (7, 3, 5, 16, T.MODE_PATH),
                                                (13, 11, 7, 2, T.MODE_PATH_MIS), (16, 16, 2, 16, T.MODE_REFERENCE)])
def test_edge_sizes_match_oracle(ctx, W, H, spp, depth, mode):
    """A one-pixel frame, sample counts that are not squares (the reference's
    (short)sqrtf(spp) grid puts the extra samples below the pixel), depth 0
    and the maximum depth, in every mode."""
    sd = scenes.cornell_emissive(area_light=True)
    sc = api.Scene(ctx, sd)
    p = T.render_params(W, H, spp, depth, seed=13, mode=mode)
    img = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd), p, table=sc.mis_table() if mode == T.MODE_PATH_MIS else None)
    assert np.array_equal(img, ref)
