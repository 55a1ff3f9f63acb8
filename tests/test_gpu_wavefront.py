"""Batched wavefront integrator: every scene's frame equals the plain renderer's."""
import numpy as np
import pytest

from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu


def _scenes():
    return [scenes.cornell(), scenes.cornell_sphere(seed=2), scenes.sphere_scene(5, max_tris=20000),
            scenes.sphere_scene(9, max_tris=5000)]


def _params(mode, sizes, spp=4, depth=3):
    return [T.render_params(w, h, spp, depth, seed=7, mode=mode, scene_id=i) for i, (w, h) in enumerate(sizes)]


@pytest.mark.parametrize("mode", [T.MODE_PATH, T.MODE_REFERENCE])
@pytest.mark.parametrize("tuning", [dict(paths_in_flight=1024, samples_per_wave=1, block_size=64, blocks_per_sm=2),
                                    dict()])
def test_wavefront_equals_plain(ctx, mode, tuning):
    sds = _scenes()
    scs = [api.Scene(ctx, sd) for sd in sds]
    sizes = [(40, 32), (24, 24), (33, 17), (16, 40)]
    prm = _params(mode, sizes)
    batch = api.Batch(ctx, scs, prm, tuning=api.make_tuning(**tuning) if tuning else None)
    frames = batch.render()
    iters = batch.status()
    assert iters > 0
    for sc, p, f in zip(scs, prm, frames):
        plain = sc.render(p).cpu().numpy()
        assert np.array_equal(f.cpu().numpy(), plain)
    # a second launch of the same graph adds the same samples again
    frames2 = batch.render(frames)
    batch.status()
    for sc, p, f in zip(scs, prm, frames2):
        twice = sc.render(p, accum=sc.render(p))
        assert np.array_equal(f.cpu().numpy(), twice.cpu().numpy())


@pytest.mark.parametrize("mode", [T.MODE_PATH, T.MODE_PATH_MIS, T.MODE_REFERENCE])
def test_wavefront_frames_match_oracle(ctx, mode):
    """Batch frames against the oracle directly (not through aur_render, which
    shares the device helpers): a sphere scene, the Cornell box with a sphere,
    and emissive triangles plus an area light, in one batch whose pool is small
    enough to refill several times."""
    import oracle
    sds = [scenes.sphere_scene(5, max_tris=20000), scenes.cornell_sphere(seed=2),
           scenes.cornell_emissive(area_light=True)]
    scs = [api.Scene(ctx, sd) for sd in sds]
    sizes = [(32, 24), (24, 24), (20, 28)]
    prm = [T.render_params(w, h, 4, 4, seed=11, mode=mode, scene_id=i) for i, (w, h) in enumerate(sizes)]
    batch = api.Batch(ctx, scs, prm, tuning=api.make_tuning(1024, 1, 64, 2))
    frames = batch.render()
    assert batch.status() > 0
    for sd, sc, p, f in zip(sds, scs, prm, frames):
        table = sc.mis_table() if mode == T.MODE_PATH_MIS else None
        ref, _ = oracle.render(oracle.NmhScene(sd), p, table=table)
        assert np.array_equal(f.cpu().numpy(), ref), sd.name


def _specular(sd, k0=10, k1=22, k2=34):
    """The scene with a mirror-like block (reflectivity 0.6) and a glass-like
    one (translucence 0.7, index 1.5)."""
    sh = np.concatenate([sd.shaders, np.stack([T.lambert((0.9, 0.9, 0.9)), T.lambert((0.8, 0.9, 1.0))])])
    n = sd.shaders.shape[0]
    sh["reflectivity"][n] = 0.6
    sh["translucence"][n + 1] = 0.7
    sh["refractive_index"][n + 1] = 1.5
    sids = sd.shader_ids.copy()
    sids[k0:k1] = n + 1
    sids[k1:k2] = n + 2
    return scenes.SceneData(sd.name + "_specular", sd.vertices, sd.normals, sids, sh, sd.lights, sd.camera)


@pytest.mark.parametrize("mode", [T.MODE_REFERENCE, T.MODE_PATH, T.MODE_PATH_MIS])
@pytest.mark.parametrize("tuning", [dict(paths_in_flight=1024, samples_per_wave=1, block_size=64, blocks_per_sm=2),
                                    dict()])
def test_wavefront_specular_equals_plain(ctx, mode, tuning):
    """Specular shaders: each path keeps its sample's pending rays (the plain
    integrator's ray stack), so reflection and refraction rays are traced in
    the same order with the same ray indices; the frames equal aur_render's,
    with specular and Lambert scenes in one batch."""
    sds = [_specular(scenes.cornell()), scenes.cornell_sphere(seed=2),
           _specular(scenes.cornell_emissive(area_light=True))]
    scs = [api.Scene(ctx, sd) for sd in sds]
    sizes = [(40, 32), (24, 24), (33, 17)]
    prm = [T.render_params(w, h, 4, 5, seed=7, mode=mode, scene_id=i) for i, (w, h) in enumerate(sizes)]
    batch = api.Batch(ctx, scs, prm, tuning=api.make_tuning(**tuning) if tuning else None)
    frames = batch.render()
    assert batch.status() > 0
    for sc, p, f in zip(scs, prm, frames):
        assert np.array_equal(f.cpu().numpy(), sc.render(p).cpu().numpy())


def test_autotune_specular_batch(ctx):
    """Specular batches carry a ray stack per path: the autotuner keeps their
    pools at 8M paths or fewer, and its pick renders the plain frame."""
    scs = [api.Scene(ctx, _specular(scenes.cornell()))]
    prm = _params(T.MODE_PATH, [(48, 40)])
    t, ms = api.autotune(ctx, scs, prm)
    assert ms > 0 and 1024 <= int(t["paths_in_flight"]) <= (1 << 23)
    b = api.Batch(ctx, scs, prm, tuning=t)
    fr = b.render()
    b.status()
    assert np.array_equal(fr[0].cpu().numpy(), scs[0].render(prm[0]).cpu().numpy())


def test_wavefront_needs_a_new_batch_for_new_specular_shaders(ctx):
    sd = scenes.cornell()
    sc = api.Scene(ctx, sd)
    p = _params(T.MODE_PATH, [(8, 8)])
    b = api.Batch(ctx, [sc], p)
    sh = sd.shaders.copy()
    sh["reflectivity"][0] = 0.5
    sc.set_shaders(sh)
    with pytest.raises(api.AuroraError) as e:
        b.render()
    assert e.value.status == 1
    b2 = api.Batch(ctx, [sc], p)
    fr = b2.render()
    b2.status()
    assert np.array_equal(fr[0].cpu().numpy(), sc.render(p[0]).cpu().numpy())


def test_autotune_returns_a_working_tuning(ctx):
    scs = [api.Scene(ctx, sd) for sd in _scenes()[:2]]
    prm = _params(T.MODE_PATH, [(64, 64), (32, 32)])
    t, ms = api.autotune(ctx, scs, prm)
    assert ms > 0 and int(t["paths_in_flight"]) >= 1024
    b = api.Batch(ctx, scs, prm, tuning=t)
    fr = b.render()
    b.status()
    assert np.array_equal(fr[0].cpu().numpy(), scs[0].render(prm[0]).cpu().numpy())


def test_iteration_limit_reports_timeout_and_context_survives(ctx):
    """The device-side integrator loop is bounded: with a limit of one
    iteration it stops, the render reports AUR_ERR_TIMEOUT, and the context
    keeps working."""
    scs = [api.Scene(ctx, sd) for sd in _scenes()[:2]]
    prm = _params(T.MODE_PATH, [(32, 32), (16, 16)])
    b = api.Batch(ctx, scs, prm, tuning=api.make_tuning(paths_in_flight=1024, max_iterations=1))
    b.render()
    with pytest.raises(api.AuroraError) as e:
        b.status()
    assert e.value.status == 4
    ok = api.Batch(ctx, scs, prm)
    fr = ok.render()
    ok.status()
    assert np.array_equal(fr[0].cpu().numpy(), scs[0].render(prm[0]).cpu().numpy())
    ext, shadow, iters = ok.counters()
    assert ext > 0 and shadow > 0 and iters > 0


def test_tuning_is_validated(ctx):
    sd = scenes.cornell()
    sc = api.Scene(ctx, sd)
    p = [T.render_params(16, 16, 2, 2, mode=T.MODE_PATH)]
    for bad in (dict(block_size=512), dict(block_size=100), dict(paths_in_flight=10), dict(blocks_per_sm=64)):
        with pytest.raises(api.AuroraError):
            api.Batch(ctx, [sc], p, tuning=api.make_tuning(**bad))
    api.Batch(ctx, [sc], p, tuning=api.make_tuning(block_size=256)).close()


def test_lights_with_more_samples_after_creation_stop_the_render(ctx):
    """The batch is sized for the light samples per hit at creation; a scene
    whose lights gain samples afterwards must stop the render with an error
    (no out-of-range writes), and the batch renders again once they are back."""
    import torch
    sd = scenes.cornell()
    sc = api.Scene(ctx, sd)
    p = [T.render_params(16, 16, 2, 2, mode=T.MODE_PATH)]
    b = api.Batch(ctx, [sc], p, tuning=api.make_tuning(2048, 1, 128, 2))
    ref = [torch.zeros((16, 16, 4), device="cuda")]
    b.render(ref)
    b.status()
    more = sd.lights.copy()
    more["samples"] = 4
    sc.set_lights(more)
    f = [torch.zeros((16, 16, 4), device="cuda")]
    b.render(f)
    with pytest.raises(api.AuroraError) as e:
        b.status()
    assert e.value.status == 1 and "samples" in str(e.value)
    sc.set_lights(sd.lights)
    f = [torch.zeros((16, 16, 4), device="cuda")]
    b.render(f)
    b.status()
    assert torch.equal(f[0], ref[0])
