"""AUR_MODE_PATH_MIS on the GPU: the light-selection table and the images
against the oracle, unbiasedness at high sample counts, the tile entry point
and the wavefront batch against the fused renderer (the adjoint's
finite-difference checks are in test_gpu_adjoint.py)."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu


def _specular(sd):
    sh = np.concatenate([sd.shaders, np.stack([T.lambert((0.9, 0.9, 0.9)), T.lambert((0.8, 0.9, 1.0))])])
    k = sd.shaders.shape[0]
    sh["reflectivity"][k] = 0.6
    sh["translucence"][k + 1] = 0.7
    sh["refractive_index"][k + 1] = 1.5
    sids = sd.shader_ids.copy()
    sids[10:22] = k + 1
    sids[22:34] = k + 2
    return scenes.SceneData(sd.name + "_specular", sd.vertices, sd.normals, sids, sh, sd.lights, sd.camera)


def _all_lights(sd):
    """Every light type around the emitters, area lights with several samples
    between the delta lights: the order in which a hit's shadow rays are
    walked and summed."""
    lights = np.zeros(5, T.light_dtype)
    lights[0] = T.area_light((0.2, 0.99, 0.3), (0.3, 0.0, 0.0), (0.0, 0.0, 0.2), (0.0, -1.0, 0.0),
                             color=(1.0, 0.8, 0.6), intensity=1.5, samples=3)
    lights[1]["type"], lights[1]["position"], lights[1]["color"], lights[1]["intensity"] = (
        T.LIGHT_POINT, (0.5, 0.8, 0.5), (0.3, 0.3, 1.0), 0.4)
    lights[2]["type"], lights[2]["position"], lights[2]["color"] = T.LIGHT_AMBIENT, (0.5, 0.5, 0.5), (1, 1, 1)
    lights[2]["intensity"], lights[2]["ambient"] = 0.3, 0.25
    lights[3] = T.area_light((0.6, 0.5, 0.999), (0.2, 0.0, 0.0), (0.0, 0.2, 0.0), (0.0, 0.0, -1.0), samples=2)
    lights[4]["type"], lights[4]["direction"], lights[4]["color"], lights[4]["intensity"] = (
        T.LIGHT_DIRECTIONAL, (0.3, -1.0, -0.2), (1.0, 1.0, 1.0), 0.2)
    return scenes.SceneData(sd.name + "_lights", sd.vertices, sd.normals, sd.shader_ids, sd.shaders, lights,
                            sd.camera)


def test_table_matches_oracle(ctx):
    for sd in (scenes.cornell_emissive(), scenes.cornell_emissive(area_light=True), scenes.cornell()):
        sc = api.Scene(ctx, sd)
        tri, cdf, pa = sc.mis_table()
        otri, ocdf, opa = oracle.mis_table(oracle.NmhScene(sd))
        assert np.array_equal(tri, otri)
        assert np.allclose(cdf, ocdf, rtol=3e-7, atol=0) and (len(cdf) == 0 or cdf[-1] == np.float32(1.0))
        assert np.allclose(pa, opa, rtol=1e-5, atol=0) and np.array_equal(pa > 0, opa > 0)


def test_table_of_many_emitters_matches_oracle(ctx):
    """Multi-tile scans: 300,001 triangles, a third of them emitting."""
    V = scenes.random_soup(300_001, seed=7)
    n = V.shape[0]
    sh = np.stack([T.lambert((0.5, 0.5, 0.5)), T.lambert((0.5, 0.5, 0.5), emission=(1.0, 2.0, 3.0)),
                   T.lambert((0.5, 0.5, 0.5), emission=(4.0, 0.0, 0.0))])
    sh["emission"][1], sh["emission"][2] = 0.7, 2.5
    sids = (np.arange(n) % 3 + 1).astype(np.uint16)
    sd = scenes.SceneData("soup", V, np.zeros_like(V), sids, sh, np.zeros(0, T.light_dtype), scenes.cornell_camera())
    sc = api.Scene(ctx, sd)
    tri, cdf, pa = sc.mis_table()
    otri, ocdf, opa = oracle.mis_table(oracle.NmhScene(sd, perm=sc.nmh.export()[0]))
    assert len(tri) > 190_000 and np.array_equal(tri, otri)
    assert np.max(np.abs(cdf.astype(np.float64) - ocdf)) <= 2.0 ** -23
    assert np.allclose(pa, opa, rtol=2e-3, atol=0)      # cdf differences of an ulp, divided


@pytest.mark.parametrize("scene", ["cornell", "emissive", "emissive_area", "emissive_specular", "emissive_all_lights",
                                   "emissive_all_lights_specular"])
def test_render_matches_oracle(ctx, scene):
    sd = {"cornell": scenes.cornell, "emissive": scenes.cornell_emissive,
          "emissive_area": lambda: scenes.cornell_emissive(area_light=True),
          "emissive_specular": lambda: _specular(scenes.cornell_emissive(area_light=True)),
          "emissive_all_lights": lambda: _all_lights(scenes.cornell_emissive()),
          "emissive_all_lights_specular": lambda: _specular(_all_lights(scenes.cornell_emissive()))}[scene]()
    sc = api.Scene(ctx, sd)
    p = T.render_params(40, 40, 4, 4, seed=9, mode=T.MODE_PATH_MIS)
    img = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd), p, table=sc.mis_table())
    assert np.array_equal(img, ref)                 # same arithmetic, same order: bit-exact
    assert img[..., :3].mean() > 0.01


def test_textured_render_matches_oracle(ctx):
    """Textured shaders in the MIS mode: the colour of a textured shader enters
    f, and both strategies and the emitter sample, bit for bit."""
    sd = scenes.cornell_textured(seed=2)
    sd.shaders = np.concatenate([sd.shaders, np.stack([T.lambert((1.0, 1.0, 1.0), emission=(3.0, 2.0, 1.0))])])
    sd.shaders["emission"][-1] = 1.0
    sd.shader_ids = sd.shader_ids.copy()
    sd.shader_ids[2:4] = len(sd.shaders)              # the ceiling emits
    sc = api.Scene(ctx, sd)
    sc.set_textures(sd.texcoords, sd.textures)
    p = T.render_params(40, 40, 4, 3, seed=5, mode=T.MODE_PATH_MIS)
    img = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd), p, table=sc.mis_table())
    assert np.array_equal(img, ref)
    assert len(sc.mis_table()[0]) == 2


def test_mis_matches_path_mode_one_bounce_deeper(ctx):
    """Emissive geometry only: E[MIS at depth d] = E[path mode at depth d + 1];
    48 x 48 pixels, 8 independent 1024-sample renders of each. Path mode's
    per-pixel estimates are far from normal in dark corners (rare large
    contributions), so the comparison is on the image mean (a z-test over
    the 8 renders) and on 8 x 8-pixel block means."""
    sc = api.Scene(ctx, scenes.cornell_emissive())
    W = 48

    def renders(mode, d):
        return np.stack([sc.render(T.render_params(W, W, 1024, d, seed=s, mode=mode)).cpu().numpy()[..., :3]
                         for s in range(8)]).astype(np.float64)

    mis, path = renders(T.MODE_PATH_MIS, 2), renders(T.MODE_PATH, 3)
    im, ip = mis.mean(axis=(1, 2, 3)), path.mean(axis=(1, 2, 3))
    z = (im.mean() - ip.mean()) / np.sqrt(im.var(ddof=1) / 8 + ip.var(ddof=1) / 8)
    assert abs(z) < 4.0, z
    bm = mis.mean(0).reshape(6, 8, 6, 8, 3).mean(axis=(1, 3))
    bp = path.mean(0).reshape(6, 8, 6, 8, 3).mean(axis=(1, 3))
    assert np.max(np.abs(bm / bp - 1.0)) < 0.03
    assert im.std() < 0.25 * ip.std()                                # variance of the image mean
    assert mis.std(0).mean() < 0.5 * path.std(0).mean()              # and per pixel


def _mis_batch_scenes():
    sph = scenes.sphere_scene(5, max_tris=20000)
    sph.shaders = sph.shaders.copy()
    sph.shaders["emission"][0] = 1.0          # the first shader's triangles emit (colour set below)
    sph.shaders["emission_color"][0] = (0.5, 0.4, 0.3)
    return [scenes.cornell_emissive(area_light=True), scenes.cornell_emissive(), scenes.cornell(), sph,
            _all_lights(scenes.cornell_emissive())]


@pytest.mark.parametrize("tuning", [dict(paths_in_flight=1024, samples_per_wave=1, block_size=64, blocks_per_sm=2),
                                    dict()])
def test_wavefront_equals_plain(ctx, tuning):
    """The wavefront batch in MIS mode: every frame equals aur_render's."""
    sds = _mis_batch_scenes()
    scs = [api.Scene(ctx, sd) for sd in sds]
    sizes = [(40, 32), (24, 24), (33, 17), (16, 40), (20, 20)]
    prm = [T.render_params(w, h, 4, 3, seed=7, mode=T.MODE_PATH_MIS, scene_id=i) for i, (w, h) in enumerate(sizes)]
    batch = api.Batch(ctx, scs, prm, tuning=api.make_tuning(**tuning) if tuning else None)
    frames = batch.render()
    assert batch.status() > 0
    for sc, p, f in zip(scs, prm, frames):
        assert np.array_equal(f.cpu().numpy(), sc.render(p).cpu().numpy())
    # shaders change between renders: the batch picks up the rebuilt tables
    sh = sds[1].shaders.copy()
    sh["emission"][4] = 0.0
    scs[1].set_shaders(sh)
    frames = batch.render()
    batch.status()
    for sc, p, f in zip(scs, prm, frames):
        assert np.array_equal(f.cpu().numpy(), sc.render(p).cpu().numpy())


def test_wavefront_light_slot_limit(ctx):
    """MIS takes two slots per area-light sample plus one: 16 samples need 33
    of the 32 a path has."""
    sd = scenes.cornell()
    sd.lights = sd.lights.copy()
    sd.lights["samples"][0] = 16
    sc = api.Scene(ctx, sd)
    with pytest.raises(api.AuroraError) as e:
        api.Batch(ctx, [sc], [T.render_params(8, 8, 1, 2, mode=T.MODE_PATH_MIS)])
    assert e.value.status == 6
    sd.lights["samples"][0] = 15
    sc2 = api.Scene(ctx, sd)
    p = T.render_params(8, 8, 1, 2, mode=T.MODE_PATH_MIS)
    b = api.Batch(ctx, [sc2], [p])
    fr = b.render()
    b.status()
    assert np.array_equal(fr[0].cpu().numpy(), sc2.render(p).cpu().numpy())


def test_helper_entry_points_match_fused_render(ctx):
    """generateRays + raytraceMonteCarlo tiles + drawPixels in MIS mode give
    the fused render bit for bit (the tile kernel builds the same table)."""
    import torch
    sd = scenes.cornell_emissive(area_light=True)
    sc = api.Scene(ctx, sd)
    W = H = 40
    spp = 4
    p = T.render_params(W, H, spp, 3, seed=2, mode=T.MODE_PATH_MIS)
    fused = sc.render(p).cpu().numpy()
    sc2 = api.Scene(ctx, sd)                          # table built by the tile path
    rays = torch.zeros((W * H, 9), dtype=torch.float32, device="cuda")
    hits = torch.zeros((W * H, 12), dtype=torch.float32, device="cuda")
    accum = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    api.clear_pixels(ctx, W, H, accum)
    for s in range(spp):
        api.generate_rays(ctx, W, H, s, spp, sd.camera, rays, hits)
        for off in range(0, W * H, 512):
            api.raytrace_monte_carlo(ctx, sc2, p, s, off, min(512, W * H - off), rays, hits)
        api.draw_pixels(ctx, W, H, 1.0 / spp, hits, accum)
    assert np.array_equal(accum.cpu().numpy(), fused)


def test_too_many_lights_for_the_rng_slots(ctx):
    sd = scenes.cornell()
    lights = np.repeat(sd.lights, 32767)
    sd2 = scenes.SceneData("many", sd.vertices, sd.normals, sd.shader_ids, sd.shaders, lights, sd.camera)
    sc = api.Scene(ctx, sd2)
    with pytest.raises(api.AuroraError) as e:
        sc.render(T.render_params(4, 4, 1, 1, mode=T.MODE_PATH_MIS))
    assert e.value.status == 1                          # AUR_ERR_INVALID


def test_table_follows_shader_changes(ctx):
    sd = scenes.cornell_emissive()
    sc = api.Scene(ctx, sd)
    p = T.render_params(24, 24, 4, 3, seed=2, mode=T.MODE_PATH_MIS)
    before = sc.render(p).cpu().numpy()
    assert len(sc.mis_table()[0]) == 15
    sh = sd.shaders.copy()
    sh["emission"][4] = 0.0                     # the floor block no longer in the table
    sc.set_shaders(sh)
    tri, _, _ = sc.mis_table()
    assert len(tri) == 3
    sd2 = scenes.SceneData("e2", sd.vertices, sd.normals, sd.shader_ids, sh, sd.lights, sd.camera)
    after = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd2), p, table=sc.mis_table())
    assert np.array_equal(after, ref) and not np.array_equal(after, before)
