"""Textures on the GPU against the oracle: the fetch itself, textured
renders in both integrator modes, the wavefront batch and the adjoint."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu


def _scene(ctx, sd):
    sc = api.Scene(ctx, sd)
    sc.set_textures(sd.texcoords, sd.textures)
    return sc


def test_texfetch_matches_oracle(ctx):
    import torch
    sd = scenes.cornell_textured(seed=1)
    sc = _scene(ctx, sd)
    rng = np.random.default_rng(3)
    special = np.array([[0, 0], [1, 1], [-0.0, 0.5], [-1e-30, 0.5], [0.5, -1e-7], [1 - 2 ** -24, 0.25],
                        [np.nan, 0.5], [np.inf, 0.5], [0.5, -np.inf], [1e7, -1e7]], np.float32)
    for t, tex in enumerate(sd.textures, start=1):
        h, w = tex.shape[:2]
        centres = np.stack(np.meshgrid((np.arange(w) + 0.5) / w, (np.arange(h) + 0.5) / h), -1).reshape(-1, 2)
        uv = np.concatenate([rng.uniform(-3, 4, size=(1 << 20, 2)), centres, special]).astype(np.float32)
        got = sc.texfetch(t, torch.from_numpy(uv).cuda()).cpu().numpy()
        assert np.array_equal(got, oracle.texfetch(tex, uv))
    # units past the 32 the reference binds fetch white
    got = sc.texfetch(40, torch.from_numpy(rng.random((64, 2)).astype(np.float32)).cuda()).cpu().numpy()
    assert np.all(got == 1.0)


@pytest.mark.parametrize("mode", [T.MODE_REFERENCE, T.MODE_PATH])
def test_textured_render_matches_oracle(ctx, mode):
    sd = scenes.cornell_textured(seed=2)
    sc = _scene(ctx, sd)
    p = T.render_params(48, 40, 8, 4, seed=5, mode=mode)
    img = sc.render(p).cpu().numpy()
    ref, _ = oracle.render(oracle.NmhScene(sd), p)
    assert np.all(np.abs(img - ref) <= 1e-4 * np.abs(ref) + 1e-7)
    plain = api.Scene(ctx, scenes.cornell()).render(p).cpu().numpy()
    assert np.abs(img - plain).max() > 1e-2                   # the textures show


def test_texture_past_32_is_white(ctx):
    sd = scenes.cornell_textured(seed=2)
    white = sd.shaders.copy()
    white["texture"][5] = 0                                   # diffuse_color is (1, 1, 1)
    sa = _scene(ctx, sd)
    sb = api.Scene(ctx, scenes.SceneData(sd.name, sd.vertices, sd.normals, sd.shader_ids, white, sd.lights,
                                         sd.camera))
    sb.set_textures(sd.texcoords, sd.textures)
    p = T.render_params(32, 32, 4, 3, seed=1, mode=T.MODE_PATH)
    assert np.array_equal(sa.render(p).cpu().numpy(), sb.render(p).cpu().numpy())


def test_textured_wavefront_equals_plain(ctx):
    import torch
    sds = [scenes.cornell_textured(seed=s) for s in (0, 1)]
    scs = [_scene(ctx, sd) for sd in sds]
    prm = [T.render_params(40, 32, 6, 4, seed=2, mode=T.MODE_PATH, scene_id=i) for i in range(2)]
    plain = [sc.render(p) for sc, p in zip(scs, prm)]
    b = api.Batch(ctx, scs, prm, tuning=api.make_tuning(1 << 12, 2, 128, 4))
    frames = [torch.zeros_like(f) for f in plain]
    b.render(frames)
    b.status()
    for a, c in zip(frames, plain):
        assert torch.equal(a, c)


def test_textured_shaders_get_no_albedo_gradient(ctx):
    import torch
    sd = scenes.cornell_textured(seed=3)
    sc = _scene(ctx, sd)
    p = T.render_params(32, 32, 4, 3, seed=0, mode=T.MODE_PATH)
    img = sc.render(p)
    d_diffuse, _ = sc.adjoint(p, torch.ones_like(img))
    g = d_diffuse.cpu().numpy()
    assert np.all(g[3:6] == 0.0) and np.abs(g[0:3]).max() > 0


def test_textures_are_validated(ctx):
    sd = scenes.cornell_textured()
    sc = api.Scene(ctx, sd)
    with pytest.raises(api.AuroraError):
        sc.render(T.render_params(8, 8, 1, 2))                 # shaders name textures 1 and 2, none set
    with pytest.raises(api.AuroraError):
        sc.set_textures(sd.texcoords, sd.textures * 17)        # 34 > 32 textures
    sc.set_textures(sd.texcoords, sd.textures[:1])
    with pytest.raises(api.AuroraError):
        sc.render(T.render_params(8, 8, 1, 2))                 # texture 2 missing
    sc.set_textures(sd.texcoords, sd.textures)
    sc.render(T.render_params(8, 8, 1, 2))
