"""Pins the oracle's lighting to the reference's own shading code.

The reference's Shader::getBSDF, Light::sampleL, sampleRectangle and the
three radiance estimators (radiance.cuh) are compiled unmodified as host C++
(oracle/ref_shim/ref_shade.cpp) and evaluated at the first hits of camera
rays found by the reference's own intersect(), replaying the counter-RNG
uniforms in the order that code draws them. The oracle renders the same
rays with depth 0 in reference mode, where a pixel's colour is exactly that
Li. The two must agree bit for bit, with ambient, point, directional and
area lights (one and several samples) and a Phong shader in the scene."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import scenes, types as T


def _scene():
    sd = scenes.cornell()
    sh = np.concatenate([sd.shaders, np.stack([T.lambert((0.7, 0.6, 0.2), emission=(0.05, 0.0, 0.1))])])
    sh["type"][3] = T.SHADER_PHONG
    sh["exponent"][3] = 20.0
    sids = sd.shader_ids.copy()
    sids[10:22] = 4                                           # the short box: emissive Phong
    lights = np.zeros(6, T.light_dtype)
    lights[0] = scenes.cornell_light(intensity=2.0, samples=1)
    lights[1] = T.area_light((0.2, 0.99, 0.3), (0.3, 0.0, 0.0), (0.0, 0.0, 0.2), (0.0, -1.0, 0.0),
                             color=(1.0, 0.8, 0.6), intensity=1.5, samples=3)
    lights[2]["type"], lights[2]["position"], lights[2]["color"], lights[2]["intensity"] = (
        T.LIGHT_POINT, (0.5, 0.8, 0.5), (0.3, 0.3, 1.0), 0.4)
    lights[3]["type"], lights[3]["direction"], lights[3]["color"], lights[3]["intensity"] = (
        T.LIGHT_DIRECTIONAL, (0.3, -1.0, -0.2), (1.0, 1.0, 1.0), 0.2)
    lights[4]["type"], lights[4]["position"], lights[4]["color"] = T.LIGHT_AMBIENT, (0.5, 0.5, 0.5), (1, 1, 1)
    lights[4]["intensity"], lights[4]["ambient"] = 0.3, 0.25
    lights[5] = T.area_light((0.6, 0.5, 0.999), (0.2, 0.0, 0.0), (0.0, 0.2, 0.0), (0.0, 0.0, -1.0), samples=2)
    return scenes.SceneData("pin", sd.vertices, sd.normals, sids, sh, lights, sd.camera)


def test_lighting_matches_the_reference_shading_code():
    if oracle.ref_lib() is None:
        pytest.skip("the reference sources are not on this machine")
    sd = _scene()
    ns = oracle.NmhScene(sd)
    W, H, seed = 48, 40, 5
    p = T.render_params(W, H, 1, 0, seed=seed, mode=T.MODE_REFERENCE)
    img, _ = oracle.render(ns, p)
    pr = oracle.generate_rays(ns.camera, W, H, 0, 1)                         # path rays, pixel order
    rays = np.zeros(W * H, T.ray_dtype)
    rays["ox"], rays["oy"], rays["oz"] = pr["pos"][:, 0], pr["pos"][:, 1], pr["pos"][:, 2]
    rays["dx"], rays["dy"], rays["dz"] = pr["dir"][:, 0], pr["dir"][:, 1], pr["dir"][:, 2]
    rays["tmax"] = pr["t"]
    tuv, ids = oracle.ref_trace_closest(ns.V, rays)
    assert (ids >= 0).mean() > 0.9
    tg, bt = oracle.generate_tb(ns.N)
    swap = oracle.ref_uniform_order() == 1
    per_hit = 2 * int(sum(int(l["samples"]) for l in ns.lights if l["type"] == T.LIGHT_AREA))
    uni = np.zeros((W * H, per_hit), np.float32)
    for pix in range(W * H):
        q = []
        for li, L in enumerate(ns.lights):
            if L["type"] != T.LIGHT_AREA:
                continue
            for j in range(int(L["samples"])):
                u1, u2 = oracle.draw2(seed, 0, pix, 0, 0, 1 + (li << 16) + j)
                q += [u2, u1] if swap else [u1, u2]
        uni[pix] = q
    Li = oracle.ref_shade_hits(ns, tg, bt, rays.view(np.float32).reshape(-1, 8), ids, tuv, uni)
    got = img.reshape(-1, 4)[:, :3]
    hit = ids >= 0
    assert np.array_equal(got[hit].view(np.uint32), Li[hit].view(np.uint32))
    assert np.all(got[~hit] == 0.0)
