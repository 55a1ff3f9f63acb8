"""Path-replay adjoint: gradients against central finite differences of the
plain renderer with common random numbers, and through a torch.autograd
wrapper (the wrapper lives only here, in the test harness)."""
import numpy as np
import pytest

from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu

H = 1e-3


def _loss(img, target):
    d = img.double() - target.double()
    return float((d[..., :3] ** 2).sum())


def _setup(ctx, mode, W=48, spp=8, depth=4, sd=None):
    sd = scenes.cornell_sphere(seed=3) if sd is None else sd
    sc = api.Scene(ctx, sd)
    p = T.render_params(W, W, spp, depth, seed=5, mode=mode)
    rng = np.random.default_rng(1)
    target_sh = sd.shaders.copy()
    target_sh["diffuse_color"] = np.clip(target_sh["diffuse_color"] + rng.normal(0, 0.05, (len(target_sh), 3)), 0, 1)
    sc.set_shaders(target_sh)
    target = sc.render(p)
    sc.set_shaders(sd.shaders)
    return sd, sc, p, target


def _fd(sc, sd, p, target, kind, idx, ch, h=H):
    vals = []
    for sgn in (+1, -1):
        sh, lt = sd.shaders.copy(), sd.lights.copy()
        if kind == "shader":
            sh["diffuse_color"][idx, ch] += sgn * h
        elif kind == "emission":
            sh["emission_color"][idx, ch] += sgn * h
        else:
            lt["color"][idx, ch] += sgn * h
        sc.set_shaders(sh)
        sc.set_lights(lt)
        vals.append(_loss(sc.render(p), target))
    sc.set_shaders(sd.shaders)
    sc.set_lights(sd.lights)
    return (vals[0] - vals[1]) / (2 * h)


def _specular_cornell():
    """Cornell with a mirror-like block (reflectivity 0.6, diffuse remainder)
    and a glass-like one (translucence 0.7, index 1.5)."""
    sd = scenes.cornell()
    sh = np.concatenate([sd.shaders, np.stack([T.lambert((0.9, 0.8, 0.7)), T.lambert((0.7, 0.8, 0.9))])])
    sh["reflectivity"][3] = 0.6
    sh["translucence"][4] = 0.7
    sh["refractive_index"][4] = 1.5
    sids = sd.shader_ids.copy()
    sids[10:22] = 4
    sids[22:34] = 5
    return scenes.SceneData("cornell_specular", sd.vertices, sd.normals, sids, sh, sd.lights, sd.camera)


@pytest.mark.parametrize("mode,scene", [(T.MODE_PATH, "sphere"), (T.MODE_REFERENCE, "sphere"),
                                        (T.MODE_PATH_MIS, "sphere"), (T.MODE_PATH_MIS, "emissive"),
                                        (T.MODE_REFERENCE, "specular"), (T.MODE_PATH, "specular"),
                                        (T.MODE_PATH_MIS, "specular")])
def test_adjoint_matches_finite_differences(ctx, mode, scene):
    """MIS: the area light by both strategies (sphere), and emissive
    triangles sampled from the table plus the area light (emissive).
    Specular: the ray-stack replay, with reflected and refracted rays and
    diffuse bounces under them."""
    sd = {"sphere": None, "emissive": scenes.cornell_emissive(area_light=True),
          "specular": _specular_cornell()}[scene]
    sd, sc, p, target = _setup(ctx, mode, sd=sd)
    img = sc.render(p)
    d_image = (2.0 * (img - target)).contiguous()
    d_image[..., 3] = 0.0
    g_sh, g_lt = sc.adjoint(p, d_image)
    g_sh, g_lt = g_sh.cpu().numpy(), g_lt.cpu().numpy()
    # the largest shader gradients (wall, box and sphere triangles) and the light colour
    order = np.argsort(-np.abs(g_sh).ravel())[:6]
    checks = [("shader", int(k // 3), int(k % 3), g_sh.ravel()[k]) for k in order]
    checks += [("light", 0, c, g_lt[0, c]) for c in range(3)]
    for kind, idx, ch, g in checks:
        fd = _fd(sc, sd, p, target, kind, idx, ch)
        assert abs(g - fd) <= 1e-3 * abs(fd) + 1e-6, (kind, idx, ch, g, fd)


def test_adjoint_at_the_differentiable_workload_size(ctx):
    """The differentiable workload as stated: Cornell box + 4096-triangle
    sphere with one shader per triangle, 256x256, 64 spp, depth 4, path mode,
    L2 loss against the frame at albedo + N(0, 0.05); the two largest albedo
    gradients and the light colour gradient against central differences."""
    sd = scenes.cornell_sphere(seed=0)
    sd, sc, p, target = _setup(ctx, T.MODE_PATH, W=256, spp=64, depth=4, sd=sd)
    img = sc.render(p)
    d_image = (2.0 * (img - target)).contiguous()
    d_image[..., 3] = 0.0
    g_sh, g_lt = sc.adjoint(p, d_image)
    g_sh, g_lt = g_sh.cpu().numpy(), g_lt.cpu().numpy()
    order = np.argsort(-np.abs(g_sh).ravel())[:2]
    checks = [("shader", int(k // 3), int(k % 3), g_sh.ravel()[k]) for k in order]
    checks.append(("light", 0, int(np.argmax(np.abs(g_lt[0]))), float(g_lt[0].flat[np.argmax(np.abs(g_lt[0]))])))
    for kind, idx, ch, g in checks:
        fd = _fd(sc, sd, p, target, kind, idx, ch)
        assert abs(g - fd) <= 1e-3 * abs(fd) + 1e-6, (kind, idx, ch, g, fd)


def _emissive_specular():
    """Cornell lit by emissive triangles, with a mirror-like block (reflectivity
    0.6) and a glass-like one (translucence 0.7, index 1.5)."""
    sd = scenes.cornell_emissive(area_light=True)
    sh = np.concatenate([sd.shaders, np.stack([T.lambert((0.9, 0.8, 0.7)), T.lambert((0.7, 0.8, 0.9))])])
    n = sd.shaders.shape[0]
    sh["reflectivity"][n] = 0.6
    sh["translucence"][n + 1] = 0.7
    sh["refractive_index"][n + 1] = 1.5
    sids = sd.shader_ids.copy()
    sids[10:22] = n + 1
    sids[22:34] = n + 2
    return scenes.SceneData("cornell_emissive_specular", sd.vertices, sd.normals, sids, sh, sd.lights, sd.camera)


@pytest.mark.parametrize("mode,scene", [(T.MODE_PATH, "emissive"), (T.MODE_REFERENCE, "emissive_area"),
                                        (T.MODE_PATH_MIS, "emissive"), (T.MODE_PATH_MIS, "emissive_area"),
                                        (T.MODE_PATH, "specular"), (T.MODE_REFERENCE, "specular"),
                                        (T.MODE_PATH_MIS, "specular")])
def test_adjoint_emission_matches_finite_differences(ctx, mode, scene):
    """dLoss/d(emission_color) of the emitters (a ceiling lamp, a glowing
    block, a wall triangle) and of non-emissive walls, whose emission a bounce
    would find, against central differences; in MIS mode the emission colour
    enters the hits' own emission and the emitter samples, while the table
    follows the scalar emission weight and stays fixed. The diffuse and light
    gradients of the same call are unchanged by asking for emission too.
    The render is linear in emission colour, so the central difference is
    exact for any step; h = 1e-2 keeps it above the float32 rounding of the
    frames (at 1e-3 on a colour of 1.6 that rounding reaches 3e-3 relative)."""
    sd = {"emissive": scenes.cornell_emissive(), "emissive_area": scenes.cornell_emissive(area_light=True),
          "specular": _emissive_specular()}[scene]
    sd, sc, p, target = _setup(ctx, mode, sd=sd)
    tsh = sd.shaders.copy()                    # the target also differs in emission
    tsh["emission_color"] = tsh["emission_color"] * (1.0 + np.random.default_rng(2).normal(0, 0.05, (len(tsh), 3)))
    tsh["diffuse_color"] = np.clip(tsh["diffuse_color"] + np.random.default_rng(3).normal(0, 0.05, (len(tsh), 3)), 0, 1)
    sc.set_shaders(tsh)
    target = sc.render(p)
    sc.set_shaders(sd.shaders)
    img = sc.render(p)
    d_image = (2.0 * (img - target)).contiguous()
    d_image[..., 3] = 0.0
    g_sh, g_lt, g_em = (x.cpu().numpy() for x in sc.adjoint(p, d_image, emission=True))
    g_sh0, g_lt0 = (x.cpu().numpy() for x in sc.adjoint(p, d_image))
    assert np.array_equal(g_sh, g_sh0) or np.allclose(g_sh, g_sh0, rtol=1e-5, atol=1e-7)
    assert np.allclose(g_lt, g_lt0, rtol=1e-5, atol=1e-7)
    emitters = [3, 4, 5]
    order = [int(k) for k in np.argsort(-np.abs(g_em).ravel()) if int(k // 3) not in emitters][:2]
    checks = [("emission", int(k // 3), int(k % 3), g_em.ravel()[k]) for k in order]
    # emitters that reach the image (in reference mode only directly seen ones do)
    seen = [s for s in emitters if np.abs(g_em[s]).max() > 0.0]
    assert 3 in seen                             # the ceiling lamp is in view in every mode
    checks += [("emission", s, int(np.argmax(np.abs(g_em[s]))), float(g_em[s].flat[np.argmax(np.abs(g_em[s]))]))
               for s in seen]
    for kind, idx, ch, g in checks:
        assert g != 0.0, (kind, idx, ch)
        fd = _fd(sc, sd, p, target, kind, idx, ch, h=1e-2)
        assert abs(g - fd) <= 1e-3 * abs(fd) + 1e-6, (kind, idx, ch, g, fd)


def _all_lights(sd):
    """Area lights with several samples between a point, an ambient and a
    directional light."""
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


@pytest.mark.parametrize("mode", [T.MODE_PATH, T.MODE_PATH_MIS])
def test_adjoint_with_every_light_type(ctx, mode):
    """Every light type around emissive triangles: the largest shader
    gradients and the colour gradient of each light (those above 1 % of the
    largest) against central differences."""
    sd, sc, p, target = _setup(ctx, mode, sd=_all_lights(scenes.cornell_emissive()))
    img = sc.render(p)
    d_image = (2.0 * (img - target)).contiguous()
    d_image[..., 3] = 0.0
    g_sh, g_lt = sc.adjoint(p, d_image)
    g_sh, g_lt = g_sh.cpu().numpy(), g_lt.cpu().numpy()
    order = np.argsort(-np.abs(g_sh).ravel())[:4]
    checks = [("shader", int(k // 3), int(k % 3), g_sh.ravel()[k]) for k in order]
    big = np.abs(g_lt).max()
    checks += [("light", i, c, g_lt[i, c]) for i in range(5) for c in range(3) if abs(g_lt[i, c]) > 0.01 * big]
    assert len({c[1] for c in checks if c[0] == "light"}) >= 4
    for kind, idx, ch, g in checks:
        fd = _fd(sc, sd, p, target, kind, idx, ch)
        assert abs(g - fd) <= 1e-3 * abs(fd) + 1e-6, (kind, idx, ch, g, fd)


def test_adjoint_through_torch_autograd(ctx):
    import torch
    sd, sc, p, target = _setup(ctx, T.MODE_PATH, W=32, spp=4)

    class Render(torch.autograd.Function):
        @staticmethod
        def forward(fctx, albedo, light_color):
            sh, lt = sd.shaders.copy(), sd.lights.copy()
            sh["diffuse_color"] = albedo.detach().cpu().numpy()
            lt["color"] = light_color.detach().cpu().numpy()
            sc.set_shaders(sh)
            sc.set_lights(lt)
            return sc.render(p)

        @staticmethod
        def backward(fctx, grad_img):
            g = grad_img.contiguous().clone()
            g[..., 3] = 0.0
            d_sh, d_lt = sc.adjoint(p, g)
            return d_sh.cpu().double(), d_lt[: sd.lights.shape[0]].cpu().double()

    albedo = torch.tensor(sd.shaders["diffuse_color"], dtype=torch.float64, requires_grad=True)
    light = torch.tensor(sd.lights["color"], dtype=torch.float64, requires_grad=True)
    img = Render.apply(albedo, light)
    loss = ((img.double() - target.double())[..., :3] ** 2).sum()
    loss.backward()
    k = int(torch.argmax(albedo.grad.abs()))
    fd = _fd(sc, sd, p, target, "shader", k // 3, k % 3)
    assert abs(float(albedo.grad.view(-1)[k]) - fd) <= 1e-3 * abs(fd) + 1e-6
    fdl = _fd(sc, sd, p, target, "light", 0, 1)
    assert abs(float(light.grad[0, 1]) - fdl) <= 1e-3 * abs(fdl) + 1e-6
