"""The C++ host layer (aurora_gb300/host) and its aurora_render driver:
Geometry / Scene / MonteCarloRaytracer over the C ABI, mirroring
data/geometry.cpp, core/scene.cpp and render/monteCarloRaytracer.cpp."""
import json
import subprocess

import numpy as np
import pytest

import oracle
from aurora_gb300 import api, build as ab, scenes, types as T


def _fnv1a(b):
    h = 1469598103934665603
    for x in bytes(b):
        h = ((h ^ x) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


@pytest.fixture(scope="module")
def driver(built):
    return ab.build_host()


def _run(args):
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_scene_file_round_trip(driver, tmp_path):
    sd = scenes.cornell()
    path = tmp_path / "cornell.bin"
    scenes.write_scene_file(sd, str(path))
    out = _run([driver, str(path), "--dry-run"])
    assert out["triangles"] == sd.count
    assert out["shaders"] == sd.shaders.shape[0] and out["lights"] == sd.lights.shape[0]
    assert out["vertex_checksum"] == _fnv1a(sd.vertices.tobytes())
    tsd = scenes.cornell_textured()
    scenes.write_scene_file(tsd, str(path))
    out = _run([driver, str(path), "--dry-run"])
    assert out["textures"] == 2 and out["triangles"] == tsd.count


def test_malformed_scene_file_fails(driver, tmp_path):
    path = tmp_path / "bad.bin"
    path.write_bytes(b"AURSCN1\0" + bytes(10))
    r = subprocess.run([driver, str(path), "--dry-run"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "malformed" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("mode,textured", [("path", False), ("reference", False), ("path", True), ("mis", False)])
def test_driver_render_matches_api(driver, ctx, tmp_path, mode, textured):
    """MonteCarloRaytracer::render (per-sample, 65,536-ray tiles) gives the
    image of the fused renderer bit for bit."""
    sd = scenes.cornell_textured(seed=4) if textured else scenes.cornell_sphere(seed=3, slices=24, stacks=12)
    path = tmp_path / "scene.bin"
    out = tmp_path / "out.pfm"
    scenes.write_scene_file(sd, str(path))
    W, H, spp, depth, seed = 300, 260, 3, 4, 7      # 78,000 rays: two tiles per sample
    _run([driver, str(path), str(out), "--width", str(W), "--height", str(H), "--spp", str(spp),
          "--depth", str(depth), "--seed", str(seed), "--mode", mode])
    img = scenes.read_pfm(str(out))
    m = {"path": T.MODE_PATH, "reference": T.MODE_REFERENCE, "mis": T.MODE_PATH_MIS}[mode]
    sc = api.Scene(ctx, sd)
    if textured:
        sc.set_textures(sd.texcoords, sd.textures)
    ref = sc.render(T.render_params(W, H, spp, depth, seed=seed, mode=m)).cpu().numpy()
    assert np.array_equal(img, ref[..., :3])


@pytest.mark.gpu
def test_geometry_rebuild_matches_oracle(driver, tmp_path):
    """Geometry: staging soup -> padToEven -> copyToDevice -> rebuild
    (aur_nmh_build + aur_nmh_apply) -> generateTB, against the oracle."""
    sd = scenes.cornell_sphere(seed=5, slices=20, stacks=9)
    if sd.count % 2 == 0:                               # exercise the odd-count padding
        sd = scenes.SceneData(sd.name, sd.vertices[:-1], sd.normals[:-1], sd.shader_ids[:-1], sd.shaders,
                              sd.lights, sd.camera)
    path = tmp_path / "odd.bin"
    scenes.write_scene_file(sd, str(path))
    out = _run([driver, str(path), "--geometry-check"])
    perm, levels = oracle.nmh_build(sd.vertices)
    V = oracle.gather9(oracle.pad_even(sd.vertices), perm)
    tb, _ = oracle.generate_tb(oracle.gather9(oracle.pad_even(sd.normals), perm))
    assert out["count"] == perm.shape[0] and out["levels"] == levels
    assert out["perm_checksum"] == _fnv1a(perm.tobytes())
    assert out["vertex_checksum"] == _fnv1a(V.tobytes())
    assert out["tangent_checksum"] == _fnv1a(tb.tobytes())


@pytest.mark.gpu
def test_driver_progressive_and_filter(driver, ctx, tmp_path):
    """render(true) called spp times (one sample pass each, no clearing) ends
    on render(false)'s image; --filter applies cudaFilterPixels (row-below
    clamp fixed) to the finished frame."""
    sd = scenes.cornell()
    path = tmp_path / "c.bin"
    scenes.write_scene_file(sd, str(path))
    W, H, spp = 70, 50, 5
    args = ["--width", str(W), "--height", str(H), "--spp", str(spp), "--depth", "3", "--seed", "2"]
    _run([driver, str(path), str(tmp_path / "prog.pfm"), "--progressive", *args])
    _run([driver, str(path), str(tmp_path / "filt.pfm"), "--filter", *args])
    full = api.Scene(ctx, sd).render(T.render_params(W, H, spp, 3, seed=2, mode=T.MODE_PATH)).cpu().numpy()
    assert np.array_equal(scenes.read_pfm(str(tmp_path / "prog.pfm")), full[..., :3])
    assert np.array_equal(scenes.read_pfm(str(tmp_path / "filt.pfm")), oracle.filter_pixels(full)[..., :3])
