"""The warp-packet traversal (traverse_packet, aur_traverse.cuh) against the
one-ray-per-lane traversal and the reference's own walk (intersect.cuh:
36-152), all three restated step by step in plain C (tests/packet_model.c)
and run on the CPU over NMHs the oracle builds. A packet of 32 rays of one
direction octant must give every ray its own closest hit (index and the bits
of t, u, v) and any-hit occluder. The GPU kernels are compared with the
oracle in tests/test_gpu_trace.py; this checks the packet rule itself over
many more packets, including the hard ones: diverging directions, coplanar
duplicates (ties in t), axis-parallel rays with +0 and -0 components, rays
ending before any hit."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from aurora_gb300 import scenes, types as T

HERE = os.path.dirname(os.path.abspath(__file__))


def _octant_chunks(rng, chunks, spread):
    n = 32 * chunks
    rays = np.zeros(n, T.ray_dtype)
    centre = np.repeat(rng.random((chunks, 3)), 32, axis=0)
    o = centre * (1.0 - spread) + rng.random((n, 3)) * spread
    d = np.abs(rng.normal(size=(n, 3)))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    octs = np.repeat(rng.integers(0, 8, chunks), 32)
    for a in range(3):
        d[:, a] = np.where((octs >> a) & 1, -d[:, a], d[:, a])
    rays["ox"], rays["oy"], rays["oz"] = o.astype(np.float32).T
    rays["dx"], rays["dy"], rays["dz"] = d.astype(np.float32).T
    rays["tmax"] = 1e6
    return rays


def _camera_chunks(rng, chunks):
    """Pinhole rays of 32 neighbouring pixels per chunk (one quadrant each)."""
    rays = np.zeros(32 * chunks, T.ray_dtype)
    for c in range(chunks):
        cx, cy = rng.random(2) * 0.8 + 0.1
        x = cx + (np.arange(32) % 8) * 1e-3
        y = cy + (np.arange(32) // 8) * 1e-3
        d = np.stack([x - 0.5, y - 0.5, np.ones(32)], 1)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        s = slice(32 * c, 32 * c + 32)
        rays["ox"][s], rays["oy"][s], rays["oz"][s] = 0.5, 0.5, -1.0
        rays["dx"][s], rays["dy"][s], rays["dz"][s] = d.astype(np.float32).T
    rays["tmax"] = 1e6
    return rays


@pytest.fixture(scope="module")
def model_exe():
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "packet_model")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math",
                           os.path.join(HERE, "packet_model.c"), "-o", exe, "-lm"])
    return exe


def _run(exe, V, rays):
    perm, _ = oracle.nmh_build(V)
    Vn = oracle.gather9(oracle.pad_even(V), perm)
    with tempfile.TemporaryDirectory() as d:
        paths = [os.path.join(d, f) for f in ("v", "p", "r")]
        Vn.astype(np.float32).tofile(paths[0])
        perm.astype(np.uint32).tofile(paths[1])
        np.ascontiguousarray(rays).tofile(paths[2])
        out = subprocess.run([exe, *paths, str(Vn.shape[0]), str(rays.shape[0])], capture_output=True, text=True)
    n, bad = (int(x) for x in out.stdout.split())
    assert n == rays.shape[0]
    assert bad == 0, out.stderr
    return n


@pytest.mark.parametrize("n_tris", [1, 2, 7, 300, 20000])
def test_packets_equal_per_lane_and_reference(model_exe, n_tris):
    rng = np.random.default_rng(n_tris)
    V = scenes.random_soup(n_tris, seed=n_tris)
    rays = np.concatenate([_octant_chunks(rng, 40, 0.004), _octant_chunks(rng, 20, 1.0), _camera_chunks(rng, 20)])
    assert _run(model_exe, V, rays) == 32 * 80


def test_packets_with_ties_zero_components_and_short_rays(model_exe):
    rng = np.random.default_rng(3)
    V = scenes.random_soup(3000, seed=5)
    V[2000:2200] = V[100:300]                       # coincident copies: ties in t
    rays = _octant_chunks(rng, 30, 0.01)
    # chunks of axis-parallel rays through the duplicated triangles' centres,
    # alternating +0 and -0 in the other two components
    c = np.stack([V[100:132, 0:3].mean(1), V[100:132, 3:6].mean(1), V[100:132, 6:9].mean(1)], 1)
    ax = np.zeros(96, T.ray_dtype)
    for a in range(3):
        s = slice(32 * a, 32 * a + 32)
        o = c.copy()
        o[:, a] -= 2.0
        ax["ox"][s], ax["oy"][s], ax["oz"][s] = o.astype(np.float32).T
        z = np.where(np.arange(32) % 2, -0.0, 0.0).astype(np.float32)
        comps = [z, z, z]
        comps[a] = np.ones(32, np.float32)
        ax["dx"][s], ax["dy"][s], ax["dz"][s] = comps
    ax["tmax"] = 1e6
    short = _octant_chunks(rng, 10, 0.004)
    short["tmax"] = rng.random(320).astype(np.float32) * 0.05    # most end before a hit
    assert _run(model_exe, V, np.concatenate([rays, ax, short])) == 32 * 43
