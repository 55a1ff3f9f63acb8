"""Generates the golden fixtures in tests/golden/ (run in a container that has
the reference source tree; the committed .npz files are what the tests read).

Pins, from the reference's own code:
  * traversal: intersect() / intersectAny() of kernels/lib/intersect.cuh,
    compiled unmodified as host C++ (oracle/_ref), on NMH-ordered soups;
  * NMH topology: the literal replay of kernels/rebuilder.cu's kernel
    sequence (oracle/nmh_literal.py) on a soup without key ties.
Also stores oracle renders of a small Cornell frame as regression fixtures.

Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import nmh_literal  # noqa: E402
from aurora_gb300 import scenes, types as T  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def aimed_rays(V, n, seed, tmax=1.0e6):
    """Rays from random origins toward random triangle centroids (mostly hits),
    plus a few axis-parallel rays (zero direction components)."""
    rng = np.random.default_rng(seed)
    V = V.reshape(-1, 9)
    tri = rng.integers(0, V.shape[0], n)
    c = np.stack([V[tri, 0:3].mean(1), V[tri, 3:6].mean(1), V[tri, 6:9].mean(1)], 1)
    o = rng.random((n, 3)) * 1.6 - 0.3
    d = c - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    k = n // 16
    d[:k] = 0.0
    d[np.arange(k), rng.integers(0, 3, k)] = rng.choice([-1.0, 1.0], k)
    r = np.zeros(n, T.ray_dtype)
    r["ox"], r["oy"], r["oz"] = o[:, 0], o[:, 1], o[:, 2]
    r["dx"], r["dy"], r["dz"] = d[:, 0], d[:, 1], d[:, 2]
    r["tmax"] = tmax
    r["tmax"][n // 2:n // 2 + k] = 0.5          # some finite tmax
    return r


def ref_trace(Vn, perm, rays):
    tuv, ids = oracle.ref_trace_closest(Vn, rays)
    aids = oracle.ref_trace_any(Vn, rays)
    prim = np.where(ids >= 0, perm[np.maximum(ids, 0)], T.NO_HIT).astype(np.uint32)
    aprim = np.where(aids >= 0, perm[np.maximum(aids, 0)], T.NO_HIT).astype(np.uint32)
    return tuv, prim, aprim


def main():
    if oracle.ref_lib() is None:
        raise SystemExit("the reference source tree is needed to generate the fixtures")
    # 1. tie-free random soup: topology pinned by the literal rebuilder replay
    for seed in range(100):
        V = scenes.random_soup(2048, seed=1000 + seed)
        if not nmh_literal.has_key_ties(V):
            break
    perm_lit = nmh_literal.rebuild_nmh(V)
    perm, levels = oracle.nmh_build(V)
    assert np.array_equal(perm, perm_lit), "canonical build differs from the literal replay"
    Vn = oracle.gather9(V, perm)
    rays = np.concatenate([aimed_rays(V, 3072, 5), scenes.microbench_rays(1024, seed=6)])
    tuv, prim, aprim = ref_trace(Vn, perm, rays)
    np.savez_compressed(os.path.join(OUT, "soup2048.npz"), vertices=V, perm=perm, levels=levels,
                        rays=rays.view(np.float32).reshape(-1, 8), ref_tuv=tuv, ref_prim=prim, ref_any=aprim)
    # 2. Cornell box (many key ties): canonical topology, reference traversal
    sc = scenes.cornell()
    perm_c, lv_c = oracle.nmh_build(sc.vertices)
    Vc = oracle.gather9(sc.vertices, perm_c)
    cam_rays = oracle.generate_rays(sc.camera, 48, 48, 5, 16)
    r2 = np.zeros(cam_rays.shape[0], T.ray_dtype)
    r2["ox"], r2["oy"], r2["oz"] = cam_rays["pos"][:, 0], cam_rays["pos"][:, 1], cam_rays["pos"][:, 2]
    r2["dx"], r2["dy"], r2["dz"] = cam_rays["dir"][:, 0], cam_rays["dir"][:, 1], cam_rays["dir"][:, 2]
    r2["tmax"] = cam_rays["t"]
    r2 = np.concatenate([r2, aimed_rays(sc.vertices, 1024, 7)])
    tuv2, prim2, aprim2 = ref_trace(Vc, perm_c, r2)
    ns = oracle.NmhScene(sc)
    imgs = {}
    for mode in (T.MODE_REFERENCE, T.MODE_PATH):
        p = T.render_params(32, 32, 4, 4, seed=0, mode=mode)
        imgs["image_mode%d" % mode], _ = oracle.render(ns, p)
    np.savez_compressed(os.path.join(OUT, "cornell.npz"), vertices=sc.vertices, normals=sc.normals,
                        shader_ids=sc.shader_ids, perm=perm_c, levels=lv_c, rays=r2.view(np.float32).reshape(-1, 8),
                        ref_tuv=tuv2, ref_prim=prim2, ref_any=aprim2, camera=np.asarray(sc.camera).reshape(1).view(np.uint8),
                        **imgs)
    print("wrote", os.listdir(OUT))


if __name__ == "__main__":
    main()
