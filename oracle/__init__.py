"""ctypes front end of the oracle (test infrastructure only).

The oracle is the CPU restatement of the reference algorithms in
aur_oracle.cpp. Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use it, and only as the checker or the timed CPU baseline; the
product library never loads it. ref_* functions call the reference's own
traversal code compiled through ref_shim/ (oracle/_ref), available only where
the reference source tree was present at build time.
"""
import ctypes
import os

import numpy as np

from aurora_gb300 import types as T

from .build import ORACLE_SO, REF_SO, build_oracle, build_ref

_lib = None
_ref = None
P = ctypes.c_void_p
U32 = ctypes.c_uint32


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        L.orc_philox4x32_10.argtypes = [P, P, P]
        L.orc_sincos.argtypes = [P, U32, P, P]
        L.orc_calc_partition.argtypes = [U32, P, P]
        L.orc_nmh_build.argtypes = [P, U32, P]
        L.orc_nmh_build.restype = ctypes.c_int
        L.orc_gather9.argtypes = [P, P, U32, P]
        L.orc_trace_closest.argtypes = [P, U32, P, P, U32, P, P, ctypes.c_int]
        L.orc_trace_closest.restype = ctypes.c_uint64
        L.orc_trace_any.argtypes = [P, U32, P, P, U32, P, P, ctypes.c_int]
        L.orc_trace_any.restype = ctypes.c_uint64
        L.orc_brute_closest.argtypes = [P, U32, P, U32, P, ctypes.c_int]
        L.orc_camera_make.argtypes = [P, P, ctypes.c_float, ctypes.c_float, ctypes.c_float, P]
        L.orc_generate_rays.argtypes = [P, U32, U32, U32, U32, P]
        L.orc_render.argtypes = [P, P, P, P, U32, P, U32, P, U32, P, P, P, ctypes.c_int]
        L.orc_render.restype = ctypes.c_uint64
        L.orc_transform.argtypes = [P, P, U32, P, U32, P, P]
        L.orc_generate_tb.argtypes = [P, U32, P, P]
        L.orc_render_textured.argtypes = [P, P, P, P, U32, P, U32, P, U32, P, P, P, ctypes.c_int, P, P, U32]
        L.orc_render_textured.restype = ctypes.c_uint64
        L.orc_texfetch.argtypes = [P, P, U32, P]
        L.orc_filter_pixels.argtypes = [U32, P, P, P]
        L.orc_emitters.argtypes = [P, P, U32, P, P]
        L.orc_draw2.argtypes = [U32, U32, U32, U32, U32, U32, P]
        L.orc_emitters.restype = U32
        L.orc_render_ex.argtypes = [P, P, P, P, U32, P, U32, P, U32, P, P, P, ctypes.c_int, P, P, U32, P, P, P, U32]
        L.orc_render_ex.restype = ctypes.c_uint64
        L.orc_mis_table.argtypes = [P, P, P, U32, U32, P, P, P, P]
        L.orc_mis_table.restype = U32
        L.orc_render_counted.argtypes = [P, P, P, P, U32, P, U32, P, U32, P, P, P, ctypes.c_int, P]
        L.orc_render_counted.restype = ctypes.c_uint64
        L.orc_bsdf_hits.argtypes = [P, P, P, U32, P, U32, P, P, P, U32, P, P, ctypes.c_int, P]
        L.orc_mis_weight.argtypes = [ctypes.c_float, ctypes.c_float]
        L.orc_mis_weight.restype = ctypes.c_float
        L.orc_hit_quad.argtypes = [P, P, P, P]
        L.orc_hit_quad.restype = ctypes.c_int
        _lib = L
    return _lib


def ref_lib():
    """The reference's own traversal compiled as host C++, or None."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            build_ref()
        if not os.path.exists(REF_SO):
            return None
        L = ctypes.CDLL(REF_SO)
        L.ref_trace_closest.argtypes = [P, U32, P, U32, P, P]
        L.ref_trace_any.argtypes = [P, U32, P, U32, P]
        L.ref_uniform_order.restype = ctypes.c_int
        L.ref_shade_hits.argtypes = [P, P, P, P, P, U32, P, U32, P, U32, P, P, P, U32, P, U32, P]
        L.ref_bsdf_hits.argtypes = [P, P, P, P, P, U32, P, U32, P, P, P, U32, P, P, P]
        L.ref_power_heuristic.argtypes = [ctypes.c_float, ctypes.c_float]
        L.ref_power_heuristic.restype = ctypes.c_float
        L.ref_area_hit.argtypes = [P, P, P, P]
        L.ref_area_hit.restype = ctypes.c_int
        L.ref_triangle_areas.argtypes = [P, U32, P]
        _ref = L
    return _ref


def nthreads_default():
    return max(1, os.cpu_count() or 1)


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32); k = np.asarray(key, np.uint32); o = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_ptr(c), _ptr(k), _ptr(o))
    return o


def sincos(x):
    x = np.ascontiguousarray(x, np.float32); s = np.empty_like(x); c = np.empty_like(x)
    lib().orc_sincos(_ptr(x), x.size, _ptr(s), _ptr(c))
    return s, c


def calc_partition(N):
    L = np.zeros(1, np.uint32); R = np.zeros(1, np.uint32)
    lib().orc_calc_partition(N, _ptr(L), _ptr(R))
    return int(L[0]), int(R[0])


def pad_even(vertices):
    """Geometry::padToEven: an odd soup gets a copy of its last triangle."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 9)
    if v.shape[0] % 2:
        v = np.concatenate([v, v[-1:]])
    return v


def nmh_build(vertices):
    """Canonical NMH build. Returns (perm, levels) for the even-padded soup."""
    v = pad_even(vertices)
    perm = np.zeros(v.shape[0], np.uint32)
    lv = lib().orc_nmh_build(_ptr(v), v.shape[0], _ptr(perm))
    if lv < 0:
        raise RuntimeError("orc_nmh_build failed: %d" % lv)
    return perm, lv


def gather9(src, perm):
    src = np.ascontiguousarray(src, np.float32).reshape(-1, 9)
    out = np.empty((perm.shape[0], 9), np.float32)
    lib().orc_gather9(_ptr(src), _ptr(perm), perm.shape[0], _ptr(out))
    return out


def trace_closest(V_nmh, perm, rays, nthreads=None):
    V = np.ascontiguousarray(V_nmh, np.float32); rays = np.ascontiguousarray(rays, T.ray_dtype)
    hits = np.zeros(rays.shape[0], T.hit_dtype); vis = np.zeros(rays.shape[0], np.uint32)
    tot = lib().orc_trace_closest(_ptr(V), V.shape[0], _ptr(perm), _ptr(rays), rays.shape[0], _ptr(hits),
                                  _ptr(vis), nthreads or nthreads_default())
    return hits, vis, int(tot)


def trace_any(V_nmh, perm, rays, nthreads=None):
    V = np.ascontiguousarray(V_nmh, np.float32); rays = np.ascontiguousarray(rays, T.ray_dtype)
    occ = np.zeros(rays.shape[0], np.uint32); vis = np.zeros(rays.shape[0], np.uint32)
    tot = lib().orc_trace_any(_ptr(V), V.shape[0], _ptr(perm), _ptr(rays), rays.shape[0], _ptr(occ),
                              _ptr(vis), nthreads or nthreads_default())
    return occ, vis, int(tot)


def brute_closest(vertices, rays, nthreads=None):
    V = np.ascontiguousarray(vertices, np.float32); rays = np.ascontiguousarray(rays, T.ray_dtype)
    hits = np.zeros(rays.shape[0], T.hit_dtype)
    lib().orc_brute_closest(_ptr(V), V.shape[0], _ptr(rays), rays.shape[0], _ptr(hits),
                            nthreads or nthreads_default())
    return hits


def camera_make(pos, direction, fovx, fovy, aspect=1.0):
    p = np.asarray(pos, np.float32); d = np.asarray(direction, np.float32); c = np.zeros((), T.camera_dtype)
    lib().orc_camera_make(_ptr(p), _ptr(d), fovx, fovy, aspect, _ptr(c))
    return c


def generate_rays(camera, W, H, sample, samples):
    cam = np.asarray(camera, T.camera_dtype).reshape(())
    rays = np.zeros(W * H, T.path_ray_dtype)
    lib().orc_generate_rays(_ptr(cam), W, H, sample, samples, _ptr(rays))
    return rays


def _texture_table(textures):
    imgs = [np.ascontiguousarray(t, np.uint8) for t in textures]
    table = (T.texture_ctype * max(1, len(imgs)))()
    for i, im in enumerate(imgs):
        table[i].width, table[i].height, table[i].rgba = im.shape[1], im.shape[0], im.ctypes.data
    return table, imgs


def texfetch(texture, uv):
    """Bilinear, wrapping fetch of an (H, W, 4) uint8 texture at (n, 2) uv."""
    table, keep = _texture_table([texture])
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    rgb = np.zeros((uv.shape[0], 3), np.float32)
    lib().orc_texfetch(ctypes.c_void_p(ctypes.addressof(table)), _ptr(uv), uv.shape[0], _ptr(rgb))
    return rgb


def emitters(nscene):
    """cudaCreateEmitters over an NmhScene: the emitter records (emitter_dtype)."""
    out = np.zeros(nscene.V.shape[0], T.emitter_dtype)
    m = lib().orc_emitters(_ptr(nscene.V), _ptr(nscene.S), nscene.V.shape[0], _ptr(nscene.shaders), _ptr(out))
    return out[:m]


def filter_pixels(img, region=None):
    """cudaFilterPixels with the row-below clamp fixed: img (H, W, 4) float32;
    region (left, right, bottom, top) inclusive, default the whole frame.
    Returns a copy of img with the region filtered."""
    img = np.ascontiguousarray(img, np.float32)
    H, W = img.shape[:2]
    reg = np.array(region if region is not None else (0, W - 1, 0, H - 1), np.uint32)
    out = img.copy()
    lib().orc_filter_pixels(W, _ptr(reg), _ptr(img), _ptr(out))
    return out


class NmhScene:
    """A scene reordered into NMH order, as the renderer consumes it."""

    def __init__(self, scene, perm=None):
        self.input_count = int(np.asarray(scene.vertices).reshape(-1, 9).shape[0])
        V = pad_even(scene.vertices)
        N = pad_even(scene.normals)
        S = scene.shader_ids
        if S.shape[0] % 2:
            S = np.concatenate([S, S[-1:]])
        if perm is None:
            perm, _ = nmh_build(V)
        self.perm = np.ascontiguousarray(perm, np.uint32)
        self.V = gather9(V, self.perm)
        self.N = gather9(N, self.perm)
        self.S = np.ascontiguousarray(S[self.perm], np.uint16)
        self.shaders = np.ascontiguousarray(scene.shaders, T.shader_dtype)
        self.lights = np.ascontiguousarray(scene.lights, T.light_dtype)
        self.camera = np.asarray(scene.camera, T.camera_dtype).reshape(())
        self.textures = list(getattr(scene, "textures", None) or [])
        tc = getattr(scene, "texcoords", None)
        self.TC = None
        if tc is not None:
            tc = np.ascontiguousarray(tc, np.float32).reshape(-1, 6)
            if tc.shape[0] % 2:
                tc = np.concatenate([tc, tc[-1:]])
            self.TC = np.ascontiguousarray(tc[self.perm])


def mis_table(nscene):
    """The light-selection table of AUR_MODE_PATH_MIS: (triangles, cdf, pa)
    with pa per NMH triangle."""
    n = nscene.V.shape[0]
    tri = np.zeros(n, np.uint32)
    cdf = np.zeros(n, np.float32)
    pa = np.zeros(n, np.float32)
    m = lib().orc_mis_table(_ptr(nscene.V), _ptr(nscene.S), _ptr(nscene.perm), n, nscene.input_count,
                            _ptr(nscene.shaders), _ptr(tri), _ptr(cdf), _ptr(pa))
    return tri[:m].copy(), cdf[:m].copy(), pa


def render(nscene, params, camera=None, accum=None, nthreads=None, table=None):
    """Adds the requested samples into accum (H, W, 4) float32 and returns
    (accum, node fetches). For AUR_MODE_PATH_MIS, `table` is the
    light-selection table (triangles, cdf, pa) to sample; default the
    oracle's own (mis_table)."""
    p = np.asarray(params, T.params_dtype).reshape(())
    W, H = int(p["width"]), int(p["height"])
    if accum is None:
        accum = np.zeros((H, W, 4), np.float32)
    cam = np.asarray(nscene.camera if camera is None else camera, T.camera_dtype).reshape(())
    if int(p["mode"]) == T.MODE_PATH_MIS:
        tri, cdf, pa = mis_table(nscene) if table is None else table
        tri = np.ascontiguousarray(tri, np.uint32)
        cdf = np.ascontiguousarray(cdf, np.float32)
        pa = np.ascontiguousarray(pa, np.float32)
        assert pa.shape[0] == nscene.V.shape[0] and tri.shape[0] == cdf.shape[0]
        table_t, keep = _texture_table(nscene.textures)
        tot = lib().orc_render_ex(_ptr(nscene.V), _ptr(nscene.N), _ptr(nscene.S), _ptr(nscene.perm),
                                  nscene.V.shape[0], _ptr(nscene.shaders), nscene.shaders.shape[0],
                                  _ptr(nscene.lights), nscene.lights.shape[0], _ptr(cam), _ptr(p), _ptr(accum),
                                  nthreads or nthreads_default(), _ptr(nscene.TC),
                                  ctypes.c_void_p(ctypes.addressof(table_t)) if keep else ctypes.c_void_p(0),
                                  len(keep), _ptr(tri), _ptr(cdf), _ptr(pa), tri.shape[0])
        return accum, int(tot)
    if nscene.TC is not None:
        table, keep = _texture_table(nscene.textures)
        tot = lib().orc_render_textured(_ptr(nscene.V), _ptr(nscene.N), _ptr(nscene.S), _ptr(nscene.perm),
                                        nscene.V.shape[0], _ptr(nscene.shaders), nscene.shaders.shape[0],
                                        _ptr(nscene.lights), nscene.lights.shape[0], _ptr(cam), _ptr(p), _ptr(accum),
                                        nthreads or nthreads_default(), _ptr(nscene.TC),
                                        ctypes.c_void_p(ctypes.addressof(table)), len(keep))
        return accum, int(tot)
    tot = lib().orc_render(_ptr(nscene.V), _ptr(nscene.N), _ptr(nscene.S), _ptr(nscene.perm),
                           nscene.V.shape[0], _ptr(nscene.shaders), nscene.shaders.shape[0],
                           _ptr(nscene.lights), nscene.lights.shape[0], _ptr(cam), _ptr(p), _ptr(accum),
                           nthreads or nthreads_default())
    return accum, int(tot)


def ref_trace_closest(V_nmh, rays):
    """Reference intersect(): (t, u, v) float32 (n,3) and NMH position (n,)."""
    L = ref_lib()
    V = np.ascontiguousarray(V_nmh, np.float32); rays = np.ascontiguousarray(rays, T.ray_dtype)
    tuv = np.zeros((rays.shape[0], 3), np.float32); ids = np.zeros(rays.shape[0], np.int32)
    L.ref_trace_closest(_ptr(V), V.shape[0], _ptr(rays), rays.shape[0], _ptr(tuv), _ptr(ids))
    return tuv, ids


def draw2(seed, scene, pixel, sample, ray, slot):
    """The integrators' two uniforms at one counter-RNG slot."""
    out = np.zeros(2, np.float32)
    lib().orc_draw2(seed, scene, pixel, sample, ray, slot, _ptr(out))
    return float(out[0]), float(out[1])


def ref_uniform_order():
    """0 if the reference's area-light sample scales e1 by the first uniform drawn, 1 if by the second."""
    return ref_lib().ref_uniform_order()


def ref_shade_hits(nscene, tangents, bitangents, rays8, tri, tuv, uniforms):
    """Li at camera-ray hits through the reference's own shading code (raytrace()'s light loop)."""
    n = rays8.shape[0]
    u = np.ascontiguousarray(uniforms, np.float32).reshape(n, -1)
    out = np.zeros((n, 3), np.float32)
    # converted copies are held in locals: the call reads them through pointers
    tg, bt = np.ascontiguousarray(tangents, np.float32), np.ascontiguousarray(bitangents, np.float32)
    r8, tr, tv = (np.ascontiguousarray(rays8, np.float32), np.ascontiguousarray(tri, np.int32),
                  np.ascontiguousarray(tuv, np.float32))
    ref_lib().ref_shade_hits(_ptr(nscene.V), _ptr(nscene.N), _ptr(tg), _ptr(bt), _ptr(nscene.S), nscene.V.shape[0],
                             _ptr(nscene.shaders), nscene.shaders.shape[0], _ptr(nscene.lights),
                             nscene.lights.shape[0], _ptr(r8), _ptr(tr), _ptr(tv), n, _ptr(u), u.shape[1], _ptr(out))
    return out


def ref_trace_any(V_nmh, rays):
    L = ref_lib()
    V = np.ascontiguousarray(V_nmh, np.float32); rays = np.ascontiguousarray(rays, T.ray_dtype)
    ids = np.zeros(rays.shape[0], np.int32)
    L.ref_trace_any(_ptr(V), V.shape[0], _ptr(rays), rays.shape[0], _ptr(ids))
    return ids


def transform(vertices, normals, transforms, dst_vertices=None, dst_normals=None):
    """cudaTransform restated: returns world-space (vertices, normals)."""
    V = np.ascontiguousarray(vertices, np.float32).reshape(-1, 9)
    N = np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
    xf = np.ascontiguousarray(transforms, T.object_transform_dtype)
    dv = np.zeros_like(V) if dst_vertices is None else np.array(dst_vertices, np.float32)
    dn = np.zeros_like(N) if dst_normals is None else np.array(dst_normals, np.float32)
    lib().orc_transform(_ptr(V), _ptr(N), V.shape[0], _ptr(xf), xf.shape[0], _ptr(dv), _ptr(dn))
    return dv, dn


def generate_tb(normals):
    N = np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
    t = np.zeros_like(N); b = np.zeros_like(N)
    lib().orc_generate_tb(_ptr(N), N.shape[0], _ptr(t), _ptr(b))
    return t, b


def bsdf_hits(nscene, rays8, tri, tuv, uniforms, probes, tangents=None, bitangents=None, reference=False,
              mis=False):
    """BSDF sampling at hits: (n, 6) = sampled wi.xyz, its pdf, pdf(wo, wi),
    pdf(wo, probe). The oracle's path-mode bounce (or, mis=True, the MIS
    mode's orthonormal-frame sampling), or (reference=True, with the tangent
    frames) the reference's own BSDF::samplef and BSDF::pdf."""
    n = rays8.shape[0]
    out = np.zeros((n, 6), np.float32)
    keep = [np.ascontiguousarray(a, t) for a, t in ((rays8, np.float32), (tri, np.int32), (tuv, np.float32),
                                                    (uniforms, np.float32), (probes, np.float32))]
    args = [_ptr(keep[0]), _ptr(keep[1]), _ptr(keep[2]), n, _ptr(keep[3]), _ptr(keep[4]), _ptr(out)]
    if reference:
        tb = [np.ascontiguousarray(tangents, np.float32), np.ascontiguousarray(bitangents, np.float32)]
        ref_lib().ref_bsdf_hits(_ptr(nscene.V), _ptr(nscene.N), _ptr(tb[0]), _ptr(tb[1]), _ptr(nscene.S),
                                nscene.V.shape[0], _ptr(nscene.shaders), nscene.shaders.shape[0], *args)
    else:
        lib().orc_bsdf_hits(_ptr(nscene.V), _ptr(nscene.N), _ptr(nscene.S), nscene.V.shape[0], _ptr(nscene.shaders),
                            nscene.shaders.shape[0], *args[:-1], 1 if mis else 0, args[-1])
    return out


def mis_weight(a, b, reference=False):
    """The oracle's MIS weight 1 / (1 + (b/a)^2), or the reference's powerHeuristic(1, a, 1, b)."""
    return (ref_lib().ref_power_heuristic if reference else lib().orc_mis_weight)(a, b)


def area_hit(light, pos, direction, reference=False):
    """(hit, t) of a ray against an area light's quad: the oracle's hitQuad or
    the reference's Light::visibleArea with nothing to occlude."""
    lt = np.ascontiguousarray(light, T.light_dtype).reshape(())
    p = np.ascontiguousarray(pos, np.float32)           # held here: the call reads them through pointers
    d = np.ascontiguousarray(direction, np.float32)
    t = np.zeros(1, np.float32)
    f = ref_lib().ref_area_hit if reference else lib().orc_hit_quad
    h = f(_ptr(lt), _ptr(p), _ptr(d), _ptr(t))
    return bool(h), float(t[0])


def render_counted(nscene, params, camera=None, nthreads=None):
    """orc_render of an untextured scene in reference or path mode: (accum,
    node fetches of the reference algorithm, shading points)."""
    p = np.asarray(params, T.params_dtype).reshape(())
    accum = np.zeros((int(p["height"]), int(p["width"]), 4), np.float32)
    cam = np.asarray(nscene.camera if camera is None else camera, T.camera_dtype).reshape(())
    sp = np.zeros(1, np.uint64)
    tot = lib().orc_render_counted(_ptr(nscene.V), _ptr(nscene.N), _ptr(nscene.S), _ptr(nscene.perm),
                                   nscene.V.shape[0], _ptr(nscene.shaders), nscene.shaders.shape[0],
                                   _ptr(nscene.lights), nscene.lights.shape[0], _ptr(cam), _ptr(p), _ptr(accum),
                                   nthreads or nthreads_default(), _ptr(sp))
    return accum, int(tot), int(sp[0])


def ref_triangle_areas(V):
    """Primitive3::area of each triangle (reference layout, (n, 9))."""
    V = np.ascontiguousarray(V, np.float32).reshape(-1, 9)
    out = np.zeros(V.shape[0], np.float32)
    ref_lib().ref_triangle_areas(_ptr(V), V.shape[0], _ptr(out))
    return out
