"""ctypes front end of libaurora_gb300.so (the C ABI of include/aurora_gb300.h).

Device memory and the launch stream come from torch: a Context launches on
torch's current CUDA stream, so its work is ordered with torch's own. Every
call raises AuroraError when the library returns a non-zero status. Nothing
here computes on the CPU: the CUDA library must be built (build.py) and a
GPU present, otherwise loading fails loudly.
"""
import ctypes
import json
import os

import numpy as np

from . import types as T
from .build import LIB

_lib = None
P = ctypes.c_void_p
U32 = ctypes.c_uint32


class AuroraError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("aurora_gb300 status %d: %s" % (status, message))
        self.status = status


SIGNATURES = {
    "aur_last_error": ([], ctypes.c_char_p),
    "aur_version": ([], ctypes.c_char_p),
    "aur_debug_fail_allocation": ([U32], ctypes.c_int),
    "aur_ctx_create": ([ctypes.c_int, P], ctypes.c_int),
    "aur_ctx_destroy": ([P], ctypes.c_int),
    "aur_ctx_set_stream": ([P, P], ctypes.c_int),
    "aur_ctx_get_stream": ([P, P], ctypes.c_int),
    "aur_ctx_synchronize": ([P], ctypes.c_int),
    "aur_ctx_sm_count": ([P, P], ctypes.c_int),
    "aur_nmh_build": ([P, P, U32, P], ctypes.c_int),
    "aur_debug_lookback_timeout": ([P, U32], ctypes.c_int),
    "aur_debug_nmh_drop_texture": ([P], ctypes.c_int),
    "aur_debug_trace_deferred": ([P, P], ctypes.c_int),
    "aur_nmh_destroy": ([P], ctypes.c_int),
    "aur_nmh_info": ([P, P, P], ctypes.c_int),
    "aur_nmh_export": ([P, P, P, P], ctypes.c_int),
    "aur_nmh_perm_device": ([P, P], ctypes.c_int),
    "aur_nmh_build_noalloc": ([P, U32, P, P, P, P, P], ctypes.c_int),
    "aur_nmh_apply": ([P, P, P, U32, P], ctypes.c_int),
    "aur_malloc": ([P, ctypes.c_size_t, ctypes.c_int, P], ctypes.c_int),
    "aur_free": ([P, P, ctypes.c_int], ctypes.c_int),
    "aur_memzero": ([P, P, ctypes.c_size_t, ctypes.c_int], ctypes.c_int),
    "aur_memupload": ([P, P, P, ctypes.c_size_t, ctypes.c_int], ctypes.c_int),
    "aur_memdownload": ([P, P, P, ctypes.c_size_t], ctypes.c_int),
    "aur_trace_closest": ([P, P, P, U32, P], ctypes.c_int),
    "aur_trace_any": ([P, P, P, U32, P], ctypes.c_int),
    "aur_trace_closest_host": ([P, P, P, U32, P], ctypes.c_int),
    "aur_trace_any_host": ([P, P, P, U32, P], ctypes.c_int),
    "aur_trace_count_visits": ([P, P, P, U32, P], ctypes.c_int),
    "aur_trace_stats": ([P, P, P, U32, P, P], ctypes.c_int),
    "aur_scene_create": ([P, P, P, P, U32, P, U32, P, U32, P], ctypes.c_int),
    "aur_scene_destroy": ([P], ctypes.c_int),
    "aur_scene_nmh": ([P, P], ctypes.c_int),
    "aur_scene_set_shaders": ([P, P, P, U32], ctypes.c_int),
    "aur_scene_set_lights": ([P, P, P, U32], ctypes.c_int),
    "aur_scene_set_textures": ([P, P, P, P, U32], ctypes.c_int),
    "aur_scene_texfetch": ([P, P, U32, P, U32, P], ctypes.c_int),
    "aur_scene_emitters": ([P, P, P, P], ctypes.c_int),
    "aur_scene_mis_table": ([P, P, P, P, P, P], ctypes.c_int),
    "aur_camera_make": None,  # struct-by-value arguments; not bound
    "aur_render": ([P, P, P, P, P], ctypes.c_int),
    "aur_generate_rays": ([P, U32, U32, U32, U32, P, P, P], ctypes.c_int),
    "aur_raytrace_monte_carlo": ([P, P, P, U32, U32, U32, P, P], ctypes.c_int),
    "aur_draw_pixels": ([P, U32, U32, ctypes.c_float, P, P], ctypes.c_int),
    "aur_clear_pixels": ([P, U32, U32, P], ctypes.c_int),
    "aur_filter_pixels": ([P, U32, U32, P, P, P], ctypes.c_int),
    "aur_accum_save": ([P, ctypes.c_char_p, U32, U32, U32, U32, P], ctypes.c_int),
    "aur_accum_load": ([P, ctypes.c_char_p, U32, U32, P, P, P], ctypes.c_int),
    "aur_debug_nmh_layout": ([U32, U32, P], ctypes.c_int),
    "aur_batch_create": ([P, P, P, P, U32, P, P], ctypes.c_int),
    "aur_batch_render": ([P, P, P], ctypes.c_int),
    "aur_batch_status": ([P, P, P], ctypes.c_int),
    "aur_batch_tuning": ([P, P], ctypes.c_int),
    "aur_batch_destroy": ([P], ctypes.c_int),
    "aur_batch_autotune": ([P, P, P, P, U32, P, P], ctypes.c_int),
    "aur_render_adjoint": ([P, P, P, P, P, P, P, P], ctypes.c_int),
    "aur_batch_profile": ([P, P, P, P], ctypes.c_int),
    "aur_batch_counters": ([P, P, P], ctypes.c_int),
    "aur_transform": ([P, P, P, U32, P, U32, P, P], ctypes.c_int),
    "aur_generate_tb": ([P, P, U32, P, P], ctypes.c_int),
}


def lib():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError("libaurora_gb300.so is not built (run aurora_gb300.build.build())")
        L = ctypes.CDLL(LIB)
        for name, sig in SIGNATURES.items():
            fn = getattr(L, name)
            if sig is not None:
                fn.argtypes, fn.restype = sig
        _lib = L
    return _lib


def check(status):
    if status != 0:
        raise AuroraError(status, lib().aur_last_error().decode())


def _dense(t):
    """The tensor itself if it is contiguous. The library reads device memory
    asynchronously on its own stream, so a temporary contiguous copy could be
    freed and reused before the read: callers pass contiguous tensors."""
    if not t.is_contiguous():
        raise ValueError("aurora_gb300: pass a contiguous tensor (the library reads it asynchronously)")
    return t


def _ptr(x):
    """Address of a numpy array / torch tensor / None."""
    if x is None:
        return P(0)
    if isinstance(x, np.ndarray):
        return P(x.ctypes.data)
    return P(x.data_ptr())


def _torch():
    import torch
    return torch


class Context:
    """aur_ctx on one device, launching on torch's current stream."""

    def __init__(self, device=0):
        torch = _torch()
        self.device = device
        self.handle = None
        h = P()
        check(lib().aur_ctx_create(device, ctypes.byref(h)))
        self.handle = h
        torch.cuda.set_device(device)
        self.use_torch_stream()

    def use_torch_stream(self):
        torch = _torch()
        h = torch.cuda.current_stream(self.device).cuda_stream
        # torch's default stream is the legacy default stream, handle 0; the
        # ABI reads NULL as "the context's own stream", so name it explicitly
        # as cudaStreamLegacy ((cudaStream_t)0x1).
        check(lib().aur_ctx_set_stream(self.handle, P(h if h else 1)))

    def synchronize(self):
        check(lib().aur_ctx_synchronize(self.handle))

    def sm_count(self):
        v = ctypes.c_int()
        check(lib().aur_ctx_sm_count(self.handle, ctypes.byref(v)))
        return v.value

    def close(self):
        if self.handle:
            lib().aur_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Nmh:
    """aur_nmh built from a device tensor of count*9 float32 vertices."""

    def __init__(self, ctx, vertices_dev, count=None, handle=None):
        self.ctx = ctx
        self.owned = handle is None
        self.handle = None
        if handle is None:
            count = vertices_dev.numel() // 9 if count is None else count
            h = P()
            check(lib().aur_nmh_build(ctx.handle, _ptr(vertices_dev), count, ctypes.byref(h)))
            handle = h
        self.handle = handle

    def info(self):
        c, lv = U32(), U32()
        check(lib().aur_nmh_info(self.handle, ctypes.byref(c), ctypes.byref(lv)))
        return c.value, lv.value

    def export(self, with_vertices=True):
        count, _ = self.info()
        perm = np.zeros(count, np.uint32)
        verts = np.zeros((count, 9), np.float32) if with_vertices else None
        check(lib().aur_nmh_export(self.ctx.handle, self.handle, _ptr(perm), _ptr(verts)))
        return perm, verts

    def close(self):
        if self.handle and self.owned:
            lib().aur_nmh_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rays_tensor(rays_np, device="cuda"):
    """numpy ray_dtype records -> (n, 8) float32 device tensor (same bytes)."""
    torch = _torch()
    a = np.ascontiguousarray(rays_np, T.ray_dtype).view(np.float32).reshape(-1, 8)
    return torch.from_numpy(a).to(device)


def trace_closest(ctx, nmh, rays_dev, hits_dev=None):
    torch = _torch()
    n = rays_dev.shape[0]
    if hits_dev is None:
        hits_dev = torch.empty((n, 4), dtype=torch.float32, device=rays_dev.device)
    check(lib().aur_trace_closest(ctx.handle, nmh.handle, _ptr(rays_dev), n, _ptr(hits_dev)))
    return hits_dev


def trace_any(ctx, nmh, rays_dev, occ_dev=None):
    torch = _torch()
    n = rays_dev.shape[0]
    if occ_dev is None:
        occ_dev = torch.empty((n,), dtype=torch.int32, device=rays_dev.device)
    check(lib().aur_trace_any(ctx.handle, nmh.handle, _ptr(rays_dev), n, _ptr(occ_dev)))
    return occ_dev


def hits_to_numpy(hits_dev):
    return hits_dev.cpu().numpy().view(T.hit_dtype).reshape(-1)


def trace_deferred(ctx):
    """Chunks of 32 rays that the context's last device trace left to the
    one-ray-per-thread kernel (test hook)."""
    c = ctypes.c_uint32()
    check(lib().aur_debug_trace_deferred(ctx.handle, ctypes.byref(c)))
    return c.value


def trace_closest_host(ctx, nmh, rays_host, hits_host):
    check(lib().aur_trace_closest_host(ctx.handle, nmh.handle, _ptr(rays_host), rays_host.shape[0], _ptr(hits_host)))
    return hits_host


def trace_any_host(ctx, nmh, rays_host, occ_host):
    check(lib().aur_trace_any_host(ctx.handle, nmh.handle, _ptr(rays_host), rays_host.shape[0], _ptr(occ_host)))
    return occ_host


def count_visits(ctx, nmh, rays_dev):
    out = (ctypes.c_ulonglong * 2)()
    check(lib().aur_trace_count_visits(ctx.handle, nmh.handle, _ptr(rays_dev), rays_dev.shape[0], out))
    return int(out[0]), int(out[1])


def trace_stats(ctx, nmh, rays_dev):
    """Work of the shipped (box-pruned) traversal: per kind ("closest",
    "any") the node fetches, slab crossings and child-box loads."""
    c = (ctypes.c_ulonglong * 3)()
    a = (ctypes.c_ulonglong * 3)()
    check(lib().aur_trace_stats(ctx.handle, nmh.handle, _ptr(rays_dev), rays_dev.shape[0], c, a))
    keys = ("node_fetches", "slab_crossings", "box_loads")
    return {"closest": dict(zip(keys, map(int, c))), "any": dict(zip(keys, map(int, a)))}


class Scene:
    """aur_scene from a scenes.SceneData (host arrays)."""

    def __init__(self, ctx, sd):
        self.ctx = ctx
        self.data = sd
        self.handle = None
        h = P()
        check(lib().aur_scene_create(ctx.handle, _ptr(sd.vertices), _ptr(sd.normals), _ptr(sd.shader_ids), sd.count,
                                     _ptr(sd.shaders), sd.shaders.shape[0], _ptr(sd.lights), sd.lights.shape[0],
                                     ctypes.byref(h)))
        self.handle = h
        nh = P()
        check(lib().aur_scene_nmh(self.handle, ctypes.byref(nh)))
        self.nmh = Nmh(ctx, None, handle=nh)

    def set_shaders(self, shaders):
        shaders = np.ascontiguousarray(shaders, T.shader_dtype)
        check(lib().aur_scene_set_shaders(self.ctx.handle, self.handle, _ptr(shaders), shaders.shape[0]))

    def set_textures(self, texcoords, textures):
        """texcoords: (count, 6) float32 in the original triangle order;
        textures: list of (height, width, 4) uint8 RGBA images."""
        tc = np.ascontiguousarray(texcoords, np.float32).reshape(-1, 6)
        imgs = [np.ascontiguousarray(t, np.uint8) for t in textures]
        table = (T.texture_ctype * max(1, len(imgs)))()
        for i, im in enumerate(imgs):
            table[i].width, table[i].height = im.shape[1], im.shape[0]
            table[i].rgba = im.ctypes.data
        check(lib().aur_scene_set_textures(self.ctx.handle, self.handle, _ptr(tc), P(ctypes.addressof(table)),
                                           len(imgs)))
        self._textures = imgs

    def emitters(self):
        """The scene's emissive-triangle table (numpy, emitter_dtype)."""
        import torch
        n = self.nmh.info()[0]
        buf = torch.empty((max(1, n) * T.emitter_dtype.itemsize,), dtype=torch.uint8, device="cuda")
        m = ctypes.c_uint32(0)
        check(lib().aur_scene_emitters(self.ctx.handle, self.handle, _ptr(buf), ctypes.byref(m)))
        return buf[:m.value * T.emitter_dtype.itemsize].cpu().numpy().view(T.emitter_dtype)

    def mis_table(self):
        """The light-selection table of AUR_MODE_PATH_MIS as numpy arrays
        (triangles, cdf, pa per NMH triangle)."""
        n = self.nmh.info()[0]
        tri = np.zeros(max(1, n), np.uint32)
        cdf = np.zeros(max(1, n), np.float32)
        pa = np.zeros(max(1, n), np.float32)
        m = ctypes.c_uint32(0)
        check(lib().aur_scene_mis_table(self.ctx.handle, self.handle, _ptr(tri), _ptr(cdf), _ptr(pa),
                                        ctypes.byref(m)))
        return tri[:m.value].copy(), cdf[:m.value].copy(), pa[:n].copy()

    def texfetch(self, texture, uv_dev):
        """RGB of texture `texture` (1-based) at n device (u, v) pairs."""
        import torch
        out = torch.empty((uv_dev.shape[0], 3), dtype=torch.float32, device="cuda")
        uv = _dense(uv_dev)
        check(lib().aur_scene_texfetch(self.ctx.handle, self.handle, texture, _ptr(uv), uv.shape[0], _ptr(out)))
        return out

    def set_lights(self, lights):
        lights = np.ascontiguousarray(lights, T.light_dtype)
        check(lib().aur_scene_set_lights(self.ctx.handle, self.handle, _ptr(lights), lights.shape[0]))

    def render(self, params, camera=None, accum=None):
        """Adds the samples of `params` into accum (H, W, 4) float32 device tensor."""
        torch = _torch()
        p = np.asarray(params, T.params_dtype).reshape(())
        if accum is None:
            accum = torch.zeros((int(p["height"]), int(p["width"]), 4), dtype=torch.float32, device="cuda")
        cam = np.asarray(self.data.camera if camera is None else camera, T.camera_dtype).reshape(())
        check(lib().aur_render(self.ctx.handle, self.handle, _ptr(cam), _ptr(p), _ptr(accum)))
        return accum

    def adjoint(self, params, d_image, d_diffuse=None, d_light=None, camera=None, d_emission=None,
                emission=False):
        """Adds dLoss/d(diffuse_color) and dLoss/d(light color) for
        dLoss/d(image); with emission=True (or a d_emission buffer) also
        dLoss/d(emission_color), returned third."""
        torch = _torch()
        p = np.asarray(params, T.params_dtype).reshape(())
        if d_diffuse is None:
            d_diffuse = torch.zeros((self.data.shaders.shape[0], 3), dtype=torch.float32, device="cuda")
        if d_light is None:
            d_light = torch.zeros((max(1, self.data.lights.shape[0]), 3), dtype=torch.float32, device="cuda")
        if emission and d_emission is None:
            d_emission = torch.zeros((self.data.shaders.shape[0], 3), dtype=torch.float32, device="cuda")
        cam = np.asarray(self.data.camera if camera is None else camera, T.camera_dtype).reshape(())
        check(lib().aur_render_adjoint(self.ctx.handle, self.handle, _ptr(cam), _ptr(p),
                                       _ptr(_dense(d_image)), _ptr(d_diffuse), _ptr(d_light),
                                       _ptr(d_emission) if d_emission is not None else None))
        return (d_diffuse, d_light, d_emission) if d_emission is not None else (d_diffuse, d_light)

    def close(self):
        if self.handle:
            self.nmh.handle = None
            lib().aur_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def generate_rays(ctx, W, H, sample, samples, camera, rays_dev, hits_dev):
    cam = np.asarray(camera, T.camera_dtype).reshape(())
    check(lib().aur_generate_rays(ctx.handle, W, H, sample, samples, _ptr(cam), _ptr(rays_dev), _ptr(hits_dev)))


def raytrace_monte_carlo(ctx, scene, params, sample, offset, num, rays_dev, hits_dev):
    p = np.asarray(params, T.params_dtype).reshape(())
    check(lib().aur_raytrace_monte_carlo(ctx.handle, scene.handle, _ptr(p), sample, offset, num, _ptr(rays_dev),
                                         _ptr(hits_dev)))


def draw_pixels(ctx, W, H, weight, hits_dev, accum_dev):
    check(lib().aur_draw_pixels(ctx.handle, W, H, weight, _ptr(hits_dev), _ptr(accum_dev)))


def filter_pixels(ctx, W, H, in_dev, out_dev, region=None):
    """aur_filter_pixels: region = (left, right, bottom, top) inclusive or None."""
    r = None if region is None else np.array(region, np.uint32)
    check(lib().aur_filter_pixels(ctx.handle, W, H, _ptr(r), _ptr(in_dev), _ptr(out_dev)))


def accum_save(ctx, path, accum_dev, samples_done, spp):
    """Checkpoint of an (H, W, 4) device accumulation buffer."""
    H, W = accum_dev.shape[:2]
    check(lib().aur_accum_save(ctx.handle, os.fsencode(path), W, H, samples_done, spp, _ptr(_dense(accum_dev))))


def accum_load(ctx, path, accum_dev):
    """Loads a checkpoint into an (H, W, 4) device buffer; returns (samples_done, spp)."""
    H, W = accum_dev.shape[:2]
    done, spp = ctypes.c_uint32(0), ctypes.c_uint32(0)
    check(lib().aur_accum_load(ctx.handle, os.fsencode(path), W, H, ctypes.byref(done), ctypes.byref(spp),
                               _ptr(accum_dev)))
    return done.value, spp.value


def clear_pixels(ctx, W, H, accum_dev):
    check(lib().aur_clear_pixels(ctx.handle, W, H, _ptr(accum_dev)))


def debug_nmh_layout(n, k):
    out = np.zeros(3, np.uint32)
    check(lib().aur_debug_nmh_layout(n, k, _ptr(out)))
    return tuple(int(x) for x in out)


def exported_symbols():
    """Names declared in include/aurora_gb300.h (parsed from the header)."""
    import re
    hdr = os.path.join(os.path.dirname(LIB), "..", "..", "include", "aurora_gb300.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"^\s*(?:aur_status|const char\*)\s+(aur_\w+)\s*\(", text, re.M)))


tuning_dtype = np.dtype([("paths_in_flight", "<u4"), ("samples_per_wave", "<u4"), ("block_size", "<u4"),
                         ("blocks_per_sm", "<u4"), ("max_iterations", "<u4")])


def make_tuning(paths_in_flight=0, samples_per_wave=0, block_size=0, blocks_per_sm=0, max_iterations=0):
    t = np.zeros((), tuning_dtype)
    t["paths_in_flight"], t["samples_per_wave"] = paths_in_flight, samples_per_wave
    t["block_size"], t["blocks_per_sm"] = block_size, blocks_per_sm
    t["max_iterations"] = max_iterations
    return t


def _batch_arrays(scenes, params, cameras=None):
    n = len(scenes)
    handles = (P * n)(*[s.handle for s in scenes])
    cams = np.stack([np.asarray(s.data.camera if cameras is None else cameras[i], T.camera_dtype).reshape(())
                     for i, s in enumerate(scenes)])
    prm = np.stack([np.asarray(p, T.params_dtype).reshape(()) for p in params])
    return handles, np.ascontiguousarray(cams), np.ascontiguousarray(prm)


class Batch:
    """aur_batch: a wavefront render of several scenes as one CUDA graph."""

    def __init__(self, ctx, scenes, params, tuning=None, cameras=None):
        self.ctx, self.scenes = ctx, list(scenes)
        self.handle = None
        self._h, self._cams, self._prm = _batch_arrays(self.scenes, params, cameras)
        t = None if tuning is None else np.asarray(tuning, tuning_dtype).reshape(())
        h = P()
        check(lib().aur_batch_create(ctx.handle, self._h, _ptr(self._cams), _ptr(self._prm), len(self.scenes),
                                     _ptr(t) if t is not None else None, ctypes.byref(h)))
        self.handle = h

    def render(self, accums=None):
        """Adds every scene's samples into its (H, W, 4) float32 device frame."""
        torch = _torch()
        if accums is None:
            accums = [torch.zeros((int(p["height"]), int(p["width"]), 4), dtype=torch.float32, device="cuda")
                      for p in self._prm]
        ptrs = (P * len(accums))(*[a.data_ptr() for a in accums])
        check(lib().aur_batch_render(self.ctx.handle, self.handle, ptrs))
        return accums

    def profile(self, accums):
        """Stepped render without the graph; returns per-stage milliseconds."""
        ptrs = (P * len(accums))(*[a.data_ptr() for a in accums])
        ms = np.zeros(7, np.float32)
        check(lib().aur_batch_profile(self.ctx.handle, self.handle, ptrs, _ptr(ms)))
        return dict(zip(["setup", "generate", "extend", "shade", "shadow", "combine", "accumulate"],
                        [float(x) for x in ms]))

    def status(self):
        it = U32()
        check(lib().aur_batch_status(self.ctx.handle, self.handle, ctypes.byref(it)))
        return it.value

    def counters(self):
        """(closest-hit rays, shadow rays, iterations) of the last render."""
        out = (ctypes.c_ulonglong * 3)()
        check(lib().aur_batch_counters(self.ctx.handle, self.handle, out))
        return int(out[0]), int(out[1]), int(out[2])

    def tuning(self):
        t = np.zeros((), tuning_dtype)
        check(lib().aur_batch_tuning(self.handle, _ptr(t)))
        return t

    def close(self):
        if self.handle:
            lib().aur_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tuning_key(gpu_name, sm_count, scenes, params):
    """Cache key of an autotuning result: the GPU and the batch's shape (per
    scene: triangles, lights, frame size, spp, depth, mode)."""
    shape = []
    for sc, p in zip(scenes, params):
        p = np.asarray(p, T.params_dtype).reshape(())
        shape.append([int(sc.data.count), int(sc.data.lights.shape[0]), int(p["width"]), int(p["height"]),
                      int(p["spp"]), int(p["max_depth"]), int(p["mode"])])
    return json.dumps({"gpu": gpu_name, "sms": int(sm_count), "scenes": shape}, sort_keys=True)


def tuning_cache_get(path, key):
    """The cached tuning record for `key` in the JSON file `path`, or None."""
    import json as _json
    if not path or not os.path.exists(path):
        return None
    entry = _json.load(open(path)).get(key)
    if entry is None:
        return None
    t = np.zeros((), tuning_dtype)
    for k in tuning_dtype.names:
        t[k] = entry["tuning"][k]
    return t, float(entry["ms"])


def tuning_cache_put(path, key, tuning, ms):
    import json as _json
    data = _json.load(open(path)) if os.path.exists(path) else {}
    data[key] = {"tuning": {k: int(tuning[k]) for k in tuning_dtype.names}, "ms": float(ms)}
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        _json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def autotune(ctx, scenes, params, cameras=None, cache=None):
    """Runs the C-side autotuner; returns (tuning record, milliseconds of a
    1-spp render). With `cache` (a JSON file path), results are kept per GPU
    and batch shape, and a hit skips the search."""
    scenes = list(scenes)
    key = None
    if cache:
        import torch
        key = tuning_key(torch.cuda.get_device_name(ctx.device), ctx.sm_count(), scenes, params)
        hit = tuning_cache_get(cache, key)
        if hit is not None:
            return hit
    h, cams, prm = _batch_arrays(scenes, params, cameras)
    t = np.zeros((), tuning_dtype)
    ms = ctypes.c_float()
    check(lib().aur_batch_autotune(ctx.handle, h, _ptr(cams), _ptr(prm), len(scenes), _ptr(t), ctypes.byref(ms)))
    if cache:
        tuning_cache_put(cache, key, t, ms.value)
    return t, ms.value


def transform(ctx, src_vertices, src_normals, transforms, dst_vertices, dst_normals):
    """aur_transform on device tensors (count*9 floats each); transforms: host records."""
    xf = np.ascontiguousarray(transforms, T.object_transform_dtype)
    check(lib().aur_transform(ctx.handle, _ptr(src_vertices), _ptr(src_normals), src_vertices.numel() // 9,
                              _ptr(xf), xf.shape[0], _ptr(dst_vertices), _ptr(dst_normals)))


def generate_tb(ctx, normals, tangents, bitangents):
    check(lib().aur_generate_tb(ctx.handle, _ptr(normals), normals.numel() // 9, _ptr(tangents), _ptr(bitangents)))
