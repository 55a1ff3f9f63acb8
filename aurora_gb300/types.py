"""numpy dtypes mirroring the POD structs of include/aurora_gb300.h.

The layouts are part of the C ABI: a record of one of these dtypes is
byte-identical to the C struct of the same name.
"""
import numpy as np

F3 = ("<f4", (3,))

ray_dtype = np.dtype([("ox", "<f4"), ("oy", "<f4"), ("oz", "<f4"), ("tmax", "<f4"),
                      ("dx", "<f4"), ("dy", "<f4"), ("dz", "<f4"), ("pad", "<f4")])
hit_dtype = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4")])

shader_dtype = np.dtype([("type", "<i4"), ("diffuse_color",) + F3, ("emission_color",) + F3,
                         ("specular_color",) + F3, ("reflection_color",) + F3,
                         ("diffuse", "<f4"), ("emission", "<f4"), ("exponent", "<f4"),
                         ("reflectivity", "<f4"), ("translucence", "<f4"), ("refractive_index", "<f4"),
                         ("texture", "<u4")])

light_dtype = np.dtype([("type", "<i4"), ("intensity", "<f4"), ("ambient", "<f4"), ("area", "<f4"),
                        ("samples", "<i4"), ("position",) + F3, ("color",) + F3, ("direction",) + F3,
                        ("e1",) + F3, ("e2",) + F3])

camera_dtype = np.dtype([("position",) + F3, ("forward",) + F3, ("right",) + F3, ("up",) + F3,
                         ("tanfov_x", "<f4"), ("tanfov_y", "<f4"), ("aspect", "<f4")])

params_dtype = np.dtype([("width", "<u4"), ("height", "<u4"), ("spp", "<u4"), ("max_depth", "<u4"),
                         ("seed", "<u4"), ("mode", "<u4"), ("sample_begin", "<u4"), ("sample_end", "<u4"),
                         ("scene_id", "<u4")])

path_ray_dtype = np.dtype([("pos",) + F3, ("dir",) + F3, ("t", "<f4"), ("weight", "<f4"), ("eta", "<f4")])
hitpoint_dtype = np.dtype([("color",) + F3, ("position",) + F3, ("wo",) + F3, ("u", "<f4"), ("v", "<f4"),
                           ("triangle_id", "<i4")])

emitter_dtype = np.dtype([("area", "<f4"), ("pdf", "<f4"), ("cdf", "<f4"), ("power",) + F3, ("triangle_id", "<u4")])

object_transform_dtype = np.dtype([("offset", "<u4"), ("size", "<u4"), ("world_matrix", "<f4", (4, 4)),
                                   ("normal_matrix", "<f4", (4, 4))])

assert ray_dtype.itemsize == 32 and hit_dtype.itemsize == 16
assert object_transform_dtype.itemsize == 136 and emitter_dtype.itemsize == 28
assert shader_dtype.itemsize == 80 and light_dtype.itemsize == 80
assert camera_dtype.itemsize == 60 and params_dtype.itemsize == 36
assert path_ray_dtype.itemsize == 36 and hitpoint_dtype.itemsize == 48

import ctypes  # noqa: E402


class texture_ctype(ctypes.Structure):
    """aur_texture: width, height, host RGBA8 pointer."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("rgba", ctypes.c_void_p)]


NO_HIT = 0xFFFFFFFF
MODE_REFERENCE, MODE_PATH, MODE_PATH_MIS = 0, 1, 2
SHADER_LAMBERT, SHADER_PHONG = 0, 1
LIGHT_AMBIENT, LIGHT_POINT, LIGHT_DIRECTIONAL, LIGHT_AREA = 0, 1, 2, 3


def render_params(width, height, spp, max_depth, seed=0, mode=MODE_PATH, sample_begin=0, sample_end=0,
                  scene_id=0):
    p = np.zeros((), params_dtype)
    p["width"], p["height"], p["spp"], p["max_depth"] = width, height, spp, max_depth
    p["seed"], p["mode"], p["sample_begin"], p["sample_end"] = seed, mode, sample_begin, sample_end
    p["scene_id"] = scene_id
    return p


def lambert(color, diffuse=1.0, emission=(0.0, 0.0, 0.0)):
    s = np.zeros((), shader_dtype)
    s["type"] = SHADER_LAMBERT
    s["diffuse_color"] = color
    s["emission_color"] = emission
    s["diffuse"] = diffuse
    s["refractive_index"] = 1.0
    return s


def area_light(corner, e1, e2, direction, color=(1.0, 1.0, 1.0), intensity=1.0, samples=1):
    lt = np.zeros((), light_dtype)
    lt["type"] = LIGHT_AREA
    lt["position"], lt["e1"], lt["e2"], lt["direction"] = corner, e1, e2, direction
    lt["color"], lt["intensity"], lt["samples"] = color, intensity, samples
    lt["area"] = np.float32(np.linalg.norm(np.asarray(e1, np.float32)) * np.linalg.norm(np.asarray(e2, np.float32)))
    return lt
