"""Seeded synthetic scenes for the five workloads this library is measured on.

There is no public dataset for this path: every input is generated here from a
fixed seed with the shapes, sizes and value distributions of the workloads:
  cornell()            Cornell-style box: 5 wall quads (10 tris) + 2 blocks
                       (24 tris), one 1x1 area light, Lambert albedos.
  random_soup()        n triangles, centroids U[0,1]^3, edge lengths
                       LogNormal(mu=-4, sigma=0.5), directions uniform on S^2.
  microbench_rays()    half coherent pinhole rays (4096x4096 image, even rows)
                       and half random origin / uniform-sphere direction rays.
  sphere_scene()       N in [1,200] tessellated spheres (80-5000 tris each,
                       1k-500k tris total) + one area light.
  cornell_sphere()     Cornell box + 64x32 UV sphere (4096 tris), one shader
                       per triangle with RGB albedo U[0.2,0.8].
  terrain()            2048x2048-vertex fBm heightfield (2*2047^2 tris) with
                       16 area lights placed uniformly above it.
Triangles use the reference layout: vertices [x1 x2 x3 y1 y2 y3 z1 z2 z3],
normals [n1 n2 n3] per triangle, 1-based uint16 shader ids.
"""
import math

import numpy as np

from . import types as T


class SceneData:
    def __init__(self, name, vertices, normals, shader_ids, shaders, lights, camera):
        self.name = name
        self.vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 9)
        self.normals = np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
        self.shader_ids = np.ascontiguousarray(shader_ids, np.uint16).reshape(-1)
        self.shaders = np.ascontiguousarray(shaders, T.shader_dtype).reshape(-1)
        self.lights = np.ascontiguousarray(lights, T.light_dtype).reshape(-1)
        self.camera = np.asarray(camera, T.camera_dtype).reshape(())

    @property
    def count(self):
        return self.vertices.shape[0]


SCENE_MAGIC = b"AURSCN1\0"


def write_scene_file(sd, path):
    """Writes sd in the binary scene format read by the C++ host layer's
    loadSceneFile: magic "AURSCN1\\0", uint32 counts (triangles, shaders,
    lights, textures), the aur_camera record, 4 pad bytes, vertices and
    normals (36 B per triangle each), shader ids (uint16, padded to an even
    count), shaders (80 B each), lights (80 B each); with textures, then the
    texcoords (24 B per triangle) and per texture uint32 width, height and its
    RGBA8 texels; all little-endian."""
    n = sd.count
    ids = sd.shader_ids
    if n % 2:
        ids = np.concatenate([ids, np.zeros(1, np.uint16)])
    with open(path, "wb") as f:
        f.write(SCENE_MAGIC)
        textures = list(getattr(sd, "textures", None) or [])
        f.write(np.array([n, sd.shaders.shape[0], sd.lights.shape[0], len(textures)], "<u4").tobytes())
        f.write(sd.camera.reshape(1).tobytes())
        f.write(bytes(4))
        f.write(sd.vertices.astype("<f4").tobytes())
        f.write(sd.normals.astype("<f4").tobytes())
        f.write(ids.astype("<u2").tobytes())
        f.write(sd.shaders.tobytes())
        f.write(sd.lights.tobytes())
        if textures:
            f.write(np.ascontiguousarray(sd.texcoords, "<f4").reshape(n, 6).tobytes())
            for t in textures:
                t = np.ascontiguousarray(t, np.uint8)
                f.write(np.array([t.shape[1], t.shape[0]], "<u4").tobytes())
                f.write(t.tobytes())


def read_pfm(path):
    """Reads an RGB PFM (bottom row first) into an (H, W, 3) float32 array
    with row 0 at the bottom, the layout of the accumulation buffers."""
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = (int(x) for x in f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), "<f4" if scale < 0 else ">f4")
    return data.reshape(h, w, 3).astype(np.float32)


# ----------------------------------------------------------------- helpers

def _f(x):
    return np.float32(x)


def make_camera(position, direction, tanfov_x, tanfov_y, aspect=1.0):
    """Camera::Camera (util/camera.h:15-28) in float32, tanfov given directly."""
    d = [_f(v) for v in direction]
    inv = _f(1.0) / np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    f = [d[0] * inv, d[1] * inv, d[2] * inv]
    up0 = [_f(0.0), _f(1.0), _f(0.0)]

    def cross(a, b):
        return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]

    right = cross(f, up0)
    up = cross(right, f)
    c = np.zeros((), T.camera_dtype)
    c["position"], c["forward"], c["right"], c["up"] = position, f, right, up
    c["tanfov_x"], c["tanfov_y"], c["aspect"] = tanfov_x, tanfov_y, aspect
    return c


def tris_to_soa(p1, p2, p3):
    """(n,3) corner arrays -> (n,9) reference layout [x1 x2 x3 y1 y2 y3 z1 z2 z3]."""
    v = np.empty((p1.shape[0], 9), np.float32)
    for a in range(3):
        v[:, 3 * a + 0] = p1[:, a]
        v[:, 3 * a + 1] = p2[:, a]
        v[:, 3 * a + 2] = p3[:, a]
    return v


def normals_to_aos(n1, n2, n3):
    return np.concatenate([n1, n2, n3], axis=1).astype(np.float32)


def face_normals(p1, p2, p3):
    n = np.cross(p2 - p1, p3 - p1)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return (n / ln).astype(np.float32)


def _orient(p1, p2, p3, want):
    """Swap p2/p3 where the winding normal (p2-p1)x(p3-p1) opposes `want`,
    so the front face (the one Moller-Trumbore with culling hits) faces it."""
    n = np.cross(p2 - p1, p3 - p1)
    flip = np.einsum("ij,ij->i", n, want) < 0
    q2 = np.where(flip[:, None], p3, p2)
    q3 = np.where(flip[:, None], p2, p3)
    return p1, q2, q3


def _quad(c0, c1, c2, c3, normal):
    p = np.array([c0, c0], np.float64), np.array([c1, c2], np.float64), np.array([c2, c3], np.float64)
    w = np.array([normal, normal], np.float64)
    return _orient(p[0], p[1], p[2], w)


def _box(center, size, yaw_deg):
    """Axis-aligned box rotated about +y, outward-facing triangles (12)."""
    cx, cy, cz = center
    sx, sy, sz = (s / 2.0 for s in size)
    a = math.radians(yaw_deg)
    rot = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    # corner index = 4*[x+] + 2*[y+] + [z+]; each face lists its corners cyclically
    c = np.array([[x, y, z] for x in (-sx, sx) for y in (-sy, sy) for z in (-sz, sz)]) @ rot.T + [cx, cy, cz]
    faces = [(0, 1, 3, 2, (-1, 0, 0)), (4, 5, 7, 6, (1, 0, 0)), (0, 1, 5, 4, (0, -1, 0)),
             (2, 3, 7, 6, (0, 1, 0)), (0, 2, 6, 4, (0, 0, -1)), (1, 3, 7, 5, (0, 0, 1))]
    out = []
    for i0, i1, i2, i3, n in faces:
        out.append(_quad(c[i0], c[i1], c[i2], c[i3], rot @ np.array(n, np.float64)))
    p1 = np.concatenate([o[0] for o in out]); p2 = np.concatenate([o[1] for o in out])
    p3 = np.concatenate([o[2] for o in out])
    return p1, p2, p3


def _uv_sphere(center, radius, slices, stacks):
    """UV sphere, 2*slices*stacks triangles (pole triangles are degenerate)."""
    c = np.asarray(center, np.float64)
    th = np.linspace(0.0, math.pi, stacks + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, slices + 1)
    P = np.stack([np.sin(th)[:, None] * np.cos(ph)[None, :], np.repeat(np.cos(th)[:, None], slices + 1, 1),
                  np.sin(th)[:, None] * np.sin(ph)[None, :]], -1)
    j, i = np.meshgrid(np.arange(stacks), np.arange(slices), indexing="ij")
    j, i = j.ravel(), i.ravel()
    a, b = P[j, i], P[j, i + 1]
    cc, d = P[j + 1, i + 1], P[j + 1, i]
    n1s = np.concatenate([a, a]); n2s = np.concatenate([b, cc]); n3s = np.concatenate([cc, d])
    p1, p2, p3 = c + radius * n1s, c + radius * n2s, c + radius * n3s
    want = (p1 + p2 + p3) / 3.0 - c
    flip = np.einsum("ij,ij->i", np.cross(p2 - p1, p3 - p1), want) < 0
    p2f = np.where(flip[:, None], p3, p2); p3f = np.where(flip[:, None], p2, p3)
    n2f = np.where(flip[:, None], n3s, n2s); n3f = np.where(flip[:, None], n2s, n3s)
    return p1, p2f, p3f, n1s, n2f, n3f


# -------------------------------------------------------------- workloads

WHITE = (0.73, 0.73, 0.73)
RED = (0.63, 0.065, 0.05)
GREEN = (0.14, 0.45, 0.09)


def _cornell_parts():
    walls = [
        ((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), 1),     # floor, white
        ((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1), (0, -1, 0), 1),    # ceiling, white
        ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), 1),     # back, white
        ((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (1, 0, 0), 2),     # left, red
        ((1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1), (-1, 0, 0), 3),    # right, green
    ]
    P1, P2, P3, S = [], [], [], []
    for c0, c1, c2, c3, n, sid in walls:
        p1, p2, p3 = _quad(c0, c1, c2, c3, n)
        P1.append(p1); P2.append(p2); P3.append(p3); S += [sid, sid]
    for center, size, yaw in (((0.66, 0.15, 0.63), (0.3, 0.3, 0.3), 18.0),
                              ((0.33, 0.3, 0.35), (0.3, 0.6, 0.3), -20.0)):
        p1, p2, p3 = _box(center, size, yaw)
        P1.append(p1); P2.append(p2); P3.append(p3); S += [1] * p1.shape[0]
    p1, p2, p3 = np.concatenate(P1), np.concatenate(P2), np.concatenate(P3)
    return p1, p2, p3, np.array(S, np.uint16)


def cornell_light(intensity=3.0, samples=1):
    """The 1x1 area light of the Cornell workload: a unit quad at y=0.999
    spanning the box's ceiling, emitting downwards."""
    return T.area_light((0.0, 0.999, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0), (0.0, -1.0, 0.0),
                        intensity=intensity, samples=samples)


def cornell_camera():
    return make_camera((0.5, 0.5, 2.3), (0.0, 0.0, -1.0), 0.8, 0.8)


def cornell():
    p1, p2, p3, sids = _cornell_parts()
    fn = face_normals(p1, p2, p3)
    shaders = np.stack([T.lambert(WHITE), T.lambert(RED), T.lambert(GREEN)])
    return SceneData("cornell", tris_to_soa(p1, p2, p3), normals_to_aos(fn, fn, fn), sids, shaders,
                     np.stack([cornell_light()]), cornell_camera())


def cornell_emissive(area_light=False):
    """The Cornell box lit by emissive geometry instead of an area light: a
    0.3 x 0.3 quad under the ceiling (emission colour 12, weight 1), a small
    glowing block on the floor (orange, weight 0.5) and, last, one emissive
    triangle on the back wall, which makes the count odd so that the even
    padding duplicates an emitter. `area_light` adds the Cornell area light."""
    p1, p2, p3, sids = _cornell_parts()
    P1, P2, P3, S = [p1], [p2], [p3], [sids]
    q = _quad((0.35, 0.998, 0.35), (0.65, 0.998, 0.35), (0.65, 0.998, 0.65), (0.35, 0.998, 0.65), (0, -1, 0))
    P1.append(q[0]); P2.append(q[1]); P3.append(q[2]); S.append(np.full(2, 4, np.uint16))
    b = _box((0.82, 0.04, 0.2), (0.1, 0.08, 0.1), 30.0)
    P1.append(b[0]); P2.append(b[1]); P3.append(b[2]); S.append(np.full(12, 5, np.uint16))
    t = _orient(np.array([[0.1, 0.7, 0.001]]), np.array([[0.25, 0.7, 0.001]]), np.array([[0.17, 0.85, 0.001]]),
                np.array([[0.0, 0.0, 1.0]]))
    P1.append(t[0]); P2.append(t[1]); P3.append(t[2]); S.append(np.full(1, 6, np.uint16))
    p1, p2, p3 = np.concatenate(P1), np.concatenate(P2), np.concatenate(P3)
    fn = face_normals(p1, p2, p3)
    lamp = T.lambert(WHITE, emission=(12.0, 12.0, 12.0)); lamp["emission"] = 1.0
    glow = T.lambert((0.9, 0.5, 0.2), emission=(3.0, 1.6, 0.6)); glow["emission"] = 0.5
    spot = T.lambert(WHITE, emission=(2.0, 4.0, 6.0)); spot["emission"] = 2.0
    shaders = np.stack([T.lambert(WHITE), T.lambert(RED), T.lambert(GREEN), lamp, glow, spot])
    lights = np.stack([cornell_light(intensity=1.5)]) if area_light else np.zeros(0, T.light_dtype)
    return SceneData("cornell_emissive", tris_to_soa(p1, p2, p3), normals_to_aos(fn, fn, fn), np.concatenate(S),
                     shaders, lights, cornell_camera())


def planar_texcoords(vertices, scale=1.0):
    """Per-triangle texcoords (n, 6) = (u1 v1 u2 v2 u3 v3): each triangle's
    corners projected onto the two axes orthogonal to its dominant normal
    axis, times `scale` (values above 1 exercise the wrapping)."""
    V = np.asarray(vertices, np.float32).reshape(-1, 9)
    P = np.stack([V[:, 0::3], V[:, 1::3], V[:, 2::3]], -1)         # (n, corner, xyz)
    n = np.abs(np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]))
    dom = np.argmax(n, axis=1)
    a1 = np.where(dom == 0, 2, 0)
    a2 = np.where(dom == 1, 2, 1)
    idx = np.arange(V.shape[0])
    tc = np.empty((V.shape[0], 6), np.float32)
    for k in range(3):
        tc[:, 2 * k] = P[idx, k, a1] * scale
        tc[:, 2 * k + 1] = P[idx, k, a2] * scale
    return tc


def cornell_textured(seed=0):
    """The Cornell workload with textures: the floor and back wall use
    shaders with textures 1 and 2 (random RGBA8 images of odd size, mapped
    with wrapping), the short box a shader naming texture 40 (beyond the 32
    units the reference binds: white)."""
    rng = np.random.default_rng(seed)
    sd = cornell()
    tex = [rng.integers(0, 256, size=(9, 13, 4), dtype=np.uint8),
           rng.integers(0, 256, size=(32, 17, 4), dtype=np.uint8)]
    sh = np.concatenate([sd.shaders, np.stack([T.lambert((1.0, 1.0, 1.0), diffuse=0.8),
                                               T.lambert((1.0, 1.0, 1.0), diffuse=0.7),
                                               T.lambert((1.0, 1.0, 1.0), diffuse=0.6)])])
    sh["texture"][3], sh["texture"][4], sh["texture"][5] = 1, 2, 40
    sids = sd.shader_ids.copy()
    V = sd.vertices
    ys = V[:, 3:6]
    zs = V[:, 6:9]
    floor = np.all(ys == 0.0, axis=1)
    back = np.all(zs == 0.0, axis=1)
    sids[floor] = 4
    sids[back] = 5
    sids[10:22] = 6                                                    # the short box
    out = SceneData("cornell_textured", V, sd.normals, sids, sh, sd.lights, sd.camera)
    out.texcoords = planar_texcoords(V, scale=2.5)
    out.textures = tex
    return out


def cornell_sphere(seed=0, slices=64, stacks=32):
    """Cornell box + UV sphere; one shader per triangle, albedo U[0.2, 0.8]."""
    rng = np.random.default_rng(seed)
    p1, p2, p3, _ = _cornell_parts()
    fn = face_normals(p1, p2, p3)
    q1, q2, q3, m1, m2, m3 = _uv_sphere((0.5, 0.35, 0.7), 0.18, slices, stacks)
    V = np.concatenate([tris_to_soa(p1, p2, p3), tris_to_soa(q1, q2, q3)])
    N = np.concatenate([normals_to_aos(fn, fn, fn), normals_to_aos(m1, m2, m3)])
    n = V.shape[0]
    albedo = rng.uniform(0.2, 0.8, size=(n, 3)).astype(np.float32)
    shaders = np.zeros(n, T.shader_dtype)
    shaders["type"] = T.SHADER_LAMBERT
    shaders["diffuse_color"] = albedo
    shaders["diffuse"] = 1.0
    shaders["refractive_index"] = 1.0
    sids = np.arange(1, n + 1, dtype=np.uint16)
    return SceneData("cornell_sphere", V, N, sids, shaders, np.stack([cornell_light()]), cornell_camera())


def random_soup(n=1_000_000, seed=0):
    """Triangle soup: centroid U[0,1]^3, two edges L_i*d_i with
    L_i ~ LogNormal(-4, 0.5) and d_i uniform on the unit sphere."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    L = rng.lognormal(mean=-4.0, sigma=0.5, size=(n, 2))
    d = rng.normal(size=(n, 2, 3))
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    e1 = L[:, 0:1] * d[:, 0]
    e2 = L[:, 1:2] * d[:, 1]
    p1 = c - (e1 + e2) / 3.0
    p2, p3 = p1 + e1, p1 + e2
    return tris_to_soa(p1, p2, p3)


def microbench_rays(n=1 << 24, seed=1, image=4096, tmax=1.0e6):
    """First half: pinhole at (0.5, 0.5, -1) looking +z through an image x
    image grid over [0,1]^2 at z=0, rows with even y, row-major. Second half:
    origin U[0,1]^3, direction uniform on the unit sphere."""
    half = n // 2
    r = np.zeros(n, T.ray_dtype)
    k = np.arange(half, dtype=np.int64)
    x = k % image
    y = 2 * (k // image) % image
    px = ((x + 0.5) / image - 0.5).astype(np.float32)
    py = ((y + 0.5) / image - 0.5).astype(np.float32)
    inv = (1.0 / np.sqrt(px.astype(np.float64) ** 2 + py.astype(np.float64) ** 2 + 1.0)).astype(np.float32)
    r["ox"][:half], r["oy"][:half], r["oz"][:half] = 0.5, 0.5, -1.0
    r["dx"][:half], r["dy"][:half], r["dz"][:half] = px * inv, py * inv, inv
    rng = np.random.default_rng(seed)
    m = n - half
    o = rng.random((m, 3)).astype(np.float32)
    d = rng.normal(size=(m, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    r["ox"][half:], r["oy"][half:], r["oz"][half:] = o[:, 0], o[:, 1], o[:, 2]
    r["dx"][half:], r["dy"][half:], r["dz"][half:] = d[:, 0], d[:, 1], d[:, 2]
    r["tmax"] = tmax
    return r


def sphere_scene(seed, min_tris=1000, max_tris=500_000):
    """N ~ U{1..200} spheres, radius U[0.05, 0.3], centre U[0,1]^3, each a UV
    sphere with a log-uniform triangle count in [80, 5000]; the total is kept
    within [min_tris, max_tris] by dropping or adding spheres. One area light
    above the unit cube, camera looking at the cube from +z."""
    rng = np.random.default_rng(seed)
    ns = int(rng.integers(1, 201))
    parts, total = [], 0
    i = 0
    while i < ns or total < min_tris:
        r = rng.uniform(0.05, 0.3)
        c = rng.random(3)
        tri = math.exp(rng.uniform(math.log(80), math.log(5000)))
        stacks = max(2, int(round(math.sqrt(tri / 4.0))))
        slices = max(3, int(round(tri / (2.0 * stacks))))
        if total + 2 * slices * stacks > max_tris:
            break
        parts.append(_uv_sphere(c, r, slices, stacks))
        total += 2 * slices * stacks
        i += 1
    q1 = np.concatenate([p[0] for p in parts]); q2 = np.concatenate([p[1] for p in parts])
    q3 = np.concatenate([p[2] for p in parts]); m1 = np.concatenate([p[3] for p in parts])
    m2 = np.concatenate([p[4] for p in parts]); m3 = np.concatenate([p[5] for p in parts])
    n = q1.shape[0]
    ncol = 8
    shaders = np.stack([T.lambert(tuple(rng.uniform(0.2, 0.9, 3))) for _ in range(ncol)])
    sids = rng.integers(1, ncol + 1, size=n).astype(np.uint16)
    light = T.area_light((0.25, 1.6, 0.25), (0.5, 0.0, 0.0), (0.0, 0.0, 0.5), (0.0, -1.0, 0.0),
                         intensity=4.0, samples=1)
    cam = make_camera((0.5, 0.5, 2.4), (0.0, 0.0, -1.0), 0.75, 0.75)
    return SceneData("spheres_%d" % seed, tris_to_soa(q1, q2, q3), normals_to_aos(m1, m2, m3), sids, shaders,
                     np.stack([light]), cam)


def _fbm(res, seed, octaves=8, lacunarity=2.0, gain=0.5):
    """Fractional Brownian motion of seeded gradient (Perlin-style) noise on
    a res x res grid over [0,1]^2."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 1.0, res, dtype=np.float64)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    h = np.zeros((res, res))
    freq, amp = 4.0, 1.0
    for _ in range(octaves):
        g = int(math.ceil(freq)) + 2
        ang = rng.uniform(0.0, 2.0 * math.pi, size=(g, g))
        gx, gy = np.cos(ang), np.sin(ang)
        fx, fy = X * freq, Y * freq
        ix, iy = np.floor(fx).astype(np.int64), np.floor(fy).astype(np.int64)
        tx, ty = fx - ix, fy - iy

        def dotg(ox, oy):
            return gx[iy + oy, ix + ox] * (tx - ox) + gy[iy + oy, ix + ox] * (ty - oy)

        sx = tx * tx * tx * (tx * (tx * 6 - 15) + 10)
        sy = ty * ty * ty * (ty * (ty * 6 - 15) + 10)
        n0 = dotg(0, 0) + sx * (dotg(1, 0) - dotg(0, 0))
        n1 = dotg(0, 1) + sx * (dotg(1, 1) - dotg(0, 1))
        h += amp * (n0 + sy * (n1 - n0))
        freq *= lacunarity
        amp *= gain
    return h


def terrain(res=2048, seed=0, n_lights=16, height=0.25):
    """res x res vertex heightfield over [0,1]^2 (2*(res-1)^2 tris), fBm
    height, smooth vertex normals, 16 area lights placed U above it."""
    rng = np.random.default_rng(seed + 7)
    h = (_fbm(res, seed) * height).astype(np.float32)
    xs = np.linspace(0.0, 1.0, res, dtype=np.float32)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    P = np.stack([X, h, Z], -1)
    dhx = np.gradient(h, xs, axis=1)
    dhz = np.gradient(h, xs, axis=0)
    Nv = np.stack([-dhx, np.ones_like(h), -dhz], -1)
    Nv /= np.linalg.norm(Nv, axis=-1, keepdims=True)
    j, i = np.meshgrid(np.arange(res - 1), np.arange(res - 1), indexing="ij")
    j, i = j.ravel(), i.ravel()
    a, b, c, d = (j, i), (j, i + 1), (j + 1, i + 1), (j + 1, i)
    p1 = np.concatenate([P[a], P[a]]); p2 = np.concatenate([P[c], P[b]]); p3 = np.concatenate([P[b], P[c]])
    n1 = np.concatenate([Nv[a], Nv[a]]); n2 = np.concatenate([Nv[c], Nv[b]]); n3 = np.concatenate([Nv[b], Nv[c]])
    del P, Nv
    up = np.zeros_like(p1); up[:, 1] = 1.0
    flip = np.einsum("ij,ij->i", np.cross(p2 - p1, p3 - p1), up) < 0
    p2, p3 = np.where(flip[:, None], p3, p2), np.where(flip[:, None], p2, p3)
    n2, n3 = np.where(flip[:, None], n3, n2), np.where(flip[:, None], n2, n3)
    lights = []
    for _ in range(n_lights):
        cx, cz = rng.uniform(0.0, 1.0, 2)
        s = rng.uniform(0.03, 0.1)
        y = rng.uniform(0.6, 1.0)
        lights.append(T.area_light((cx - s / 2, y, cz - s / 2), (s, 0.0, 0.0), (0.0, 0.0, s), (0.0, -1.0, 0.0),
                                   color=tuple(rng.uniform(0.6, 1.0, 3)), intensity=1.5, samples=1))
    # looking down across the terrain from above its near edge: the terrain
    # fills the frame (98 % of the camera rays hit it)
    cam = make_camera((0.5, 0.9, 1.45), (0.0, -0.8, -1.0), 0.6, 0.6 * 1080.0 / 1920.0, 1920.0 / 1080.0)
    return SceneData("terrain", tris_to_soa(p1, p2, p3), normals_to_aos(n1, n2, n3),
                     np.ones(p1.shape[0], np.uint16), np.stack([T.lambert((0.55, 0.5, 0.45))]),
                     np.stack(lights), cam)
