// aur_integrate.cuh — the Monte-Carlo integrator of one camera sample, shared
// by the plain renderer and the renderer-helper entry points.
//
// raytrace() + cudaRaytraceKernel (kernels/monteCarloRaytracer.cu:23-113):
// a stack of rays per sample; at every hit Li = emission + ambient + direct
// lighting from every light (radiance.cuh:13-80, light.cuh:228-293); specular
// reflection / refraction rays are pushed when the shader has them; the
// colour is accumulated as Li * ray weight. AUR_MODE_PATH adds the diffuse
// bounce of BSDF::samplef (bsdf.cuh:222-236) with an RGB throughput.
#pragma once

#include "aur_math.cuh"
#include "aur_traverse.cuh"

namespace aur {

struct SceneView {
    const float4* recs;
    uint32_t nodes;
    const uint32_t* perm;
    const float* normals;      // NMH order, 9 floats per triangle
    const uint16_t* sids;      // NMH order, 1-based
    const aur_shader* shaders;
    const aur_light* lights;
    uint32_t num_lights;
    const float* texcoords;    // NMH order, 6 floats per triangle (null without textures)
    const uchar4* texels;      // RGBA8 texels of all textures
    const uint4* tex_info;     // per texture: first texel, width, height
    // AUR_MODE_PATH_MIS only:
    const float* verts;        // NMH order, 9 floats per triangle (x1 x2 x3 y1 y2 y3 z1 z2 z3)
    const uint32_t* mis_tri;   // light-selection table: NMH positions of the sampled emitters
    const float* mis_cdf;      //   and their CDF (inclusive, normalised)
    const float* mis_pa;       // per NMH triangle: selection probability / area (0 if not in the table)
    uint32_t mis_count;
};

SceneView scene_view(const aur_scene* sc);

// Texture units of the reference (texunit.cuh:11-18): normalised
// coordinates, wrap addressing, linear filtering, RGBA8 read as byte / 255.
// Filtered here in software, by the formula the CUDA C++ Programming Guide
// gives for tex2D linear filtering (appendix "Texture Fetching"): wrap
// replaces u by frac(u); xB = frac(u) * width - 0.5; texels floor(xB) and
// floor(xB) + 1 (wrapped); weight alpha = frac(xB) rounded to 8 fractional
// bits (to nearest, as a probe of the hardware shows); result
// (1-a)(1-b) T00 + a(1-b) T10 + (1-a) b T01 + a b T11 in float. The hardware
// blends at a precision the guide leaves open (within 1.3e-3 of this on
// GB300); the software form is exact and the same on every GPU and the CPU.
__device__ __forceinline__ float tex_weight(float f) { return floorf(f * 256.0f + 0.5f) * (1.0f / 256.0f); }

__device__ __forceinline__ f3 texel(const uchar4* __restrict__ t, uint32_t w, uint32_t i, uint32_t j) {
    const uchar4 q = __ldg(t + (size_t)j * w + i);
    return mk3((float)q.x / 255.0f, (float)q.y / 255.0f, (float)q.z / 255.0f);
}

// texfetch (kernels/lib/texunit.cuh:54-94); units past the 32 the reference
// binds return white.
__device__ __forceinline__ f3 texfetch(const SceneView& sc, uint32_t id, float u, float v) {
    if (id >= (uint32_t)AUR_MAX_TEXTURES) return mk3(1.0f, 1.0f, 1.0f);
    const uint4 ti = __ldg(sc.tex_info + id);
    const uchar4* t = sc.texels + ti.x;
    const uint32_t W = ti.y, H = ti.z;
    if (W == 0 || H == 0) return mk3(1.0f, 1.0f, 1.0f);   // no such texture (render entry points reject this)
    float xu = u - floorf(u), xv = v - floorf(v);
    if (!(xu >= 0.0f && xu <= 1.0f)) xu = 0.0f;   // NaN / inf coordinates
    if (!(xv >= 0.0f && xv <= 1.0f)) xv = 0.0f;
    const float xb = xu * (float)W - 0.5f, yb = xv * (float)H - 0.5f;
    const float fi = floorf(xb), fj = floorf(yb);
    const float a = tex_weight(xb - fi), b = tex_weight(yb - fj);
    const uint32_t i0 = fi < 0.0f ? W - 1 : min((uint32_t)fi, W - 1);
    const uint32_t j0 = fj < 0.0f ? H - 1 : min((uint32_t)fj, H - 1);
    const uint32_t i1 = i0 + 1 == W ? 0 : i0 + 1, j1 = j0 + 1 == H ? 0 : j0 + 1;
    const f3 t00 = texel(t, W, i0, j0), t10 = texel(t, W, i1, j0), t01 = texel(t, W, i0, j1),
             t11 = texel(t, W, i1, j1);
    return t00 * ((1.0f - a) * (1.0f - b)) + t10 * (a * (1.0f - b)) + t01 * ((1.0f - a) * b) + t11 * (a * b);
}

struct PathRay {
    f3 pos, dir;
    float weight, eta;
    f3 thr;
    float pdf;   // AUR_MODE_PATH_MIS: solid-angle density of the diffuse bounce that made the ray, 0 otherwise
};

struct Bsdf { f3 N, S, T, color1; };

// cudaGenerateTBKernel (kernels/utility.cu:136-167) evaluated per vertex at
// shading time: tangent = n x up (n x forward if that is shorter than
// Epsilon), bitangent = n x tangent.
__device__ __forceinline__ void vertex_tb(const f3& n, f3& t, f3& b) {
    t = cross(n, mk3(0.0f, 1.0f, 0.0f));
    if (length(t) < kEpsilon) t = cross(n, mk3(0.0f, 0.0f, 1.0f));
    b = cross(n, t);
}

// getBasisVectors + Shader::getBSDF (common.cuh:314-327, shader.cuh:243-262)
// Shader::getBSDF (kernels/lib/shader.cuh) with the texture branch of
// raytrace() (monteCarloRaytracer.cu:37-40): a textured shader's colour is
// texfetch(texture - 1, uv) * diffuse, uv from getTexCoord (common.cuh:45-51).
__device__ __forceinline__ Bsdf get_bsdf(const SceneView& sc, const aur_shader* sh, uint32_t tri, float u, float v) {
    const float* nv = sc.normals + (size_t)tri * 9;
    const f3 n1 = mk3(nv[0], nv[1], nv[2]), n2 = mk3(nv[3], nv[4], nv[5]), n3 = mk3(nv[6], nv[7], nv[8]);
    f3 t1, t2, t3, b1, b2, b3;
    vertex_tb(n1, t1, b1);
    vertex_tb(n2, t2, b2);
    vertex_tb(n3, t3, b3);
    Bsdf b;
    b.N = normalize(bclerp(n1, n2, n3, u, v));
    b.S = normalize(bclerp(t1, t2, t3, u, v));
    b.T = normalize(bclerp(b1, b2, b3, u, v));
    if (sh->texture > 0) {
        f3 c = mk3(1.0f, 1.0f, 1.0f);   // units past the 32 bound fetch white
        if (sh->texture <= (uint32_t)AUR_MAX_TEXTURES) {
            const float* tc = sc.texcoords + (size_t)tri * 6;
            const float w = 1.0f - u - v;
            const float tu = w * tc[0] + u * tc[2] + v * tc[4];
            const float tv = w * tc[1] + u * tc[3] + v * tc[5];
            c = texfetch(sc, sh->texture - 1, tu, tv);
        }
        b.color1 = c * sh->diffuse;
    } else {
        b.color1 = from(sh->diffuse_color) * sh->diffuse;
    }
    return b;
}

__device__ __forceinline__ f3 bsdf_f(const Bsdf& b) { return b.color1 * kInvPi; }  // bsdf.cuh:202-210

// Light::sampleL (light.cuh:228-259). For area lights u1, u2 come from the
// counter RNG at `slot`.
__device__ __forceinline__ f3 sample_light(const aur_light& L, const f3& from_pos, uint32_t seed, uint32_t scene,
                                           uint32_t pixel, uint32_t sample, uint32_t ray, uint32_t slot, f3& dir,
                                           float& t, float& pdf) {
    const f3 color = from(L.color);
    if (L.type == AUR_LIGHT_AMBIENT || L.type == AUR_LIGHT_POINT) {
        dir = from(L.position) - from_pos;
        t = length(dir);
        dir = dir / t;
        pdf = 1.0f;
        if (L.type == AUR_LIGHT_AMBIENT) return (color * L.intensity) * (1.0f - L.ambient);
        return (color * L.intensity) / (t * t);
    }
    if (L.type == AUR_LIGHT_DIRECTIONAL) {
        dir = -from(L.direction);
        t = kInfinity;
        pdf = 1.0f;
        return color * L.intensity;
    }
    float u1, u2;
    draw2(seed, scene, pixel, sample, ray, slot, u1, u2);
    const f3 P = from(L.position) + ((from(L.e1) * u1) + (from(L.e2) * u2));
    dir = P - from_pos;
    t = length(dir);
    dir = dir / t;
    pdf = 1.0f / fabsf(dot(from(L.direction), -dir));
    return (color * L.intensity) * fmaxf(0.0f, dot(from(L.direction), -dir));
}

struct SampleResult {
    f3 color;
    bool any_hit;
    uint32_t last_tri;   // NMH position of the last hit
    float last_u, last_v;
    f3 last_pos, last_wo;
};

// ------------------------------------------------------------------- MIS
// AUR_MODE_PATH_MIS: path mode with physically based direct lighting and
// multiple importance sampling (Veach & Guibas, SIGGRAPH 1995), the half of
// estimateDirectRadiance the reference compiles out (radiance.cuh:55-71).
// * Area lights keep the reference's emission model, radiance
//   Light::L(w) = colour * intensity * max(0, direction . w) (light.cuh:18-22),
//   and are estimated by both strategies of estimateDirectRadiance: a point
//   sampled on the quad (density t^2 / (cos_l * area) in solid angle, where
//   the reference's Light::pdf returns 1 / |cos_l|, light.cuh:78-89) and a
//   direction sampled from the BSDF (BSDF::samplef, bsdf.cuh:53-67) traced to
//   the quad (Light::visibleArea, light.cuh:62-76), each weighted by the power
//   heuristic against the other's density.
// * Emissive triangles (shader emission > 0, emission colour at the hit as in
//   raytrace()) are sampled once per hit from a table with probability
//   proportional to emission * area; the emission a diffuse bounce finds is
//   weighted against that density, and the sampled one against the bounce's.
//   A hit from which no diffuse bounce follows gives its sample full weight.

// Slots of the counter RNG: the BSDF half of light i's j-th sample, and the
// two draws of the emitter sample (light indices < 32767).
__host__ __device__ __forceinline__ uint32_t bsdf_light_slot(uint32_t light, uint32_t j) {
    return light_slot(light, j) | 0x80000000u;
}
constexpr uint32_t kSlotEmitter = 0xFFFFFFF0u;

// Power heuristic with exponent 2 (powerHeuristic, sampling.cuh:162-169) as
// 1 / (1 + (p_other / p_this)^2), which does not overflow for large densities.
__device__ __forceinline__ float mis_weight(float p_this, float p_other) {
    const float r = p_other / p_this;
    return 1.0f / (1.0f + r * r);
}

// The Lambert density of BSDF::pdf (bsdf.cuh:22-30), |cos| / pi on wo's
// side, with the cosine taken against the shading normal in world space.
__device__ __forceinline__ float bsdf_pdf(const Bsdf& b, const f3& wo, const f3& wi) {
    const float co = dot(wo, b.N), ci = dot(wi, b.N);
    return (co * ci > 0.0f) ? fabsf(ci) * kInvPi : 0.0f;
}

// BSDF::samplef (bsdf.cuh:53-67) in an orthonormal frame about the shading
// normal: the tangent made orthogonal to N (Gram-Schmidt), bitangent N x S.
// The reference's interpolated tangent frame is not orthonormal on curved
// meshes, so its directions are neither unit nor distributed as |cos| / pi;
// in this frame they are (up to rounding), and the returned density is
// bsdf_pdf of the returned direction, the one the light strategies weigh
// against.
__device__ __forceinline__ f3 bsdf_sample(const Bsdf& b, const f3& wo, float u1, float u2, float& pdf) {
    f3 S = b.S - b.N * dot(b.N, b.S);
    float l = length(S);
    if (!(l > 1e-6f)) {   // tangent (anti)parallel to N: any perpendicular
        S = fabsf(b.N.x) < 0.9f ? cross(b.N, mk3(1.0f, 0.0f, 0.0f)) : cross(b.N, mk3(0.0f, 1.0f, 0.0f));
        l = length(S);
    }
    S = S / l;
    const f3 T = cross(b.N, S);
    f3 lwi = sample_hemisphere_cosine(u1, u2);
    if (dot(wo, b.N) < 0.0f) lwi.z *= -1.0f;
    const f3 wi = local_to_world(lwi, b.N, S, T);
    pdf = bsdf_pdf(b, wo, wi);
    return wi;
}

// The diffuse bounce of the MIS mode (slot 0, as diffuse_bounce): the
// direction from bsdf_sample, throughput f * |wi.N| / pdf.
__device__ __forceinline__ bool mis_bounce(const Bsdf& b, const f3& wo, const f3& thr, uint32_t seed, uint32_t scene,
                                           uint32_t pixel, uint32_t sample, uint32_t rix, f3& wi, f3& nthr,
                                           float& pdf) {
    float u1, u2;
    draw2(seed, scene, pixel, sample, rix, 0u, u1, u2);
    wi = bsdf_sample(b, wo, u1, u2, pdf);
    const f3 f = bsdf_f(b);
    if (pdf > 0.0f && !zero(f)) {
        nthr = thr * (f * (fabsf(dot(wi, b.N)) / pdf));
        return true;
    }
    return false;
}

// Distance t > Epsilon along dir from pos to the parallelogram
// p0 + a e1 + b e2 (a, b in [0, 1]), either face.
__device__ __forceinline__ bool hit_quad(const f3& pos, const f3& dir, const f3& p0, const f3& e1, const f3& e2,
                                         float& t) {
    const f3 P = cross(dir, e2);
    const float det = dot(e1, P);
    if (det == 0.0f) return false;
    const float inv = 1.0f / det;
    const f3 T = pos - p0;
    const float a = dot(T, P) * inv;
    if (!(a >= 0.0f && a <= 1.0f)) return false;
    const f3 Q = cross(T, e1);
    const float b = dot(dir, Q) * inv;
    if (!(b >= 0.0f && b <= 1.0f)) return false;
    t = dot(e2, Q) * inv;
    return t > kEpsilon;
}

__device__ __forceinline__ void tri_verts(const float* __restrict__ V, uint32_t tri, f3& v1, f3& v2, f3& v3) {
    const float* v = V + (size_t)tri * 9;
    v1 = mk3(v[0], v[3], v[6]);
    v2 = mk3(v[1], v[4], v[7]);
    v3 = mk3(v[2], v[5], v[8]);
}

// Cosine at an emitter seen along dir, as the culling test of the traversal
// sees it: the Moller-Trumbore determinant e1 . (dir x e2) (ray.cuh:198-223)
// over |e1 x e2|. Below Epsilon / |e1 x e2| the traversal cannot hit it.
__device__ __forceinline__ float emitter_det(const f3& v1, const f3& v2, const f3& v3, const f3& dir, float& len) {
    const f3 e1 = v2 - v1, e2 = v3 - v1;
    len = length(cross(e1, e2));
    return dot(e1, cross(dir, e2));
}

// Weight of the emission a ray found at triangle `tri` after travelling t
// along dir from a diffuse bounce of density prev_pdf (0: camera or
// specular ray, full weight).
__device__ __forceinline__ float emission_weight(const SceneView& sc, uint32_t tri, const f3& dir, float t,
                                                 float prev_pdf) {
    if (!(prev_pdf > 0.0f)) return 1.0f;
    const float pa = __ldg(sc.mis_pa + tri);
    if (!(pa > 0.0f)) return 1.0f;
    f3 v1, v2, v3;
    tri_verts(sc.verts, tri, v1, v2, v3);
    float len;
    const float det = emitter_det(v1, v2, v3, dir, len);
    const float epdf = (pa * (t * t)) / (det / len);
    return mis_weight(prev_pdf, epdf);
}

// A sample of the direct-lighting estimator up to its shadow ray: the
// contribution `c` it adds if the segment from o along d over (Epsilon, tmax)
// is unoccluded; cand false when it adds nothing whatever the visibility.
// The plain integrators trace the ray at once, the wavefront queues it.
// For the adjoint, c = f * e * geo up to rounding: e is the emitted colour
// scale (an area light's colour * intensity, an emitter's emission colour).
struct ShadowSample {
    f3 c, o, d, e;
    float tmax, geo;
    bool cand;
    uint32_t esi;   // emitter sample only: the shader index of the sampled triangle
};

__device__ __forceinline__ f3 offset_origin(const f3& position, const f3& dir) {
    f3 p = position;   // Ray::offset(Epsilon) (ray.cuh:184-191)
    p.x += kEpsilon * dir.x;
    p.y += kEpsilon * dir.y;
    p.z += kEpsilon * dir.z;
    return p;
}

// An area light seen by the MIS estimator: quad, emission, area, and whether
// it can contribute at all (positive area, non-black BSDF).
struct AreaLightMis {
    f3 p0, e1, e2, ldir, Le0;
    float area;
    bool active;
};
__device__ __forceinline__ AreaLightMis area_light_setup(const aur_light& L, const f3& f) {
    AreaLightMis q;
    q.p0 = from(L.position);
    q.e1 = from(L.e1);
    q.e2 = from(L.e2);
    q.ldir = from(L.direction);
    q.Le0 = from(L.color) * L.intensity;
    q.area = length(cross(q.e1, q.e2));
    q.active = q.area > 0.0f && !zero(f);
    return q;
}

// Light strategy of sample j of area light li: a point on the quad.
__device__ __forceinline__ ShadowSample area_light_sample(const AreaLightMis& q, uint32_t li, uint32_t j, const Bsdf& b,
                                                          const f3& f, const f3& position, const f3& wo,
                                                          uint32_t seed, uint32_t scene, uint32_t pixel,
                                                          uint32_t sample, uint32_t rix) {
    ShadowSample s;
    s.cand = false;
    s.c = mk3(0.0f);
    float u1, u2;
    draw2(seed, scene, pixel, sample, rix, light_slot(li, j), u1, u2);
    const f3 P = q.p0 + ((q.e1 * u1) + (q.e2 * u2));
    f3 wdir = P - position;
    const float wt = length(wdir);
    wdir = wdir / wt;
    const float cl = dot(q.ldir, -wdir);
    const float cs = fmaxf(0.0f, dot(wdir, b.N));
    if (cl > 0.0f && cs > 0.0f) {
        const float lpdf = (wt * wt) / (cl * q.area);
        const float w = mis_weight(lpdf, bsdf_pdf(b, wo, wdir));
        s.c = f * (q.Le0 * cl) * ((cs * w) / lpdf);
        s.e = q.Le0;
        s.geo = cl * ((cs * w) / lpdf);
        s.o = offset_origin(position, wdir);
        s.d = wdir;
        s.tmax = wt + kEpsilon;
        s.cand = true;
    }
    return s;
}

// BSDF strategy of sample j of area light li: a direction traced to the quad.
__device__ __forceinline__ ShadowSample area_bsdf_sample(const AreaLightMis& q, uint32_t li, uint32_t j, const Bsdf& b,
                                                         const f3& f, const f3& position, const f3& wo,
                                                         uint32_t seed, uint32_t scene, uint32_t pixel,
                                                         uint32_t sample, uint32_t rix) {
    ShadowSample s;
    s.cand = false;
    s.c = mk3(0.0f);
    float u1, u2;
    draw2(seed, scene, pixel, sample, rix, bsdf_light_slot(li, j), u1, u2);
    float bpdf, tl;
    const f3 wi = bsdf_sample(b, wo, u1, u2, bpdf);
    if (bpdf > 0.0f && hit_quad(position, wi, q.p0, q.e1, q.e2, tl)) {
        const float cl = dot(q.ldir, -wi);
        const float cs = fmaxf(0.0f, dot(wi, b.N));
        if (cl > 0.0f && cs > 0.0f) {
            const float lpdf = (tl * tl) / (cl * q.area);
            const float w = mis_weight(bpdf, lpdf);
            s.c = f * (q.Le0 * cl) * ((cs * w) / bpdf);
            s.e = q.Le0;
            s.geo = cl * ((cs * w) / bpdf);
            s.o = offset_origin(position, wi);
            s.d = wi;
            s.tmax = tl + kEpsilon;
            s.cand = true;
        }
    }
    return s;
}

// One emitter sample up to its shadow ray: a table entry by its CDF, a
// uniform point on the triangle (square-root parameterisation); the shadow
// ray stops short of the emitter.
__device__ __forceinline__ ShadowSample emitter_shadow_sample(const SceneView& sc, const Bsdf& b, const f3& f,
                                                              const f3& position, const f3& wo, bool bounce,
                                                              uint32_t seed, uint32_t scene, uint32_t pixel,
                                                              uint32_t sample, uint32_t rix) {
    ShadowSample s;
    s.cand = false;
    s.c = mk3(0.0f);
    if (sc.mis_count == 0 || zero(f)) return s;
    float us, ua, ub, uc;
    draw2(seed, scene, pixel, sample, rix, kSlotEmitter, us, ua);
    draw2(seed, scene, pixel, sample, rix, kSlotEmitter + 1u, ub, uc);
    uint32_t lo = 0, hi = sc.mis_count - 1;   // first entry with cdf >= us
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(sc.mis_cdf + mid) >= us) hi = mid; else lo = mid + 1;
    }
    const uint32_t tri = __ldg(sc.mis_tri + lo);
    f3 v1, v2, v3;
    tri_verts(sc.verts, tri, v1, v2, v3);
    const float su = sqrtf(ua);
    const f3 P = ((v1 * (1.0f - su)) + (v2 * (su * (1.0f - ub)))) + (v3 * (su * ub));
    f3 wdir = P - position;
    const float t = length(wdir);
    if (!(t > kEpsilon)) return s;
    wdir = wdir / t;
    float len;
    const float det = emitter_det(v1, v2, v3, wdir, len);
    const float cs = fmaxf(0.0f, dot(wdir, b.N));
    if (det < kEpsilon || !(cs > 0.0f)) return s;
    const float epdf = (__ldg(sc.mis_pa + tri) * (t * t)) / (det / len);
    const float w = bounce ? mis_weight(epdf, bsdf_pdf(b, wo, wdir)) : 1.0f;
    const uint32_t sid = sc.sids[tri];
    s.esi = sid > 0 ? sid - 1 : 0;
    const aur_shader* sh = sc.shaders + s.esi;
    s.c = f * from(sh->emission_color) * ((cs * w) / epdf);
    s.e = from(sh->emission_color);
    s.geo = (cs * w) / epdf;
    s.o = offset_origin(position, wdir);
    s.d = wdir;
    s.tmax = t * 0.9999f;
    s.cand = true;
    return s;
}

// Li at a hit in the MIS mode: emission weighted by ew; ambient and delta
// lights as in the reference; each area light by both strategies
// (area_light_sample, area_bsdf_sample), the two summed per sample and the
// samples averaged; then one emitter sample, whose term is always added.
// Every shadow ray of the hit (a delta light's, the two of each area-light
// sample, the emitter's) is traced at one call site: the loop walks light
// i, sample j and the strategy, so the kernel holds one inlined copy of the
// any-hit traversal for all of them instead of four.
__device__ __forceinline__ f3 direct_light_mis(const SceneView& sc, const aur_shader* sh, const Bsdf& b,
                                               const f3& position, const f3& wo, float ew, bool bounce,
                                               uint32_t seed, uint32_t scene, uint32_t pixel, uint32_t sample,
                                               uint32_t rix, const StackRef& stk, uint32_t& visits, uint32_t* err) {
    f3 Li = from(sh->emission_color) * ew;
    const f3 f = bsdf_f(b);
    const uint32_t nl = sc.num_lights;
    uint32_t i = 0;             // light; nl: the emitter sample; nl + 1: done
    int32_t j = 0;              // area-light sample
    bool second = false;        // the BSDF strategy of sample j is next
    f3 acc = mk3(0.0f), Ls = mk3(0.0f);
    while (i <= nl) {
        ShadowSample s;
        s.cand = false;
        s.c = mk3(0.0f);
        bool to_ls = false;     // a visible sample adds to Ls (area light) or to Li
        bool emitter = false;
        if (i < nl) {
            const aur_light& L = sc.lights[i];
            if (L.type != AUR_LIGHT_AREA) {
                if (L.type == AUR_LIGHT_AMBIENT) Li = Li + f * ((from(L.color) * L.intensity) * L.ambient);
                // estimateDirectRadianceDelta (radiance.cuh:18-33): no offset
                f3 wdir;
                float wt, pdf;
                const f3 Ld = sample_light(L, position, seed, scene, pixel, sample, rix, 0u, wdir, wt, pdf);
                if (pdf > 0.0f && !zero(Ld) && !zero(f)) {
                    s.c = f * Ld * fmaxf(0.0f, dot(wdir, b.N));
                    s.o = position;
                    s.d = wdir;
                    s.tmax = wt;
                    s.cand = true;
                }
                ++i;
            } else {
                const AreaLightMis q = area_light_setup(L, f);   // recomputed: nothing held across the trace
                if (q.active && j < L.samples) {
                    if (!second) {
                        Ls = mk3(0.0f);
                        s = area_light_sample(q, i, (uint32_t)j, b, f, position, wo, seed, scene, pixel, sample, rix);
                    } else {
                        s = area_bsdf_sample(q, i, (uint32_t)j, b, f, position, wo, seed, scene, pixel, sample, rix);
                    }
                    to_ls = true;
                } else {
                    const float ns = (float)L.samples;
                    Li = Li + mk3(acc.x / ns, acc.y / ns, acc.z / ns);
                    acc = mk3(0.0f);
                    j = 0;
                    ++i;
                    continue;
                }
            }
        } else {
            s = emitter_shadow_sample(sc, b, f, position, wo, bounce, seed, scene, pixel, sample, rix);
            emitter = true;
            ++i;
        }
        float du = 0.0f, dv = 0.0f;
        const bool vis =
            s.cand && traverse<true>(sc.recs, sc.nodes, sc.perm, s.o, s.d, s.tmax, du, dv, stk, visits, err) == kNoPrim;
        if (to_ls) {
            if (vis) Ls = Ls + s.c;
        } else if (emitter) {
            Li = Li + (vis ? s.c : mk3(0.0f));   // the emitter sample is always added, zero when unseen
        } else if (vis) {
            Li = Li + s.c;
        }
        if (to_ls) {
            if (second) {
                acc = acc + Ls;
                ++j;
            }
            second = !second;
        }
    }
    return Li;
}

// Li at a hit: emission + ambient + direct light of every light, in the
// reference's order (monteCarloRaytracer.cu:42-52, radiance.cuh:13-80).
// kMis: direct_light_mis; `bounce` says whether a diffuse bounce follows
// this hit.
template <bool kMis>
__device__ __forceinline__ f3 direct_light(const SceneView& sc, const aur_shader* sh, const Bsdf& b, const f3& position,
                                           const f3& wo, float ew, bool bounce, uint32_t seed, uint32_t scene,
                                           uint32_t pixel, uint32_t sample, uint32_t rix, const StackRef& stk,
                                           uint32_t& visits, uint32_t* err) {
    if constexpr (kMis)
        return direct_light_mis(sc, sh, b, position, wo, ew, bounce, seed, scene, pixel, sample, rix, stk, visits, err);
    f3 Li = from(sh->emission_color);
    for (uint32_t i = 0; i < sc.num_lights; ++i) {
        const aur_light& L = sc.lights[i];
        if (L.type == AUR_LIGHT_AMBIENT) Li = Li + bsdf_f(b) * ((from(L.color) * L.intensity) * L.ambient);
        if (L.type != AUR_LIGHT_AREA) {
            // estimateDirectRadianceDelta (radiance.cuh:18-33): no offset
            f3 wdir; float wt, pdf;
            const f3 Ls = sample_light(L, position, seed, scene, pixel, sample, rix, 0u, wdir, wt, pdf);
            if (pdf > 0.0f && !zero(Ls)) {
                const f3 f = bsdf_f(b);
                float du = 0.0f, dv = 0.0f;
                if (!zero(f) &&
                    traverse<true>(sc.recs, sc.nodes, sc.perm, position, wdir, wt, du, dv, stk, visits, err) == kNoPrim)
                    Li = Li + f * Ls * fmaxf(0.0f, dot(wdir, b.N));
            }
        } else {
            // estimateDirectRadiance (radiance.cuh:35-80), light-sampling half
            f3 acc = mk3(0.0f);
            for (int32_t j = 0; j < L.samples; ++j) {
                f3 Ls = mk3(0.0f);
                f3 wdir; float wt, lpdf;
                const f3 Lr = sample_light(L, position, seed, scene, pixel, sample, rix, light_slot(i, (uint32_t)j),
                                           wdir, wt, lpdf);
                // Ray::offset(Epsilon) (ray.cuh:184-191)
                f3 wpos = position;
                wpos.x += kEpsilon * wdir.x;
                wpos.y += kEpsilon * wdir.y;
                wpos.z += kEpsilon * wdir.z;
                wt += kEpsilon;
                if (lpdf > 0.0f && !zero(Lr)) {
                    const f3 f = bsdf_f(b);
                    float du = 0.0f, dv = 0.0f;
                    if (!zero(f) &&
                        traverse<true>(sc.recs, sc.nodes, sc.perm, wpos, wdir, wt, du, dv, stk, visits, err) == kNoPrim)
                        Ls = Ls + f * Lr * fmaxf(0.0f, dot(wdir, b.N));
                }
                acc = acc + Ls;
            }
            const float ns = (float)L.samples;
            Li = Li + mk3(acc.x / ns, acc.y / ns, acc.z / ns);
        }
    }
    return Li;
}

// Diffuse bounce of path mode: BSDF::samplef (bsdf.cuh:222-236) with
// throughput f * |wi.N| / pdf. Returns false when the path ends here.
__device__ __forceinline__ bool diffuse_bounce(const Bsdf& b, const f3& wo, const f3& thr, uint32_t seed,
                                               uint32_t scene, uint32_t pixel, uint32_t sample, uint32_t rix, f3& wi,
                                               f3& nthr, float& pdf) {
    float u1, u2;
    draw2(seed, scene, pixel, sample, rix, 0u, u1, u2);
    const f3 lwo = world_to_local(wo, b.N, b.S, b.T);
    f3 lwi = sample_hemisphere_cosine(u1, u2);
    if (lwo.z < 0.0f) lwi.z *= -1.0f;
    pdf = (lwo.z * lwi.z > 0.0f) ? fabsf(lwi.z) * kInvPi : 0.0f;
    const f3 f = bsdf_f(b);
    wi = local_to_world(lwi, b.N, b.S, b.T);
    if (pdf > 0.0f && !zero(f)) {
        nthr = thr * (f * (fabsf(dot(wi, b.N)) / pdf));
        return true;
    }
    return false;
}

// The rays a hit hands on (monteCarloRaytracer.cu:54-85): a specular
// shader's reflection and refraction rays, path mode's diffuse bounce
// otherwise, in the order they are pushed on the sample's ray stack. Updates
// the ray's weight and throughput (the throughput its colour is added with)
// and the sample's depth counter. Shared by the plain integrator, the
// wavefront's specular batches and the adjoint's stack replay.
struct Continuation {
    PathRay ray[3];
    int n;
    bool bounced;   // the last ray is the diffuse bounce
};

template <bool kMis>
__device__ __forceinline__ Continuation continue_ray(const aur_shader* sh, const Bsdf& b, PathRay& ray,
                                                     const f3& position, const f3& wo, bool path, int& depth, int maxd,
                                                     uint32_t seed, uint32_t scene, uint32_t pixel, uint32_t sample,
                                                     uint32_t rix) {
    Continuation k;
    k.n = 0;
    k.bounced = false;
    const float refl = sh->reflectivity, trans = sh->translucence;
    const bool specular = refl > 0.0f || trans > 0.0f;
    if (specular) depth++;
    if (depth <= maxd && refl > 0.0f) {
        PathRay& nr = k.ray[k.n++];
        nr.pos = position;
        nr.dir = reflect(ray.dir, b.N);
        nr.weight = refl;
        nr.eta = ray.eta;
        nr.thr = path ? ray.thr * refl : mk3(nr.weight);
        nr.pdf = 0.0f;
        ray.weight *= (1.0f - refl);
        ray.thr = path ? ray.thr * (1.0f - refl) : mk3(ray.weight);
    }
    if (depth <= maxd && trans > 0.0f) {
        f3 rN = b.N;
        float etai = ray.eta, etat = sh->refractive_index;
        if (dot(rN, wo) < 0.0f) { rN = -rN; etai = sh->refractive_index; etat = 1.0f; }
        f3 tdir;
        if (refract(tdir, ray.dir, rN, etai, etat)) {
            PathRay& nr = k.ray[k.n++];
            nr.pos = position;
            nr.dir = tdir;
            nr.weight = trans;
            nr.eta = etat;
            nr.thr = path ? ray.thr * trans : mk3(nr.weight);
            nr.pdf = 0.0f;
            ray.weight *= (1.0f - trans);
            ray.thr = path ? ray.thr * (1.0f - trans) : mk3(ray.weight);
        }
    }
    if (path && !specular) {
        depth++;
        if (depth <= maxd) {
            PathRay& nr = k.ray[k.n];
            nr.pos = position;
            nr.weight = 1.0f;
            nr.eta = ray.eta;
            if (kMis ? mis_bounce(b, wo, ray.thr, seed, scene, pixel, sample, rix, nr.dir, nr.thr, nr.pdf)
                     : diffuse_bounce(b, wo, ray.thr, seed, scene, pixel, sample, rix, nr.dir, nr.thr, nr.pdf)) {
                ++k.n;
                k.bounced = true;
            }
        }
    }
    return k;
}

// Integrates one camera ray. RNG key: (seed, scene_id) x (pixel, sample,
// ray index within the sample, slot). kMis: mode is AUR_MODE_PATH_MIS.
template <bool kMis = false>
__device__ __forceinline__ SampleResult integrate(const SceneView& sc, uint32_t max_depth, uint32_t mode,
                                                  uint32_t seed, uint32_t scene, uint32_t pixel, uint32_t sample,
                                                  const PathRay& primary, const StackRef& stk, uint32_t& visits,
                                                  uint32_t* err) {
    PathRay stack[AUR_MAX_DEPTH + 2];
    int sp = 0;
    stack[sp++] = primary;
    int depth = 0;
    SampleResult res;
    res.color = mk3(0.0f);
    res.any_hit = false;
    res.last_tri = kNoPrim;
    res.last_u = res.last_v = 0.0f;
    res.last_pos = res.last_wo = mk3(0.0f);
    uint32_t ray_index = 0;
    const int maxd = (int)max_depth;
    const bool path = kMis || mode == AUR_MODE_PATH;
    while (depth <= maxd && sp > 0) {
        PathRay ray = stack[--sp];
        const uint32_t rix = ray_index++;
        float t = kInfinity, u = 0.0f, v = 0.0f;
        const uint32_t tri = traverse<false>(sc.recs, sc.nodes, sc.perm, ray.pos, ray.dir, t, u, v, stk, visits, err);
        if (tri == kNoPrim) continue;
        res.any_hit = true;
        const f3 position = ray.pos + (ray.dir * t);
        const f3 wo = -ray.dir;
        res.last_tri = tri; res.last_u = u; res.last_v = v; res.last_pos = position; res.last_wo = wo;
        const uint32_t sid = sc.sids[tri];
        const aur_shader* sh = sc.shaders + (sid > 0 ? sid - 1 : 0);   // getSafeID (util/array.h:16-17)
        const float refl = sh->reflectivity, trans = sh->translucence;
        const Bsdf b = get_bsdf(sc, sh, tri, u, v);
        const bool specular = refl > 0.0f || trans > 0.0f;
        const float ew = kMis ? emission_weight(sc, tri, ray.dir, t, ray.pdf) : 1.0f;
        const f3 Li = direct_light<kMis>(sc, sh, b, position, wo, ew, !specular && depth + 1 <= maxd, seed, scene,
                                         pixel, sample, rix, stk, visits, err);
        const Continuation k =
            continue_ray<kMis>(sh, b, ray, position, wo, path, depth, maxd, seed, scene, pixel, sample, rix);
        for (int q = 0; q < k.n; ++q) {
            if (sp < AUR_MAX_DEPTH + 2) stack[sp++] = k.ray[q]; else atomicOr(err, 2u);
        }
        res.color = res.color + Li * ray.thr;
    }
    return res;
}

// The same estimator for scenes without specular shaders: one ray in flight
// per sample, no ray stack (a Lambert hit spawns at most the diffuse bounce).
// Same operations in the same order as integrate().
template <bool kMis = false>
__device__ __forceinline__ SampleResult integrate_diffuse(const SceneView& sc, uint32_t max_depth, uint32_t mode,
                                                          uint32_t seed, uint32_t scene, uint32_t pixel,
                                                          uint32_t sample, const PathRay& primary, const StackRef& stk,
                                                          uint32_t& visits, uint32_t* err) {
    SampleResult res;
    res.color = mk3(0.0f);
    res.any_hit = false;
    res.last_tri = kNoPrim;
    res.last_u = res.last_v = 0.0f;
    res.last_pos = res.last_wo = mk3(0.0f);
    f3 pos = primary.pos, dir = primary.dir, thr = primary.thr;
    float prev_pdf = 0.0f;
    const bool path = kMis || mode == AUR_MODE_PATH;
    uint32_t depth = 0;
    for (uint32_t rix = 0;; ++rix) {
        float t = kInfinity, u = 0.0f, v = 0.0f;
        const uint32_t tri = traverse<false>(sc.recs, sc.nodes, sc.perm, pos, dir, t, u, v, stk, visits, err);
        if (tri == kNoPrim) break;
        res.any_hit = true;
        const f3 position = pos + (dir * t);
        const f3 wo = -dir;
        res.last_tri = tri; res.last_u = u; res.last_v = v; res.last_pos = position; res.last_wo = wo;
        const uint32_t sid = sc.sids[tri];
        const aur_shader* sh = sc.shaders + (sid > 0 ? sid - 1 : 0);
        const Bsdf b = get_bsdf(sc, sh, tri, u, v);
        const float ew = kMis ? emission_weight(sc, tri, dir, t, prev_pdf) : 1.0f;
        const f3 Li = direct_light<kMis>(sc, sh, b, position, wo, ew, depth + 1 <= max_depth, seed, scene, pixel,
                                         sample, rix, stk, visits, err);
        res.color = res.color + Li * thr;
        if (!path) break;
        if (++depth > max_depth) break;
        f3 wi, nthr;
        float bpdf;
        if (!(kMis ? mis_bounce(b, wo, thr, seed, scene, pixel, sample, rix, wi, nthr, bpdf)
                   : diffuse_bounce(b, wo, thr, seed, scene, pixel, sample, rix, wi, nthr, bpdf)))
            break;
        pos = position;
        dir = wi;
        thr = nthr;
        prev_pdf = bpdf;
    }
    return res;
}

// Camera ray of pixel (x, y), sample s of `samples` (utility.cu:18-77): a
// regular sqrt(spp) x sqrt(spp) sub-pixel grid, y = 0 at the bottom.
__device__ __forceinline__ PathRay camera_ray(const aur_camera& cam, uint32_t W, uint32_t H, uint32_t x, uint32_t y,
                                              uint32_t s, uint32_t samples) {
    float px, py;
    if (samples == 1) {
        px = float(x) / float(W) - 0.5f;
        py = float(y) / float(H) - 0.5f;
    } else {
        const short sw = (short)sqrtf((float)samples);
        const short sx = (short)(s % (uint32_t)sw), sy = (short)(s / (uint32_t)sw);
        const float dx = 1.0f / float(W), dy = 1.0f / float(H);
        const float sdx = dx / sw, sdy = dy / sw;
        px = x * dx - 0.5f + (sx * sdx);
        py = y * dy - 0.5f + (sy * sdy);
    }
    PathRay r;
    r.pos = from(cam.position);
    r.weight = 1.0f;
    r.eta = 1.0f;
    r.thr = mk3(1.0f);
    r.pdf = 0.0f;
    r.dir = normalize(px * from(cam.right) * cam.tanfov_x + py * from(cam.up) * cam.tanfov_y + from(cam.forward));
    return r;
}

}  // namespace aur
