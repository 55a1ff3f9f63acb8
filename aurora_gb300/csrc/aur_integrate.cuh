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

// Li at a hit: emission + ambient + direct light of every light, in the
// reference's order (monteCarloRaytracer.cu:42-52, radiance.cuh:13-80).
__device__ __forceinline__ f3 direct_light(const SceneView& sc, const aur_shader* sh, const Bsdf& b, const f3& position,
                                           uint32_t seed, uint32_t scene, uint32_t pixel, uint32_t sample,
                                           uint32_t rix, const StackRef& stk, uint32_t& visits, uint32_t* err) {
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
                                               f3& nthr) {
    float u1, u2;
    draw2(seed, scene, pixel, sample, rix, 0u, u1, u2);
    const f3 lwo = world_to_local(wo, b.N, b.S, b.T);
    f3 lwi = sample_hemisphere_cosine(u1, u2);
    if (lwo.z < 0.0f) lwi.z *= -1.0f;
    const float pdf = (lwo.z * lwi.z > 0.0f) ? fabsf(lwi.z) * kInvPi : 0.0f;
    const f3 f = bsdf_f(b);
    wi = local_to_world(lwi, b.N, b.S, b.T);
    if (pdf > 0.0f && !zero(f)) {
        nthr = thr * (f * (fabsf(dot(wi, b.N)) / pdf));
        return true;
    }
    return false;
}

// Integrates one camera ray. RNG key: (seed, scene_id) x (pixel, sample,
// ray index within the sample, slot).
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
        const f3 Li = direct_light(sc, sh, b, position, seed, scene, pixel, sample, rix, stk, visits, err);
        const bool specular = refl > 0.0f || trans > 0.0f;
        if (specular) depth++;
        if (depth <= maxd && refl > 0.0f) {
            PathRay nr;
            nr.pos = position;
            nr.dir = reflect(ray.dir, b.N);
            nr.weight = refl;
            nr.eta = ray.eta;
            nr.thr = mode == AUR_MODE_PATH ? ray.thr * refl : mk3(nr.weight);
            ray.weight *= (1.0f - refl);
            ray.thr = mode == AUR_MODE_PATH ? ray.thr * (1.0f - refl) : mk3(ray.weight);
            if (sp < AUR_MAX_DEPTH + 2) stack[sp++] = nr; else atomicOr(err, 2u);
        }
        if (depth <= maxd && trans > 0.0f) {
            f3 rN = b.N;
            float etai = ray.eta, etat = sh->refractive_index;
            if (dot(rN, wo) < 0.0f) { rN = -rN; etai = sh->refractive_index; etat = 1.0f; }
            f3 tdir;
            if (refract(tdir, ray.dir, rN, etai, etat)) {
                PathRay nr;
                nr.pos = position;
                nr.dir = tdir;
                nr.weight = trans;
                nr.eta = etat;
                nr.thr = mode == AUR_MODE_PATH ? ray.thr * trans : mk3(nr.weight);
                ray.weight *= (1.0f - trans);
                ray.thr = mode == AUR_MODE_PATH ? ray.thr * (1.0f - trans) : mk3(ray.weight);
                if (sp < AUR_MAX_DEPTH + 2) stack[sp++] = nr; else atomicOr(err, 2u);
            }
        }
        if (mode == AUR_MODE_PATH && !specular) {
            depth++;
            if (depth <= maxd) {
                PathRay nr;
                nr.pos = position;
                nr.weight = 1.0f;
                nr.eta = ray.eta;
                if (diffuse_bounce(b, wo, ray.thr, seed, scene, pixel, sample, rix, nr.dir, nr.thr)) {
                    if (sp < AUR_MAX_DEPTH + 2) stack[sp++] = nr; else atomicOr(err, 2u);
                }
            }
        }
        res.color = res.color + Li * ray.thr;
    }
    return res;
}

// The same estimator for scenes without specular shaders: one ray in flight
// per sample, no ray stack (a Lambert hit spawns at most the diffuse bounce).
// Same operations in the same order as integrate().
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
        const f3 Li = direct_light(sc, sh, b, position, seed, scene, pixel, sample, rix, stk, visits, err);
        res.color = res.color + Li * thr;
        if (mode != AUR_MODE_PATH) break;
        if (++depth > max_depth) break;
        f3 wi, nthr;
        if (!diffuse_bounce(b, wo, thr, seed, scene, pixel, sample, rix, wi, nthr)) break;
        pos = position;
        dir = wi;
        thr = nthr;
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
    r.dir = normalize(px * from(cam.right) * cam.tanfov_x + py * from(cam.up) * cam.tanfov_y + from(cam.forward));
    return r;
}

}  // namespace aur
