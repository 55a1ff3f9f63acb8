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
};

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
__device__ __forceinline__ Bsdf get_bsdf(const SceneView& sc, const f3& diffuse_color, float diffuse, uint32_t tri,
                                         float u, float v) {
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
    b.color1 = diffuse_color * diffuse;
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
        const Bsdf b = get_bsdf(sc, from(sh->diffuse_color), sh->diffuse, tri, u, v);
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
        const Bsdf b = get_bsdf(sc, from(sh->diffuse_color), sh->diffuse, tri, u, v);
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
