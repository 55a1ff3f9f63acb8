/*
 * ref_shade.cpp — the reference's own shading code compiled as host C++.
 *
 * TEST INFRASTRUCTURE ONLY. Built by oracle/build.py into oracle/_ref/ from
 * the unmodified Nadrin/aurora headers (include path = the reference's src/
 * directory); nothing of the reference is copied here. It pins the oracle's
 * lighting (oracle/aur_oracle.cpp) to the reference's code:
 *   Shader::getBSDF (kernels/lib/shader.cuh), BSDF::f (bsdf.cuh),
 *   Light::sampleL / visiblePoint (light.cuh), sampleRectangle (sampling.cuh),
 *   estimateAmbientRadiance / estimateDirectRadianceDelta /
 *   estimateDirectRadiance (radiance.cuh), intersectAny (intersect.cuh);
 * and the pieces of the MIS mode the reference has: BSDF::samplef / pdf
 * (bsdf.cuh), powerHeuristic (sampling.cuh), Light::visibleArea (light.cuh).
 * The shim supplies what nvcc would (keywords, CUDA vector types, device
 * min/max of floats) and stands in for cuRAND: curand_uniform() replays the
 * numbers the caller passes, in the order the reference's code asks for them.
 */
#define __device__
#define __host__
#define __global__

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>

namespace gpu {
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct int3 { int x, y, z; };
struct int4 { int x, y, z, w; };
struct uint2 { unsigned x, y; };
struct uint3 { unsigned x, y, z; };
struct uint4 { unsigned x, y, z, w; };
struct uchar3 { unsigned char x, y, z; };
struct uchar4 { unsigned char x, y, z, w; };
inline float2 make_float2(float x, float y) { float2 r = {x, y}; return r; }
inline float3 make_float3(float x, float y, float z) { float3 r = {x, y, z}; return r; }
inline float4 make_float4(float x, float y, float z, float w) { float4 r = {x, y, z, w}; return r; }
inline uchar3 make_uchar3(unsigned char x, unsigned char y, unsigned char z) { uchar3 r = {x, y, z}; return r; }
inline uchar4 make_uchar4(unsigned char x, unsigned char y, unsigned char z, unsigned char w) {
    uchar4 r = {x, y, z, w};
    return r;
}
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
// cuRAND stand-in: replays supplied uniforms (0 once they run out).
struct curandState {
    const float* q;
    uint32_t n, i;
};
inline float curand_uniform(curandState* s) { return s->i < s->n ? s->q[s->i++] : 0.0f; }
}  // namespace gpu
typedef gpu::curandState RNG;
using gpu::curand_uniform;
using gpu::dim3;

#include <util/math.h>

namespace Aurora {
template <> inline float min<float>(const float a, const float b) { return fminf(a, b); }
template <> inline float max<float>(const float a, const float b) { return fmaxf(a, b); }
}  // namespace Aurora

#include <util/ray.h>
#include <util/hitpoint.h>
#include <data/geometry.h>
#include <util/light.h>
#include <util/shader.h>
#include <util/emitter.h>

namespace Aurora {
// core/memory.h is only declared; util/array.h's device arrays are not used here.
void* malloc(const size_t size, MemoryPolicy) { return std::malloc(size); }
void free(void* ptr, MemoryPolicy) { std::free(ptr); }
}  // namespace Aurora

using namespace Aurora;

#define AURORA_INTSTACK_DEPTH 32
#include <kernels/lib/common.cuh>
#include <kernels/lib/intersect.cuh>
#include <kernels/lib/sampling.cuh>
#include <kernels/lib/bsdf.cuh>
#include <kernels/lib/shader.cuh>
#include <kernels/lib/light.cuh>
#include <kernels/lib/radiance.cuh>

#include "aurora_gb300.h"

namespace {

Shader to_shader(const aur_shader& s) {
    Shader r;
    std::memset(&r, 0, sizeof(r));
    r.type = (Shader::ShaderType)s.type;
    r.diffuseColor = make_float3(s.diffuse_color.x, s.diffuse_color.y, s.diffuse_color.z);
    r.emissionColor = make_float3(s.emission_color.x, s.emission_color.y, s.emission_color.z);
    r.specularColor = make_float3(s.specular_color.x, s.specular_color.y, s.specular_color.z);
    r.reflectionColor = make_float3(s.reflection_color.x, s.reflection_color.y, s.reflection_color.z);
    r.diffuse = s.diffuse;
    r.emission = s.emission;
    r.exponent = s.exponent;
    r.reflectivity = s.reflectivity;
    r.translucence = s.translucence;
    r.refractiveIndex = s.refractive_index;
    r.texture = s.texture;
    return r;
}

Light to_light(const aur_light& l) {
    Light r;
    std::memset(&r, 0, sizeof(r));
    r.type = (Light::LightType)l.type;
    r.intensity = l.intensity;
    r.ambient = l.ambient;
    r.area = l.area;
    r.samples = (short)l.samples;
    r.position = make_float3(l.position.x, l.position.y, l.position.z);
    r.color = make_float3(l.color.x, l.color.y, l.color.z);
    r.direction = make_float3(l.direction.x, l.direction.y, l.direction.z);
    r.e1 = make_float3(l.e1.x, l.e1.y, l.e1.z);
    r.e2 = make_float3(l.e2.x, l.e2.y, l.e2.z);
    return r;
}

}  // namespace

extern "C" {

/* Which replayed uniform an area light's sample scales e1 by: 0 if the first
 * one drawn, 1 if the second (the order of the two curand_uniform() arguments
 * of sampleRectangle in Light::sampleL, light.cuh:44-48, is up to the
 * compiler). Probed with the reference's own Light::sampleL. */
int ref_uniform_order(void) {
    const float q[2] = {0.25f, 0.75f};
    RNG rng = {q, 2, 0};
    Light L;
    std::memset(&L, 0, sizeof(L));
    L.type = Light::AreaLight;
    L.intensity = 1.0f;
    L.samples = 1;
    L.position = make_float3(0.0f, 0.0f, 0.0f);
    L.e1 = make_float3(1.0f, 0.0f, 0.0f);
    L.e2 = make_float3(0.0f, 1.0f, 0.0f);
    L.direction = make_float3(0.0f, 0.0f, 1.0f);
    Ray ray(make_float3(0.0f, 0.0f, 1.0f));
    float pdf;
    L.sampleL(&rng, ray, pdf);
    const float px = ray.pos.x + ray.dir.x * ray.t;
    return fabsf(px - 0.25f) < 1e-4f ? 0 : 1;
}

/* The radiance Li at each camera-ray hit as the reference's raytrace()
 * gathers it (monteCarloRaytracer.cu:33-52, no texture): Shader::getBSDF,
 * emission, then per light estimateAmbientRadiance, and
 * estimateDirectRadianceDelta or estimateDirectRadiance. Geometry: NMH-ordered
 * vertices V, normals N, per-vertex tangents TG and bitangents BT (9 floats per
 * triangle each), shader ids S (1-based). Hit i: ray rays8[8i..] (origin,
 * tmax, direction, pad), NMH triangle tri[i] (skipped when < 0), t/u/v in
 * tuv[3i..]. The reference's cuRAND draws are replayed from
 * uniforms[i * per_hit ..], in draw order. out: 3 floats per hit. */
void ref_shade_hits(const float* V, const float* N, const float* TG, const float* BT, const uint16_t* S,
                    uint32_t count, const aur_shader* shaders, uint32_t nshaders, const aur_light* lights,
                    uint32_t nlights, const float* rays8, const int32_t* tri, const float* tuv, uint32_t n,
                    const float* uniforms, uint32_t per_hit, float* out) {
    Geometry g;
    std::memset(&g, 0, sizeof(g));
    g.vertices = const_cast<float*>(V);
    g.normals = const_cast<float*>(N);
    g.tangents = const_cast<float*>(TG);
    g.bitangents = const_cast<float*>(BT);
    g.shaders = const_cast<unsigned short*>(S);
    g.count = count;
    Shader* sh = new Shader[nshaders];
    Light* lt = new Light[nlights > 0 ? nlights : 1];
    for (uint32_t k = 0; k < nshaders; ++k) sh[k] = to_shader(shaders[k]);
    for (uint32_t k = 0; k < nlights; ++k) lt[k] = to_light(lights[k]);
    for (uint32_t i = 0; i < n; ++i) {
        out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = 0.0f;
        if (tri[i] < 0) continue;
        const float* r = rays8 + (size_t)i * 8;
        Ray ray(make_float3(r[0], r[1], r[2]), make_float3(r[4], r[5], r[6]), tuv[3 * i]);
        HitPoint hp;
        hp.triangleID = tri[i];
        hp.u = tuv[3 * i + 1];
        hp.v = tuv[3 * i + 2];
        hp.position = ray.point();
        hp.wo = -ray.dir;
        RNG rng = {uniforms + (size_t)i * per_hit, per_hit, 0};
        const Shader& shader = sh[getSafeID(g.shaders[hp.triangleID])];
        BSDF bsdf = shader.getBSDF(g, hp.triangleID, hp.u, hp.v);
        float3 Li = shader.emissionColor;
        for (uint32_t k = 0; k < nlights; ++k) {
            const Light& light = lt[k];
            if (light.isAmbientLight()) Li = Li + estimateAmbientRadiance(light, bsdf);
            if (light.isDeltaLight())
                Li = Li + estimateDirectRadianceDelta(g, light, shader, bsdf, hp);
            else
                Li = Li + estimateDirectRadiance(&rng, g, light, shader, bsdf, hp);
        }
        out[3 * i] = Li.x;
        out[3 * i + 1] = Li.y;
        out[3 * i + 2] = Li.z;
    }
    delete[] sh;
    delete[] lt;
}

/* The BSDF sampling pieces of the MIS mode, through the reference's code at
 * each hit (located as in ref_shade_hits): BSDF::samplef with two replayed
 * uniforms per hit, then BSDF::pdf of the sampled direction and of a given
 * probe direction (bsdf.cuh:22-30, 48-67). out, 6 floats per hit: sampled
 * wi.xyz, samplef's pdf, pdf(wo, wi), pdf(wo, probe). */
void ref_bsdf_hits(const float* V, const float* N, const float* TG, const float* BT, const uint16_t* S,
                   uint32_t count, const aur_shader* shaders, uint32_t nshaders, const float* rays8,
                   const int32_t* tri, const float* tuv, uint32_t n, const float* uniforms, const float* probes,
                   float* out) {
    Geometry g;
    std::memset(&g, 0, sizeof(g));
    g.vertices = const_cast<float*>(V);
    g.normals = const_cast<float*>(N);
    g.tangents = const_cast<float*>(TG);
    g.bitangents = const_cast<float*>(BT);
    g.shaders = const_cast<unsigned short*>(S);
    g.count = count;
    Shader* sh = new Shader[nshaders];
    for (uint32_t k = 0; k < nshaders; ++k) sh[k] = to_shader(shaders[k]);
    for (uint32_t i = 0; i < n; ++i) {
        float* o = out + (size_t)i * 6;
        for (int q = 0; q < 6; ++q) o[q] = 0.0f;
        if (tri[i] < 0) continue;
        const float* r = rays8 + (size_t)i * 8;
        Ray ray(make_float3(r[0], r[1], r[2]), make_float3(r[4], r[5], r[6]), tuv[3 * i]);
        const float3 wo = -ray.dir;
        const Shader& shader = sh[getSafeID(g.shaders[tri[i]])];
        BSDF bsdf = shader.getBSDF(g, tri[i], tuv[3 * i + 1], tuv[3 * i + 2]);
        RNG rng = {uniforms + (size_t)i * 2, 2, 0};
        float3 wi;
        float pdf;
        bsdf.samplef(&rng, wo, wi, pdf);
        const float3 pr = make_float3(probes[3 * i], probes[3 * i + 1], probes[3 * i + 2]);
        o[0] = wi.x; o[1] = wi.y; o[2] = wi.z;
        o[3] = pdf;
        o[4] = bsdf.pdf(wo, wi);
        o[5] = bsdf.pdf(wo, pr);
    }
    delete[] sh;
}

/* Primitive3::area (primitive.cuh:74-85) of n triangles in the reference
 * layout (readPoints), the emitter table's area. */
void ref_triangle_areas(const float* V, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        Primitive3 p;
        p.readPoints(V + (size_t)i * 9);
        out[i] = p.area();
    }
}

/* powerHeuristic(1, a, 1, b) (sampling.cuh:162-169). */
float ref_power_heuristic(float a, float b) { return powerHeuristic(1, a, 1, b); }

/* Light::visibleArea (light.cuh:62-76) with no geometry to occlude: 1 and
 * the distance to the light's quad when the ray meets one of its two
 * triangles (Ray::intersect, culled), else 0. */
int ref_area_hit(const aur_light* l, const float* pos, const float* dir, float* t) {
    const Light L = to_light(*l);
    Geometry g;
    std::memset(&g, 0, sizeof(g));
    Ray ray(make_float3(pos[0], pos[1], pos[2]), make_float3(dir[0], dir[1], dir[2]), Infinity);
    const bool hit = L.visibleArea(g, ray);
    *t = ray.t;
    return hit ? 1 : 0;
}

}  // extern "C"
