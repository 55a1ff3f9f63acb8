/*
 * ref_traverse.cpp — the reference's own traversal code compiled as host C++.
 *
 * TEST INFRASTRUCTURE ONLY. Built by build_ref() in oracle/build.py into
 * oracle/_ref/ from the unmodified Nadrin/aurora headers (include path = the reference's
 * src/ directory); nothing of the reference is copied here. It exists to pin
 * the oracle's traversal (oracle/aur_oracle.cpp) to the reference's code:
 *   util/math.h, util/ray.h, util/hitpoint.h, data/geometry.h,
 *   kernels/lib/intersect.cuh, stack.cuh, ray.cuh, primitive.cuh.
 * The shim below supplies what nvcc would: the __device__/__host__ keywords,
 * the CUDA vector types (in namespace gpu, as stdafx.h:22-26 arranges), and
 * device min/max of floats (fminf/fmaxf semantics). Maya types named by
 * util/math.h come from the minimal stand-ins in maya/.
 */
#define __device__
#define __host__
#define __global__

#include <cmath>
#include <cstdint>
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
}  // namespace gpu

#include <util/math.h>

// nvcc resolves min/max of two floats in device code to fminf/fmaxf.
namespace Aurora {
template <> inline float min<float>(const float a, const float b) { return fminf(a, b); }
template <> inline float max<float>(const float a, const float b) { return fmaxf(a, b); }
}  // namespace Aurora

#include <util/ray.h>
#include <util/hitpoint.h>
#include <data/geometry.h>

using namespace Aurora;

#define AURORA_INTSTACK_DEPTH 32
#include <kernels/lib/intersect.cuh>

extern "C" {

/* intersect() over an NMH-ordered soup: t, u, v, NMH position (or -1). */
void ref_trace_closest(const float* vertices, uint32_t count, const float* rays8, uint32_t n, float* out_tuv,
                       int32_t* out_id) {
    Geometry g;
    std::memset(&g, 0, sizeof(g));
    g.vertices = const_cast<float*>(vertices);
    g.count = count;
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays8 + (size_t)i * 8;
        Ray ray(make_float3(r[0], r[1], r[2]), make_float3(r[4], r[5], r[6]), r[3]);
        HitPoint hp;
        const bool hit = intersect(g, ray, hp);
        out_tuv[3 * i + 0] = ray.t;
        out_tuv[3 * i + 1] = hit ? hp.u : 0.0f;
        out_tuv[3 * i + 2] = hit ? hp.v : 0.0f;
        out_id[i] = hit ? hp.triangleID : -1;
    }
}

/* intersectAny(): NMH position of the first hit found, or -1. */
void ref_trace_any(const float* vertices, uint32_t count, const float* rays8, uint32_t n, int32_t* out_id) {
    Geometry g;
    std::memset(&g, 0, sizeof(g));
    g.vertices = const_cast<float*>(vertices);
    g.count = count;
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays8 + (size_t)i * 8;
        Ray ray(make_float3(r[0], r[1], r[2]), make_float3(r[4], r[5], r[6]), r[3]);
        unsigned int id = 0;
        out_id[i] = intersectAny(g, ray, id) ? (int32_t)id : -1;
    }
}

}  // extern "C"
