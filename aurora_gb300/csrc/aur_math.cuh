// aur_math.cuh — device scalar math shared by the traversal, integrator and
// adjoint kernels.
//
// All kernels are compiled with -fmad=false and IEEE division / square root,
// and every expression keeps the operation order of the reference source
// cited beside it, so results are reproducible bit for bit by a host
// implementation compiled without contraction.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/aurora_gb300.h"

namespace aur {

// util/math.h:17-21
constexpr float kInfinity = 1000000.0f;
constexpr float kEpsilon = 0.0000001f;
constexpr float kPi = 3.1415926536f;
constexpr float kInvPi = 0.3183098862f;

struct f3 { float x, y, z; };

__host__ __device__ __forceinline__ f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__host__ __device__ __forceinline__ f3 mk3(float v) { return mk3(v, v, v); }
__host__ __device__ __forceinline__ f3 from(const aur_float3& a) { return mk3(a.x, a.y, a.z); }
__host__ __device__ __forceinline__ aur_float3 to(const f3& a) { aur_float3 r; r.x = a.x; r.y = a.y; r.z = a.z; return r; }

// util/math.h:92-185
__host__ __device__ __forceinline__ f3 operator-(const f3& a) { return mk3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ f3 operator+(const f3& a, const f3& b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ f3 operator-(const f3& a, const f3& b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ f3 operator*(const f3& a, float b) { return mk3(a.x * b, a.y * b, a.z * b); }
__host__ __device__ __forceinline__ f3 operator*(float a, const f3& b) { return mk3(a * b.x, a * b.y, a * b.z); }
__host__ __device__ __forceinline__ f3 operator*(const f3& a, const f3& b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ f3 operator/(const f3& a, float b) { return mk3(a.x / b, a.y / b, a.z / b); }

// util/math.h:190-191 (left to right)
__host__ __device__ __forceinline__ float dot(const f3& a, const f3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float length(const f3& v) { return sqrtf(dot(v, v)); }
// util/math.h:210-211 with the reference's host rsqrtf = 1/sqrtf (util/math.h:45-46)
__host__ __device__ __forceinline__ f3 normalize(const f3& v) { return v * (1.0f / sqrtf(dot(v, v))); }
// util/math.h:222-224
__host__ __device__ __forceinline__ f3 bclerp(const f3& a, const f3& b, const f3& c, float u, float v) {
    return (1.0f - u - v) * a + u * b + v * c;
}
// util/math.h:227-228
__host__ __device__ __forceinline__ f3 cross(const f3& a, const f3& b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// util/math.h:231-232
__host__ __device__ __forceinline__ f3 reflect(const f3& i, const f3& n) { return i - 2.0f * n * dot(n, i); }
// util/math.h:235-246
__host__ __device__ __forceinline__ bool refract(f3& r, const f3& i, const f3& n, float eta1, float eta2) {
    const float eta = eta1 / eta2;
    const float cosi = dot(n, i);
    const float sint = eta * eta * (1.0f - cosi * cosi);
    if (sint > 1.0f) return false;
    r = eta * i - (eta + sqrtf(1.0f - sint)) * n;
    return true;
}
// util/math.h:86-87
__host__ __device__ __forceinline__ bool zero(const f3& v) { return v.x < kEpsilon && v.y < kEpsilon && v.z < kEpsilon; }
__host__ __device__ __forceinline__ float comp(const f3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// --------------------------------------------------------------------- RNG
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): round function and constants as published.
struct u4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ u4 philox4x32_10(u4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        u4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
    }
    return c;
}

// Uniform in (0, 1] like curand_uniform: ((x >> 8) + 1) * 2^-24 (exact).
__host__ __device__ __forceinline__ float u01(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }

// Two uniforms for (pixel, sample, ray, slot) under key (seed, scene).
// slot 0 is the BSDF sample; slot 1 + (light << 16) + j is sample j of a light.
__host__ __device__ __forceinline__ void draw2(uint32_t seed, uint32_t scene, uint32_t pixel, uint32_t sample,
                                               uint32_t ray, uint32_t slot, float& u1, float& u2) {
    u4 c; c.x = pixel; c.y = sample; c.z = ray; c.w = slot;
    const u4 r = philox4x32_10(c, seed, scene);
    u1 = u01(r.x);
    u2 = u01(r.y);
}

__host__ __device__ __forceinline__ uint32_t light_slot(uint32_t light, uint32_t j) { return 1u + (light << 16) + j; }

// -------------------------------------------------------------- sin / cos
// Own implementation: Cody-Waite reduction by pi/2 (hi part with four low zero
// bits, exact for |q| <= 8) into [-pi/4, pi/4], Taylor polynomials for sin (to
// x^11) and cos (to x^12) by Horner's rule, separately rounded operations.
__host__ __device__ __forceinline__ void own_sincos(float x, float& s, float& c) {
    const float q = rintf(x * 0.636619747f);
    const float r = (x - q * 1.5707950592041016f) - q * 1.2675908465098473e-06f;
    const float r2 = r * r;
    float ps = -2.50521084e-08f;
    ps = ps * r2 + 2.75573192e-06f;
    ps = ps * r2 + -1.98412698e-04f;
    ps = ps * r2 + 8.33333333e-03f;
    ps = ps * r2 + -1.66666667e-01f;
    const float sr = r + (r * r2) * ps;
    float pc = 2.08767570e-09f;
    pc = pc * r2 + -2.75573192e-07f;
    pc = pc * r2 + 2.48015873e-05f;
    pc = pc * r2 + -1.38888889e-03f;
    pc = pc * r2 + 4.16666667e-02f;
    pc = pc * r2 + -0.5f;
    const float cr = 1.0f + r2 * pc;
    const int qi = ((int)q) & 3;
    if (qi == 0) { s = sr; c = cr; }
    else if (qi == 1) { s = cr; c = -sr; }
    else if (qi == 2) { s = -sr; c = -cr; }
    else { s = -cr; c = sr; }
}

// kernels/lib/sampling.cuh:51-82 (concentric disk -> cosine hemisphere)
__host__ __device__ __forceinline__ f3 sample_hemisphere_cosine(float u1, float u2) {
    const float x = 2.0f * u1 - 1.0f;
    const float y = 2.0f * u2 - 1.0f;
    float r, theta;
    if (x >= -y) {
        if (x > y) { r = x; theta = kPi / 4.0f * (y / x); }
        else { r = y; theta = kPi / 4.0f * (2.0f - x / y); }
    } else {
        if (x < y) { r = -x; theta = kPi / 4.0f * (4.0f + y / x); }
        else {
            r = -y;
            if (y != 0.0f) theta = kPi / 4.0f * (6.0f - x / y);
            else theta = 0.0f;
        }
    }
    float s, c;
    own_sincos(theta, s, c);
    const float dx = r * c, dy = r * s;
    return mk3(dx, dy, sqrtf(fmaxf(0.0f, 1.0f - dx * dx - dy * dy)));
}

// kernels/lib/common.cuh:340-354
__host__ __device__ __forceinline__ f3 world_to_local(const f3& v, const f3& N, const f3& S, const f3& T) {
    return mk3(v.x * S.x + v.y * S.y + v.z * S.z, v.x * T.x + v.y * T.y + v.z * T.z, v.x * N.x + v.y * N.y + v.z * N.z);
}
__host__ __device__ __forceinline__ f3 local_to_world(const f3& v, const f3& N, const f3& S, const f3& T) {
    return mk3(S.x * v.x + T.x * v.y + N.x * v.z, S.y * v.x + T.y * v.y + N.y * v.z, S.z * v.x + T.z * v.y + N.z * v.z);
}

// ------------------------------------------------------ geometric tests
// kernels/lib/ray.cuh:198-223 — Moller-Trumbore with back-face culling, on a
// triangle stored as (v1, e1 = v2 - v1, e2 = v3 - v1).
__device__ __forceinline__ bool intersect_tri(const f3& pos, const f3& dir, const f3& v1, const f3& e1, const f3& e2,
                                              float& u, float& v, float& t) {
    const f3 P = cross(dir, e2);
    const float det = dot(e1, P);
    if (det < kEpsilon) return false;
    const f3 T = pos - v1;
    const float du = dot(T, P);
    // Early rejects, taken only where the test below rejects too, so that the
    // division is paid only by likely hits: du < -1e-30 det makes
    // u = du * (1/det) <= -1e-30 (negative, no underflow to -0 since
    // det >= Epsilon); du > 1.000001 det makes u > 1 after both roundings;
    // likewise for v < 0 and u + v > 1 (margin 1e-5 covers three roundings).
    if (du < -1e-30f * det || du > 1.000001f * det) return false;
    const f3 Q = cross(T, e1);
    const float dv = dot(dir, Q);
    if (dv < -1e-30f * det || du + dv > 1.00001f * det) return false;
    const float invdet = 1.0f / det;
    u = du * invdet;
    if (u < 0.0f || u > 1.0f) return false;
    v = dv * invdet;
    if (v < 0.0f || u + v > 1.0f) return false;
    t = dot(e2, Q) * invdet;
    return true;
}

}  // namespace aur
