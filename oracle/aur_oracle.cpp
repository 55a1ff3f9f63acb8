/*
 * aur_oracle.cpp — CPU restatement of the Aurora rendering hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker the CUDA kernels in
 * aurora_gb300/csrc are compared against, and the timed CPU baseline of the
 * benchmark. It is never linked into, loaded by or called from the product
 * library.
 *
 * Every function restates the algorithm of the Nadrin/aurora source file cited
 * beside it, in the same floating-point operation order, compiled with
 * -ffp-contract=off so that no multiply-add is fused. Where the reference is
 * racy or unspecified the deterministic rule marked [canon] is used instead:
 *   - NMH build: every ordering ties by the lower original prim id; the
 *     max-key swap ties by the lower prim id (the reference's atomicCAS loop,
 *     kernels/rebuilder.cu:93-125, is nondeterministic on ties).
 *   - Closest hit: equal t goes to the lower original prim id (the reference
 *     keeps the first tested, intersect.cuh:123-136).
 *   - RNG: a counter-based Philox4x32-10 keyed by (seed, scene, pixel, sample,
 *     ray, slot) replaces per-pixel cuRAND XORWOW state (utility.cu:182-197);
 *     the two area-light uniforms are drawn in a fixed order.
 *   - normalize(v) = v * (1/sqrtf(dot(v,v))), the reference's host definition
 *     of rsqrtf (util/math.h:45-46), so CPU and GPU round identically.
 *   - sin/cos are this project's own (Cody-Waite reduction + Taylor series).
 */
#include "../include/aurora_gb300.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// util/math.h:17-21
const float kInfinity = 1000000.0f;
const float kEpsilon = 0.0000001f;
const float kPi = 3.1415926536f;
const float kInvPi = 0.3183098862f;

struct F2 { float x, y; };
struct F3 { float x, y, z; };

inline F3 mk3(float x, float y, float z) { F3 r; r.x = x; r.y = y; r.z = z; return r; }
inline F3 mk3(float v) { return mk3(v, v, v); }
inline F3 from(const aur_float3& a) { return mk3(a.x, a.y, a.z); }
// util/math.h:92-185, component-wise, left to right
inline F3 operator-(const F3& a) { return mk3(-a.x, -a.y, -a.z); }
inline F3 operator+(const F3& a, const F3& b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline F3 operator-(const F3& a, const F3& b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline F3 operator*(const F3& a, float b) { return mk3(a.x * b, a.y * b, a.z * b); }
inline F3 operator*(float a, const F3& b) { return mk3(a * b.x, a * b.y, a * b.z); }
inline F3 operator*(const F3& a, const F3& b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline F3 operator/(const F3& a, float b) { return mk3(a.x / b, a.y / b, a.z / b); }
// util/math.h:190-191
inline float dot(const F3& a, const F3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// util/math.h:196-197
inline float length(const F3& v) { return sqrtf(dot(v, v)); }
// util/math.h:210-211 with rsqrtf = 1/sqrtf (util/math.h:45-46)
inline F3 normalize(const F3& v) { return v * (1.0f / sqrtf(dot(v, v))); }
// util/math.h:222-224
inline F3 bclerp(const F3& a, const F3& b, const F3& c, float u, float v) {
    return (1.0f - u - v) * a + u * b + v * c;
}
// util/math.h:227-228
inline F3 cross(const F3& a, const F3& b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// util/math.h:231-232
inline F3 reflect(const F3& i, const F3& n) { return i - 2.0f * n * dot(n, i); }
// util/math.h:235-246
inline bool refract(F3& r, const F3& i, const F3& n, float eta1, float eta2) {
    const float eta = eta1 / eta2;
    const float cosi = dot(n, i);
    const float sint = eta * eta * (1.0f - cosi * cosi);
    if (sint > 1.0f) return false;
    r = eta * i - (eta + sqrtf(1.0f - sint)) * n;
    return true;
}
// util/math.h:86-87
inline bool zero(const F3& v) { return v.x < kEpsilon && v.y < kEpsilon && v.z < kEpsilon; }
inline float comp(const F3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// util/math.h:253-261
inline uint32_t log2i(uint32_t x) {
    uint32_t r = (uint32_t)(-1);
    while (x) { x >>= 1; r++; }
    return r;
}
// util/math.h:264-272
inline uint32_t exp2i(uint32_t x) {
    if (x == 0) return 1;
    uint32_t r = 2;
    while (--x) r *= 2;
    return r;
}

// ------------------------------------------------------------------ RNG
// Philox4x32-10, J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11. Round function and
// constants as published there.
struct U4 { uint32_t x, y, z, w; };

inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        U4 n;
        n.x = (uint32_t)(p1 >> 32) ^ c.y ^ k0;
        n.y = (uint32_t)p1;
        n.z = (uint32_t)(p0 >> 32) ^ c.w ^ k1;
        n.w = (uint32_t)p0;
        c = n;
    }
    return c;
}

// Uniform in (0, 1], the range of curand_uniform: ((x >> 8) + 1) * 2^-24.
inline float u01(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }

struct RngKey { uint32_t seed, scene; };
// slot 0: BSDF sample; slot 1 + (light << 16) + j: j-th sample of light `light`.
inline void draw2(const RngKey& k, uint32_t pixel, uint32_t sample, uint32_t ray, uint32_t slot,
                  float& u1, float& u2) {
    U4 c; c.x = pixel; c.y = sample; c.z = ray; c.w = slot;
    const U4 r = philox4x32_10(c, k.seed, k.scene);
    u1 = u01(r.x);
    u2 = u01(r.y);
}

// ------------------------------------------------------------ sin / cos
// Own implementation: Cody-Waite reduction by pi/2 into [-pi/4, pi/4], then
// Taylor polynomials (sin to x^11, cos to x^12) evaluated by Horner's rule
// with separately rounded multiplies and adds.
inline void own_sincos(float x, float& s, float& c) {
    const float kTwoOverPi = 0.636619747f;
    const float kPio2Hi = 1.5707950592041016f;  // pi/2 = hi + lo; hi has 4 low zero bits,
    const float kPio2Lo = 1.2675908465098473e-06f;  // so q*hi is exact for |q| <= 8
    const float q = rintf(x * kTwoOverPi);
    const float r = (x - q * kPio2Hi) - q * kPio2Lo;
    const float r2 = r * r;
    float ps = -2.50521084e-08f;               // -1/11!
    ps = ps * r2 + 2.75573192e-06f;            //  1/9!
    ps = ps * r2 + -1.98412698e-04f;           // -1/7!
    ps = ps * r2 + 8.33333333e-03f;            //  1/5!
    ps = ps * r2 + -1.66666667e-01f;           // -1/3!
    const float sr = r + (r * r2) * ps;
    float pc = 2.08767570e-09f;                //  1/12!
    pc = pc * r2 + -2.75573192e-07f;           // -1/10!
    pc = pc * r2 + 2.48015873e-05f;            //  1/8!
    pc = pc * r2 + -1.38888889e-03f;           // -1/6!
    pc = pc * r2 + 4.16666667e-02f;            //  1/4!
    pc = pc * r2 + -0.5f;                      // -1/2!
    const float cr = 1.0f + r2 * pc;
    const int qi = ((int)q) & 3;
    if (qi == 0) { s = sr; c = cr; }
    else if (qi == 1) { s = cr; c = -sr; }
    else if (qi == 2) { s = -sr; c = -cr; }
    else { s = -cr; c = sr; }
}

// -------------------------------------------------------------- sampling
// kernels/lib/sampling.cuh:51-73
inline F2 sampleDiskConcentric(float u1, float u2) {
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
    F2 d; d.x = r * c; d.y = r * s;
    return d;
}
// kernels/lib/sampling.cuh:76-82
inline F3 sampleHemisphereCosine(float u1, float u2) {
    const F2 d = sampleDiskConcentric(u1, u2);
    return mk3(d.x, d.y, sqrtf(fmaxf(0.0f, 1.0f - d.x * d.x - d.y * d.y)));
}
// kernels/lib/common.cuh:340-354
inline F3 worldToLocal(const F3& v, const F3& N, const F3& S, const F3& T) {
    return mk3(v.x * S.x + v.y * S.y + v.z * S.z, v.x * T.x + v.y * T.y + v.z * T.z,
               v.x * N.x + v.y * N.y + v.z * N.z);
}
inline F3 localToWorld(const F3& v, const F3& N, const F3& S, const F3& T) {
    return mk3(S.x * v.x + T.x * v.y + N.x * v.z, S.y * v.x + T.y * v.y + N.y * v.z,
               S.z * v.x + T.z * v.y + N.z * v.z);
}

// ------------------------------------------------------------ traversal
struct Ray {
    F3 pos, dir;
    float t, weight, eta;
    F3 thr;          // RGB path throughput (path mode); (weight,weight,weight) otherwise
    float pdf = 0.0f; // AUR_MODE_PATH_MIS: density of the diffuse bounce that made the ray, 0 otherwise
};

// kernels/lib/ray.cuh:198-223 (Moller-Trumbore with back-face culling)
inline bool intersectTri(const Ray& ray, const float* v, float& u, float& vv, float& t) {
    const F3 v1 = mk3(v[0], v[3], v[6]);
    const F3 v2 = mk3(v[1], v[4], v[7]);
    const F3 v3 = mk3(v[2], v[5], v[8]);
    const F3 e1 = v2 - v1;
    const F3 e2 = v3 - v1;
    const F3 P = cross(ray.dir, e2);
    const float det = dot(e1, P);
    if (det < kEpsilon) return false;
    const float invdet = 1.0f / det;
    const F3 T = ray.pos - v1;
    u = dot(T, P) * invdet;
    if (u < 0.0f || u > 1.0f) return false;
    const F3 Q = cross(T, e1);
    vv = dot(ray.dir, Q) * invdet;
    if (vv < 0.0f || u + vv > 1.0f) return false;
    t = dot(e2, Q) * invdet;
    return true;
}

// kernels/lib/ray.cuh:225-237; device min/max of floats are fminf/fmaxf
inline bool intersectSlab(const Ray& ray, float s0, float s1, int axis, F2& range) {
    const float p = comp(ray.pos, axis);
    const float d = comp(ray.dir, axis);
    const float dx = (s0 - p) / d;
    const float dy = (s1 - p) / d;
    range.x = fmaxf(fminf(dx, dy), range.x);
    range.y = fminf(fmaxf(dx, dy), range.y);
    return (range.x <= range.y) && (range.x <= ray.t);
}

inline float vmin(const float* v, int a) { return fminf(fminf(v[3 * a], v[3 * a + 1]), v[3 * a + 2]); }
inline float vmax(const float* v, int a) { return fmaxf(fmaxf(v[3 * a], v[3 * a + 1]), v[3 * a + 2]); }

struct TState { uint32_t index; int axis; F2 range; };

// kernels/lib/intersect.cuh:95-152 (closest hit), [canon] tie on t -> lower perm id.
// Returns the NMH position of the hit (or -1). ray.t is updated.
inline int64_t traceClosest(const float* V, uint32_t count, const uint32_t* perm, Ray& ray,
                            float& hu, float& hv, uint64_t* visits) {
    int64_t hit = -1;
    TState stack[64];
    int sp = 0;
    TState s0; s0.index = 0; s0.axis = 0; s0.range.x = kEpsilon; s0.range.y = kInfinity;
    stack[sp++] = s0;
    while (sp > 0) {
        TState st = stack[--sp];
        if (st.index >= count) continue;
        if (visits) ++*visits;
        const float* v1 = V + (size_t)st.index * 9;
        const float* v2 = V + (size_t)(st.index + 1) * 9;
        const float s0x = fminf(vmin(v1, st.axis), vmin(v2, st.axis));
        const float s0y = fmaxf(vmax(v1, st.axis), vmax(v2, st.axis));
        if (!intersectSlab(ray, s0x, s0y, st.axis, st.range)) continue;
        for (uint32_t k = 0; k < 2; ++k) {
            float u, v, t;
            const uint32_t idx = st.index + k;
            if (intersectTri(ray, V + (size_t)idx * 9, u, v, t) && t > kEpsilon) {
                bool take = t < ray.t;
                if (!take && t == ray.t && hit >= 0 && perm && perm[idx] < perm[(size_t)hit]) take = true;
                if (take) { ray.t = t; hu = u; hv = v; hit = idx; }
            }
        }
        const int axis = (st.axis + 1) % 3;
        uint32_t L = 2 * st.index + 2, R = 2 * st.index + 4;
        if (comp(ray.dir, axis) < 0.0f) std::swap(L, R);
        TState a; a.index = R; a.axis = axis; a.range = st.range;
        TState b; b.index = L; b.axis = axis; b.range = st.range;
        stack[sp++] = a;
        stack[sp++] = b;
    }
    return hit;
}

// kernels/lib/intersect.cuh:36-86 (any hit). Returns NMH position or -1.
inline int64_t traceAny(const float* V, uint32_t count, const Ray& ray, uint64_t* visits) {
    TState stack[64];
    int sp = 0;
    TState s0; s0.index = 0; s0.axis = 0; s0.range.x = kEpsilon; s0.range.y = kInfinity;
    stack[sp++] = s0;
    while (sp > 0) {
        TState st = stack[--sp];
        if (st.index >= count) continue;
        if (visits) ++*visits;
        const float* v1 = V + (size_t)st.index * 9;
        const float* v2 = V + (size_t)(st.index + 1) * 9;
        const float s0x = fminf(vmin(v1, st.axis), vmin(v2, st.axis));
        const float s0y = fmaxf(vmax(v1, st.axis), vmax(v2, st.axis));
        if (!intersectSlab(ray, s0x, s0y, st.axis, st.range)) continue;
        float u, v, t;
        if (intersectTri(ray, v1, u, v, t) && t > kEpsilon && t < ray.t) return st.index;
        if (intersectTri(ray, v2, u, v, t) && t > kEpsilon && t < ray.t) return st.index + 1;
        const int axis = (st.axis + 1) % 3;
        uint32_t L = 2 * st.index + 2, R = 2 * st.index + 4;
        if (comp(ray.dir, axis) < 0.0f) std::swap(L, R);
        TState a; a.index = R; a.axis = axis; a.range = st.range;
        TState b; b.index = L; b.axis = axis; b.range = st.range;
        stack[sp++] = a;
        stack[sp++] = b;
    }
    return -1;
}

template <class F>
void parallel_for(uint32_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 256) { for (uint32_t i = 0; i < n; ++i) f(i, 0); return; }
    std::atomic<uint32_t> next(0);
    std::vector<std::thread> th;
    for (int w = 0; w < nthreads; ++w) {
        th.emplace_back([&, w]() {
            for (;;) {
                const uint32_t b = next.fetch_add(64);
                if (b >= n) break;
                const uint32_t e = std::min(n, b + 64);
                for (uint32_t i = b; i < e; ++i) f(i, w);
            }
        });
    }
    for (auto& t : th) t.join();
}

inline Ray rayFrom(const aur_ray& r) {
    Ray ray;
    ray.pos = mk3(r.ox, r.oy, r.oz);
    ray.dir = mk3(r.dx, r.dy, r.dz);
    ray.t = r.tmax;
    ray.weight = 1.0f;
    ray.eta = 1.0f;
    ray.thr = mk3(1.0f);
    return ray;
}

// ------------------------------------------------------------ NMH build
// kernels/rebuilder.cu:40-50
inline void calcPartition(uint32_t N, uint32_t& L, uint32_t& R) {
    const uint32_t n = N / 2;
    const uint32_t H = log2i(n);
    const uint32_t s = exp2i(H - 1) - 1;
    const uint32_t S = exp2i(H) - 1;
    const int o = int((n - 1) - s - S);
    const uint32_t O = (uint32_t)(o > 0 ? o : 0);
    R = 2 * (s + O);
    L = 2 * (n - 1) - R;
}

struct Bounds { std::vector<float> mn[3], mx[3]; };

// kernels/rebuilder.cu:72-91
void triangleBounds(const float* V, uint32_t n, Bounds& b) {
    for (int a = 0; a < 3; ++a) { b.mn[a].resize(n); b.mx[a].resize(n); }
    for (uint32_t i = 0; i < n; ++i) {
        const float* v = V + (size_t)i * 9;
        for (int a = 0; a < 3; ++a) { b.mn[a][i] = vmin(v, a); b.mx[a][i] = vmax(v, a); }
    }
}

}  // namespace

extern "C" {

// Philox known-answer hook for tests.
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    U4 c; c.x = ctr[0]; c.y = ctr[1]; c.z = ctr[2]; c.w = ctr[3];
    const U4 r = philox4x32_10(c, key[0], key[1]);
    out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}

void orc_sincos(const float* x, uint32_t n, float* s, float* c) {
    for (uint32_t i = 0; i < n; ++i) own_sincos(x[i], s[i], c[i]);
}

void orc_calc_partition(uint32_t N, uint32_t* L, uint32_t* R) { calcPartition(N, *L, *R); }

/*
 * NMH build, [canon] restatement of cudaRebuildNMH (kernels/rebuilder.cu:311-450).
 * Node k holds triangles at positions 2k, 2k+1; its children are nodes 2k+1,
 * 2k+2 (intersect.cuh:139-140). Level d uses axis d mod 3. For a node with
 * member set S at level d (axis a):
 *   - sort S by (min-key on a, prim id) (sortTriangles, :262-289);
 *   - pair[0] = first; pair[1] = largest max-key on a among the rest, ties to
 *     the lower prim id (swapMaxTriangleTPS/TPT, :93-151);
 *   - the remainder, ordered by (min-key on axis a+1, prim id) as the next
 *     level's sort does, gives its first numL to the left child and the rest
 *     to the right (calcPartition + emitSplits, :40-50, :189-215).
 * The final level's sort (:381-385) leaves every pair ordered by
 * (min-key on the last level's axis, prim id).
 * vertices: n*9 (n even). perm_out[i] = original id at NMH position i.
 * Returns the number of levels, or -1 on an invalid count.
 */
int orc_nmh_build(const float* vertices, uint32_t n, uint32_t* perm_out) {
    if (n == 0) return 0;
    if (n % 2) return -1;
    const uint32_t nodes = n / 2;
    const uint32_t levels = log2i(nodes) + 1;
    Bounds b;
    triangleBounds(vertices, n, b);
    std::vector<std::vector<uint32_t>> members(nodes);
    std::vector<uint32_t> all(n);
    for (uint32_t i = 0; i < n; ++i) all[i] = i;
    members[0] = all;
    auto byMin = [&](int a) {
        return [&b, a](uint32_t p, uint32_t q) {
            const float kp = b.mn[a][p], kq = b.mn[a][q];
            if (kp != kq) return kp < kq;
            return p < q;
        };
    };
    std::vector<uint32_t> pair0(nodes), pair1(nodes);
    for (uint32_t k = 0; k < nodes; ++k) {
        const uint32_t level = log2i(k + 1);
        const int a = (int)(level % 3);
        std::vector<uint32_t>& S = members[k];
        std::sort(S.begin(), S.end(), byMin(a));
        pair0[k] = S[0];
        if (S.size() == 2) { pair1[k] = S[1]; continue; }
        size_t best = 1;
        for (size_t i = 2; i < S.size(); ++i) {
            const float kv = b.mx[a][S[i]], kb = b.mx[a][S[best]];
            if (kv > kb || (kv == kb && S[i] < S[best])) best = i;
        }
        pair1[k] = S[best];
        std::vector<uint32_t> rest;
        rest.reserve(S.size() - 2);
        for (size_t i = 1; i < S.size(); ++i) if (i != best) rest.push_back(S[i]);
        std::sort(rest.begin(), rest.end(), byMin((a + 1) % 3));
        uint32_t numL, numR;
        calcPartition((uint32_t)S.size(), numL, numR);
        if (numL + numR != rest.size()) return -2;
        const uint32_t cl = 2 * k + 1, cr = 2 * k + 2;
        if ((numL > 0) != (cl < nodes) || (numR > 0) != (cr < nodes)) return -3;
        if (numL) members[cl].assign(rest.begin(), rest.begin() + numL);
        if (numR) members[cr].assign(rest.begin() + numL, rest.end());
        std::vector<uint32_t>().swap(S);
    }
    const int al = (int)((levels - 1) % 3);
    auto less = byMin(al);
    for (uint32_t k = 0; k < nodes; ++k) {
        uint32_t p = pair0[k], q = pair1[k];
        if (less(q, p)) std::swap(p, q);
        perm_out[2 * k] = p;
        perm_out[2 * k + 1] = q;
    }
    return (int)levels;
}

/* applyIndices (rebuilder.cu:217-245) for 9-float attributes. */
void orc_gather9(const float* src, const uint32_t* perm, uint32_t n, float* dst) {
    for (uint32_t i = 0; i < n; ++i) std::memcpy(dst + (size_t)i * 9, src + (size_t)perm[i] * 9, 36);
}

/*
 * Closest hit over an NMH-ordered soup (intersect.cuh:95-152), [canon] ties.
 * V: count*9 NMH-ordered vertices; perm: NMH position -> original id.
 * hits[i].prim = original id or AUR_NO_HIT. visits (nullable): per-ray node
 * fetch counts. Returns total node fetches.
 */
uint64_t orc_trace_closest(const float* V, uint32_t count, const uint32_t* perm, const aur_ray* rays,
                           uint32_t n, aur_hit* hits, uint32_t* visits, int nthreads) {
    std::vector<uint64_t> tot((size_t)std::max(1, nthreads), 0);
    parallel_for(n, nthreads, [&](uint32_t i, int w) {
        Ray ray = rayFrom(rays[i]);
        float u = 0.0f, v = 0.0f;
        uint64_t vis = 0;
        const int64_t h = traceClosest(V, count, perm, ray, u, v, &vis);
        aur_hit out;
        if (h >= 0) { out.t = ray.t; out.u = u; out.v = v; out.prim = perm[h]; }
        else { out.t = rays[i].tmax; out.u = 0.0f; out.v = 0.0f; out.prim = AUR_NO_HIT; }
        hits[i] = out;
        if (visits) visits[i] = (uint32_t)vis;
        tot[(size_t)w] += vis;
    });
    uint64_t s = 0;
    for (uint64_t x : tot) s += x;
    return s;
}

/* Any hit (intersect.cuh:36-86): occluder[i] = original id or AUR_NO_HIT. */
uint64_t orc_trace_any(const float* V, uint32_t count, const uint32_t* perm, const aur_ray* rays,
                       uint32_t n, uint32_t* occluder, uint32_t* visits, int nthreads) {
    std::vector<uint64_t> tot((size_t)std::max(1, nthreads), 0);
    parallel_for(n, nthreads, [&](uint32_t i, int w) {
        const Ray ray = rayFrom(rays[i]);
        uint64_t vis = 0;
        const int64_t h = traceAny(V, count, ray, &vis);
        occluder[i] = h >= 0 ? perm[h] : AUR_NO_HIT;
        if (visits) visits[i] = (uint32_t)vis;
        tot[(size_t)w] += vis;
    });
    uint64_t s = 0;
    for (uint64_t x : tot) s += x;
    return s;
}

/*
 * Brute-force closest hit over an ORIGINAL-order soup: the algorithm-
 * independent check of traversal. Same triangle test and acceptance
 * (Epsilon < t < tmax), minimum (t, prim id).
 */
void orc_brute_closest(const float* V, uint32_t count, const aur_ray* rays, uint32_t n, aur_hit* hits,
                       int nthreads) {
    parallel_for(n, nthreads, [&](uint32_t i, int) {
        Ray ray = rayFrom(rays[i]);
        aur_hit out; out.t = rays[i].tmax; out.u = 0.0f; out.v = 0.0f; out.prim = AUR_NO_HIT;
        for (uint32_t k = 0; k < count; ++k) {
            float u, v, t;
            if (intersectTri(ray, V + (size_t)k * 9, u, v, t) && t > kEpsilon && t < ray.t) {
                ray.t = t; out.t = t; out.u = u; out.v = v; out.prim = k;
            }
        }
        hits[i] = out;
    });
}

}  // extern "C"

// ============================================================ integrator
namespace {

struct Scene {
    const float* V;            // NMH-ordered vertices, count*9
    const float* N;            // NMH-ordered normals, count*9
    const uint16_t* S;         // NMH-ordered shader ids (1-based)
    const uint32_t* perm;
    uint32_t count;
    const aur_shader* shaders;
    uint32_t nshaders;
    const aur_light* lights;
    uint32_t nlights;
    const float* TC = nullptr;          // NMH-ordered texcoords, count*6
    const aur_texture* tex = nullptr;
    uint32_t ntex = 0;
    // AUR_MODE_PATH_MIS light-selection table (see orc_mis_table)
    const uint32_t* misTri = nullptr;
    const float* misCdf = nullptr;
    const float* misPa = nullptr;        // per NMH triangle
    uint32_t misCount = 0;
};

// ------------------------------------------------------------ textures
// tex2D with normalised coordinates, wrap addressing, linear filtering and
// cudaReadModeNormalizedFloat on RGBA8 (the reference's texture units,
// texunit.cuh:11-18), restated from the CUDA C++ Programming Guide appendix
// "Texture Fetching": wrap replaces the coordinate by its fractional part;
// xB = frac(u) * width - 0.5, texels floor(xB) and floor(xB) + 1 (wrapped),
// alpha = frac(xB) in fixed point with 8 fractional bits, rounded to nearest;
// result = (1-a)(1-b) T[i,j] + a(1-b) T[i+1,j] + (1-a) b T[i,j+1] + a b T[i+1,j+1]
// in float, with T = byte / 255.
inline float texWeight(float f) { return floorf(f * 256.0f + 0.5f) * (1.0f / 256.0f); }
inline F3 texel(const aur_texture& t, uint32_t i, uint32_t j) {
    const unsigned char* q = t.rgba + ((size_t)j * t.width + i) * 4;
    return mk3((float)q[0] / 255.0f, (float)q[1] / 255.0f, (float)q[2] / 255.0f);
}
inline F3 texFetch(const aur_texture& t, float u, float v) {
    const uint32_t W = t.width, H = t.height;
    float xu = u - floorf(u), xv = v - floorf(v);
    if (!(xu >= 0.0f && xu <= 1.0f)) xu = 0.0f;   // NaN / inf coordinates
    if (!(xv >= 0.0f && xv <= 1.0f)) xv = 0.0f;
    const float xb = xu * (float)W - 0.5f, yb = xv * (float)H - 0.5f;
    const float fi = floorf(xb), fj = floorf(yb);
    const float a = texWeight(xb - fi), b = texWeight(yb - fj);
    const uint32_t i0 = fi < 0.0f ? W - 1 : std::min((uint32_t)fi, W - 1);
    const uint32_t j0 = fj < 0.0f ? H - 1 : std::min((uint32_t)fj, H - 1);
    const uint32_t i1 = i0 + 1 == W ? 0 : i0 + 1, j1 = j0 + 1 == H ? 0 : j0 + 1;
    const F3 t00 = texel(t, i0, j0), t10 = texel(t, i1, j0), t01 = texel(t, i0, j1), t11 = texel(t, i1, j1);
    return t00 * ((1.0f - a) * (1.0f - b)) + t10 * (a * (1.0f - b)) + t01 * ((1.0f - a) * b) + t11 * (a * b);
}
// texfetch (texunit.cuh:54-94): units past the 32 bound return white.
inline F3 texFetchUnit(const Scene& sc, uint32_t id, float u, float v) {
    if (id >= 32u) return mk3(1.0f, 1.0f, 1.0f);
    return texFetch(sc.tex[id], u, v);
}

struct BSDF { F3 N, S, T, color1; };

// kernels/utility.cu:136-167 (per-vertex tangent/bitangent), evaluated at
// shading time from the stored normals.
inline void vertexTB(const F3& n, F3& t, F3& b) {
    const F3 up = mk3(0.0f, 1.0f, 0.0f), fwd = mk3(0.0f, 0.0f, 1.0f);
    t = cross(n, up);
    if (length(t) < kEpsilon) t = cross(n, fwd);
    b = cross(n, t);
}

// kernels/lib/common.cuh:314-327 + shader.cuh:243-262
inline BSDF getBSDF(const Scene& sc, const aur_shader& sh, uint32_t idx, float u, float v) {
    const float* nv = sc.N + (size_t)idx * 9;
    const F3 n1 = mk3(nv[0], nv[1], nv[2]), n2 = mk3(nv[3], nv[4], nv[5]), n3 = mk3(nv[6], nv[7], nv[8]);
    F3 t1, t2, t3, b1, b2, b3;
    vertexTB(n1, t1, b1);
    vertexTB(n2, t2, b2);
    vertexTB(n3, t3, b3);
    BSDF bs;
    bs.N = normalize(bclerp(n1, n2, n3, u, v));
    bs.S = normalize(bclerp(t1, t2, t3, u, v));
    bs.T = normalize(bclerp(b1, b2, b3, u, v));
    if (sh.texture > 0) {
        // raytrace() texture branch (monteCarloRaytracer.cu:37-40), getTexCoord (common.cuh:45-51)
        F3 c = mk3(1.0f, 1.0f, 1.0f);
        if (sh.texture <= 32u) {
            const float* tc = sc.TC + (size_t)idx * 6;
            const float w = 1.0f - u - v;
            const float tu = w * tc[0] + u * tc[2] + v * tc[4];
            const float tv = w * tc[1] + u * tc[3] + v * tc[5];
            c = texFetchUnit(sc, sh.texture - 1, tu, tv);
        }
        bs.color1 = c * sh.diffuse;
    } else {
        bs.color1 = from(sh.diffuse_color) * sh.diffuse;
    }
    return bs;
}

inline F3 bsdfF(const BSDF& b) { return b.color1 * kInvPi; }   // bsdf.cuh:202-210

struct PixelCtx { RngKey key; uint32_t pixel, sample, ray; };

// light.cuh:228-259; the area case draws u1 then u2 from one Philox block.
inline F3 sampleL(const aur_light& L, const PixelCtx* pc, uint32_t slot, Ray& ray, float& pdf) {
    const F3 color = from(L.color);
    switch (L.type) {
    case AUR_LIGHT_AMBIENT:
        ray.dir = from(L.position) - ray.pos;
        ray.t = length(ray.dir);
        ray.dir = ray.dir / ray.t;
        pdf = 1.0f;
        return (color * L.intensity) * (1.0f - L.ambient);
    case AUR_LIGHT_POINT:
        ray.dir = from(L.position) - ray.pos;
        ray.t = length(ray.dir);
        ray.dir = ray.dir / ray.t;
        pdf = 1.0f;
        return (color * L.intensity) / (ray.t * ray.t);
    case AUR_LIGHT_DIRECTIONAL:
        ray.dir = -from(L.direction);
        ray.t = kInfinity;
        pdf = 1.0f;
        return color * L.intensity;
    default: {
        float u1, u2;
        draw2(pc->key, pc->pixel, pc->sample, pc->ray, slot, u1, u2);
        const F3 P = from(L.position) + ((from(L.e1) * u1) + (from(L.e2) * u2));   // sampling.cuh:148-152
        ray.dir = P - ray.pos;
        ray.t = length(ray.dir);
        ray.dir = ray.dir / ray.t;
        pdf = 1.0f / fabsf(dot(from(L.direction), -ray.dir));                       // light.cuh:282-293
        return (color * L.intensity) * fmaxf(0.0f, dot(from(L.direction), -ray.dir));
    }
    }
}

inline Ray pointRay(const F3& p) {
    Ray r; r.pos = p; r.dir = mk3(0.0f); r.t = kInfinity; r.weight = 1.0f; r.eta = 1.0f; r.thr = mk3(1.0f);
    return r;
}

// radiance.cuh:13-16
inline F3 ambientRadiance(const aur_light& L, const BSDF& b) {
    return bsdfF(b) * ((from(L.color) * L.intensity) * L.ambient);
}

// radiance.cuh:18-33 (no offset of the shadow ray)
inline F3 directDelta(const Scene& sc, const aur_light& L, const BSDF& b, const F3& pos, uint64_t* vis) {
    Ray wi = pointRay(pos);
    float pdf;
    const F3 Li = sampleL(L, nullptr, 0, wi, pdf);
    if (pdf > 0.0f && !zero(Li)) {
        const F3 f = bsdfF(b);
        if (!zero(f) && traceAny(sc.V, sc.count, wi, vis) < 0)
            return f * Li * fmaxf(0.0f, dot(wi.dir, b.N));
    }
    return mk3(0.0f);
}

// radiance.cuh:35-80 (light-sampling half; the #if 0 BSDF half stays off)
inline F3 directArea(const Scene& sc, const aur_light& L, uint32_t li, const BSDF& b, const F3& pos,
                     const PixelCtx& pc, uint64_t* vis) {
    F3 acc = mk3(0.0f);
    for (int32_t i = 0; i < L.samples; ++i) {
        F3 Ls = mk3(0.0f);
        Ray wi = pointRay(pos);
        float lightPdf;
        const F3 Li = sampleL(L, &pc, 1u + (li << 16) + (uint32_t)i, wi, lightPdf);
        // Ray::offset (ray.cuh:184-191)
        wi.pos.x += kEpsilon * wi.dir.x;
        wi.pos.y += kEpsilon * wi.dir.y;
        wi.pos.z += kEpsilon * wi.dir.z;
        wi.t += kEpsilon;
        if (lightPdf > 0.0f && !zero(Li)) {
            const F3 f = bsdfF(b);
            if (!zero(f) && traceAny(sc.V, sc.count, wi, vis) < 0)
                Ls = Ls + f * Li * fmaxf(0.0f, dot(wi.dir, b.N));
        }
        acc = acc + Ls;
    }
    const float ns = (float)L.samples;
    return mk3(acc.x / ns, acc.y / ns, acc.z / ns);
}

// ------------------------------------------------------ AUR_MODE_PATH_MIS
// Path mode with physically based direct lighting and multiple importance
// sampling (Veach & Guibas 1995); the half of estimateDirectRadiance the
// reference compiles out (radiance.cuh:55-71). Area lights: the reference's
// emission model Light::L = colour * intensity * max(0, direction . w)
// (light.cuh:18-22), both strategies (a point on the quad, density
// t^2 / (cos_l * area); a BSDF direction traced to the quad, visibleArea,
// light.cuh:62-76), power heuristic (sampling.cuh:162-169) written as
// 1 / (1 + (p_other / p_this)^2). Emissive triangles: one sample per hit from
// the table (probability ~ emission * area, uniform point by the square-root
// parameterisation), weighted against the diffuse bounce's density; emission
// found by a diffuse bounce weighted against the table's. A hit from which no
// diffuse bounce follows gives its emitter sample full weight.
// RNG slots: BSDF half of light li's j-th sample = light slot | 2^31; the
// emitter sample draws at 0xFFFFFFF0 and 0xFFFFFFF1.

const uint32_t kSlotEmitter = 0xFFFFFFF0u;
inline uint32_t bsdfLightSlot(uint32_t li, uint32_t j) { return (1u + (li << 16) + j) | 0x80000000u; }

inline float misWeight(float pThis, float pOther) {
    const float r = pOther / pThis;
    return 1.0f / (1.0f + r * r);
}

// The Lambert density of BSDF::pdf (bsdf.cuh:22-30), |cos| / pi on wo's
// side, the cosine taken against the shading normal in world space.
inline float bsdfPdf(const BSDF& b, const F3& wo, const F3& wi) {
    const float co = dot(wo, b.N), ci = dot(wi, b.N);
    return (co * ci > 0.0f) ? fabsf(ci) * kInvPi : 0.0f;
}

// BSDF::samplef (bsdf.cuh:53-67) in an orthonormal frame about N: the
// tangent made orthogonal to N (Gram-Schmidt), bitangent N x S; the density
// returned is bsdfPdf of the returned direction.
inline F3 bsdfSample(const BSDF& b, const F3& wo, float u1, float u2, float& pdf) {
    F3 S = b.S - b.N * dot(b.N, b.S);
    float l = length(S);
    if (!(l > 1e-6f)) {
        S = fabsf(b.N.x) < 0.9f ? cross(b.N, mk3(1.0f, 0.0f, 0.0f)) : cross(b.N, mk3(0.0f, 1.0f, 0.0f));
        l = length(S);
    }
    S = S / l;
    const F3 T = cross(b.N, S);
    F3 lwi = sampleHemisphereCosine(u1, u2);
    if (dot(wo, b.N) < 0.0f) lwi.z *= -1.0f;
    const F3 wi = localToWorld(lwi, b.N, S, T);
    pdf = bsdfPdf(b, wo, wi);
    return wi;
}

// Distance t > Epsilon from pos along dir to the parallelogram p0 + a e1 + b e2.
inline bool hitQuad(const F3& pos, const F3& dir, const F3& p0, const F3& e1, const F3& e2, float& t) {
    const F3 P = cross(dir, e2);
    const float det = dot(e1, P);
    if (det == 0.0f) return false;
    const float inv = 1.0f / det;
    const F3 T = pos - p0;
    const float a = dot(T, P) * inv;
    if (!(a >= 0.0f && a <= 1.0f)) return false;
    const F3 Q = cross(T, e1);
    const float b = dot(dir, Q) * inv;
    if (!(b >= 0.0f && b <= 1.0f)) return false;
    t = dot(e2, Q) * inv;
    return t > kEpsilon;
}

inline void triVerts(const float* V, uint32_t tri, F3& v1, F3& v2, F3& v3) {
    const float* v = V + (size_t)tri * 9;
    v1 = mk3(v[0], v[3], v[6]);
    v2 = mk3(v[1], v[4], v[7]);
    v3 = mk3(v[2], v[5], v[8]);
}

// Moller-Trumbore's determinant e1 . (dir x e2) (ray.cuh:198-223) and |e1 x e2|.
inline float emitterDet(const F3& v1, const F3& v2, const F3& v3, const F3& dir, float& len) {
    const F3 e1 = v2 - v1, e2 = v3 - v1;
    len = length(cross(e1, e2));
    return dot(e1, cross(dir, e2));
}

inline float emissionWeight(const Scene& sc, uint32_t tri, const F3& dir, float t, float prevPdf) {
    if (!(prevPdf > 0.0f)) return 1.0f;
    const float pa = sc.misPa[tri];
    if (!(pa > 0.0f)) return 1.0f;
    F3 v1, v2, v3;
    triVerts(sc.V, tri, v1, v2, v3);
    float len;
    const float det = emitterDet(v1, v2, v3, dir, len);
    const float epdf = (pa * (t * t)) / (det / len);
    return misWeight(prevPdf, epdf);
}

// A shadow ray from pos, offset by Epsilon along dir (Ray::offset, ray.cuh:184-191).
inline Ray offsetRay(const F3& pos, const F3& dir, float t) {
    Ray r = pointRay(pos);
    r.dir = dir;
    r.pos.x += kEpsilon * dir.x;
    r.pos.y += kEpsilon * dir.y;
    r.pos.z += kEpsilon * dir.z;
    r.t = t;
    return r;
}

inline F3 areaLightMis(const Scene& sc, const aur_light& L, uint32_t li, const BSDF& b, const F3& pos, const F3& wo,
                       const PixelCtx& pc, uint64_t* vis) {
    const F3 p0 = from(L.position), e1 = from(L.e1), e2 = from(L.e2), ldir = from(L.direction);
    const F3 Le0 = from(L.color) * L.intensity;
    const float area = length(cross(e1, e2));
    const F3 f = bsdfF(b);
    F3 acc = mk3(0.0f);
    if (area > 0.0f && !zero(f)) {
        for (int32_t j = 0; j < L.samples; ++j) {
            F3 Ls = mk3(0.0f);
            float u1, u2;
            draw2(pc.key, pc.pixel, pc.sample, pc.ray, 1u + (li << 16) + (uint32_t)j, u1, u2);
            const F3 P = from(L.position) + ((e1 * u1) + (e2 * u2));
            F3 wdir = P - pos;
            const float wt = length(wdir);
            wdir = wdir / wt;
            float cl = dot(ldir, -wdir);
            float cs = fmaxf(0.0f, dot(wdir, b.N));
            if (cl > 0.0f && cs > 0.0f && traceAny(sc.V, sc.count, offsetRay(pos, wdir, wt + kEpsilon), vis) < 0) {
                const float lpdf = (wt * wt) / (cl * area);
                const float w = misWeight(lpdf, bsdfPdf(b, wo, wdir));
                Ls = Ls + f * (Le0 * cl) * ((cs * w) / lpdf);
            }
            draw2(pc.key, pc.pixel, pc.sample, pc.ray, bsdfLightSlot(li, (uint32_t)j), u1, u2);
            float bpdf, tl;
            const F3 wi = bsdfSample(b, wo, u1, u2, bpdf);
            if (bpdf > 0.0f && hitQuad(pos, wi, p0, e1, e2, tl)) {
                cl = dot(ldir, -wi);
                cs = fmaxf(0.0f, dot(wi, b.N));
                if (cl > 0.0f && cs > 0.0f && traceAny(sc.V, sc.count, offsetRay(pos, wi, tl + kEpsilon), vis) < 0) {
                    const float lpdf = (tl * tl) / (cl * area);
                    const float w = misWeight(bpdf, lpdf);
                    Ls = Ls + f * (Le0 * cl) * ((cs * w) / bpdf);
                }
            }
            acc = acc + Ls;
        }
    }
    const float ns = (float)L.samples;
    return mk3(acc.x / ns, acc.y / ns, acc.z / ns);
}

inline F3 emitterSample(const Scene& sc, const BSDF& b, const F3& pos, const F3& wo, bool bounce, const PixelCtx& pc,
                        uint64_t* vis) {
    const F3 f = bsdfF(b);
    if (sc.misCount == 0 || zero(f)) return mk3(0.0f);
    float us, ua, ub, uc;
    draw2(pc.key, pc.pixel, pc.sample, pc.ray, kSlotEmitter, us, ua);
    draw2(pc.key, pc.pixel, pc.sample, pc.ray, kSlotEmitter + 1u, ub, uc);
    // first entry whose CDF value is >= us (the last one if rounding left it below)
    const uint32_t k = (uint32_t)(std::lower_bound(sc.misCdf, sc.misCdf + (sc.misCount - 1), us) - sc.misCdf);
    const uint32_t tri = sc.misTri[k];
    F3 v1, v2, v3;
    triVerts(sc.V, tri, v1, v2, v3);
    const float su = sqrtf(ua);
    const F3 P = ((v1 * (1.0f - su)) + (v2 * (su * (1.0f - ub)))) + (v3 * (su * ub));
    F3 wdir = P - pos;
    const float t = length(wdir);
    if (!(t > kEpsilon)) return mk3(0.0f);
    wdir = wdir / t;
    float len;
    const float det = emitterDet(v1, v2, v3, wdir, len);
    const float cs = fmaxf(0.0f, dot(wdir, b.N));
    if (det < kEpsilon || !(cs > 0.0f)) return mk3(0.0f);
    if (traceAny(sc.V, sc.count, offsetRay(pos, wdir, t * 0.9999f), vis) >= 0) return mk3(0.0f);
    const float epdf = (sc.misPa[tri] * (t * t)) / (det / len);
    const float w = bounce ? misWeight(epdf, bsdfPdf(b, wo, wdir)) : 1.0f;
    const uint32_t sid = sc.S[tri];
    const aur_shader& sh = sc.shaders[sid > 0 ? sid - 1 : 0];
    return f * from(sh.emission_color) * ((cs * w) / epdf);
}

// utility.cu:18-77: camera ray for pixel (x, y), sample s of `samples`.
inline Ray cameraRay(const aur_camera& cam, uint32_t W, uint32_t H, uint32_t x, uint32_t y, uint32_t s,
                     uint32_t samples) {
    F2 pixel;
    if (samples == 1) {
        pixel.x = float(x) / float(W) - 0.5f;
        pixel.y = float(y) / float(H) - 0.5f;
    } else {
        const short sw = (short)sqrtf((float)samples);
        const short sx = (short)(s % (uint32_t)sw), sy = (short)(s / (uint32_t)sw);
        const float dx = 1.0f / float(W), dy = 1.0f / float(H);
        const float sdx = dx / sw, sdy = dy / sw;
        pixel.x = x * dx - 0.5f + (sx * sdx);
        pixel.y = y * dy - 0.5f + (sy * sdy);
    }
    Ray r;
    r.pos = from(cam.position);
    r.t = kInfinity;
    r.weight = 1.0f;
    r.eta = 1.0f;
    r.thr = mk3(1.0f);
    r.dir = normalize(pixel.x * from(cam.right) * cam.tanfov_x + pixel.y * from(cam.up) * cam.tanfov_y +
                      from(cam.forward));
    return r;
}

struct SampleOut { F3 color; bool hit; };

// monteCarloRaytracer.cu:23-113 for one camera ray; mode adds the path bounce.
SampleOut integrate(const Scene& sc, const aur_render_params& p, const Ray& primary, const PixelCtx& pc0,
                    uint64_t* vis) {
    Ray stack[AUR_MAX_DEPTH + 2];
    int sp = 0;
    stack[sp++] = primary;
    int depth = 0;
    F3 color = mk3(0.0f);
    bool anyHit = false;
    uint32_t rayIndex = 0;
    const int maxDepth = (int)p.max_depth;
    const bool mis = p.mode == AUR_MODE_PATH_MIS;
    const bool path = mis || p.mode == AUR_MODE_PATH;
    while (depth <= maxDepth && sp > 0) {
        Ray ray = stack[--sp];
        PixelCtx pc = pc0;
        pc.ray = rayIndex++;
        float u = 0.0f, v = 0.0f;
        const int64_t h = traceClosest(sc.V, sc.count, sc.perm, ray, u, v, vis);
        if (h < 0) continue;
        anyHit = true;
        ++vis[1];   // shading points (vis[0]: node fetches)
        const uint32_t tri = (uint32_t)h;
        const F3 position = ray.pos + (ray.dir * ray.t);
        const F3 wo = -ray.dir;
        const uint32_t sid = sc.S[tri];
        const aur_shader& sh = sc.shaders[sid > 0 ? sid - 1 : 0];   // getSafeID, util/array.h:16-17
        const BSDF b = getBSDF(sc, sh, tri, u, v);
        const bool specular = sh.reflectivity > 0.0f || sh.translucence > 0.0f;
        F3 Li = mis ? from(sh.emission_color) * emissionWeight(sc, tri, ray.dir, ray.t, ray.pdf)
                    : from(sh.emission_color);
        for (uint32_t i = 0; i < sc.nlights; ++i) {
            const aur_light& L = sc.lights[i];
            if (L.type == AUR_LIGHT_AMBIENT) Li = Li + ambientRadiance(L, b);
            if (L.type != AUR_LIGHT_AREA) Li = Li + directDelta(sc, L, b, position, vis);
            else if (mis) Li = Li + areaLightMis(sc, L, i, b, position, wo, pc, vis);
            else Li = Li + directArea(sc, L, i, b, position, pc, vis);
        }
        if (mis) Li = Li + emitterSample(sc, b, position, wo, !specular && depth + 1 <= maxDepth, pc, vis);
        if (specular) depth++;
        if (depth <= maxDepth && sh.reflectivity > 0.0f) {
            Ray nr = pointRay(position);
            nr.dir = reflect(ray.dir, b.N);
            nr.weight = sh.reflectivity;
            nr.eta = ray.eta;
            nr.thr = path ? ray.thr * sh.reflectivity : mk3(nr.weight);
            ray.weight *= (1.0f - sh.reflectivity);
            ray.thr = path ? ray.thr * (1.0f - sh.reflectivity) : mk3(ray.weight);
            stack[sp++] = nr;
        }
        if (depth <= maxDepth && sh.translucence > 0.0f) {
            F3 rN = b.N;
            float etai = ray.eta, etat = sh.refractive_index;
            if (dot(rN, wo) < 0.0f) { rN = -rN; etai = sh.refractive_index; etat = 1.0f; }
            F3 tdir;
            if (refract(tdir, ray.dir, rN, etai, etat)) {
                Ray nr = pointRay(position);
                nr.dir = tdir;
                nr.weight = sh.translucence;
                nr.eta = etat;
                nr.thr = path ? ray.thr * sh.translucence : mk3(nr.weight);
                ray.weight *= (1.0f - sh.translucence);
                ray.thr = path ? ray.thr * (1.0f - sh.translucence) : mk3(ray.weight);
                stack[sp++] = nr;
            }
        }
        if (mis && !specular) {
            depth++;
            if (depth <= maxDepth) {
                float u1, u2, pdf;
                draw2(pc.key, pc.pixel, pc.sample, pc.ray, 0u, u1, u2);
                const F3 wi = bsdfSample(b, wo, u1, u2, pdf);
                const F3 f = bsdfF(b);
                if (pdf > 0.0f && !zero(f)) {
                    Ray nr = pointRay(position);
                    nr.dir = wi;
                    nr.eta = ray.eta;
                    nr.thr = ray.thr * (f * (fabsf(dot(wi, b.N)) / pdf));
                    nr.pdf = pdf;
                    stack[sp++] = nr;
                }
            }
        } else if (path && !specular) {
            depth++;
            if (depth <= maxDepth) {
                // BSDF::samplef (bsdf.cuh:222-236)
                float u1, u2;
                draw2(pc.key, pc.pixel, pc.sample, pc.ray, 0u, u1, u2);
                const F3 lwo = worldToLocal(wo, b.N, b.S, b.T);
                F3 lwi = sampleHemisphereCosine(u1, u2);
                if (lwo.z < 0.0f) lwi.z *= -1.0f;
                const float pdf = (lwo.z * lwi.z > 0.0f) ? fabsf(lwi.z) * kInvPi : 0.0f;
                const F3 f = bsdfF(b);
                const F3 wi = localToWorld(lwi, b.N, b.S, b.T);
                if (pdf > 0.0f && !zero(f)) {
                    Ray nr = pointRay(position);
                    nr.dir = wi;
                    nr.eta = ray.eta;
                    nr.thr = ray.thr * (f * (fabsf(dot(wi, b.N)) / pdf));
                    nr.pdf = pdf;
                    stack[sp++] = nr;
                }
            }
        }
        color = color + Li * ray.thr;
    }
    SampleOut o; o.color = color; o.hit = anyHit;
    return o;
}

}  // namespace

extern "C" {

/* Camera::Camera (util/camera.h:15-28); tanf on the host. */
void orc_camera_make(const float pos[3], const float dir[3], float fovx, float fovy, float aspect,
                     aur_camera* out) {
    const F3 up0 = mk3(0.0f, 1.0f, 0.0f);
    const F3 fwd = normalize(mk3(dir[0], dir[1], dir[2]));
    const F3 right = cross(fwd, up0);
    const F3 up = cross(right, fwd);
    out->position.x = pos[0]; out->position.y = pos[1]; out->position.z = pos[2];
    out->forward.x = fwd.x; out->forward.y = fwd.y; out->forward.z = fwd.z;
    out->right.x = right.x; out->right.y = right.y; out->right.z = right.z;
    out->up.x = up.x; out->up.y = up.y; out->up.z = up.z;
    out->tanfov_x = tanf(fovx);
    out->tanfov_y = tanf(fovy);
    out->aspect = aspect;
}

/* Camera rays for one sample (utility.cu:45-94), reference Ray layout. */
void orc_generate_rays(const aur_camera* cam, uint32_t W, uint32_t H, uint32_t sample, uint32_t samples,
                       aur_path_ray* rays) {
    for (uint32_t y = 0; y < H; ++y)
        for (uint32_t x = 0; x < W; ++x) {
            const Ray r = cameraRay(*cam, W, H, x, y, sample, samples);
            aur_path_ray& o = rays[(size_t)y * W + x];
            o.pos.x = r.pos.x; o.pos.y = r.pos.y; o.pos.z = r.pos.z;
            o.dir.x = r.dir.x; o.dir.y = r.dir.y; o.dir.z = r.dir.z;
            o.t = r.t; o.weight = r.weight; o.eta = r.eta;
        }
}

/*
 * Renders samples [sample_begin, sample_end) of p->spp per pixel and adds
 * them into accum (W*H*4 floats) in sample order, exactly as
 * cudaDrawPixels does (utility.cu:199-219): rgb += color*(1/spp) and
 * alpha += 1/spp for samples whose camera ray hit something.
 * Scene arrays are NMH-ordered (perm: NMH position -> original id).
 * Returns the number of node fetches (closest + any).
 */
static uint64_t render_scene(const Scene& sc, const aur_camera* cam, const aur_render_params* p, float* accum,
                             int nthreads, uint64_t* shading_points = nullptr);

uint64_t orc_render(const float* V, const float* N, const uint16_t* S, const uint32_t* perm, uint32_t count,
                    const aur_shader* shaders, uint32_t nshaders, const aur_light* lights, uint32_t nlights,
                    const aur_camera* cam, const aur_render_params* p, float* accum, int nthreads) {
    Scene sc;
    sc.V = V; sc.N = N; sc.S = S; sc.perm = perm; sc.count = count;
    sc.shaders = shaders; sc.nshaders = nshaders; sc.lights = lights; sc.nlights = nlights;
    return render_scene(sc, cam, p, accum, nthreads);
}

/* orc_render with textures: TC = NMH-ordered texcoords (count*6), tex = the
 * scene's textures. */
uint64_t orc_render_textured(const float* V, const float* N, const uint16_t* S, const uint32_t* perm, uint32_t count,
                             const aur_shader* shaders, uint32_t nshaders, const aur_light* lights, uint32_t nlights,
                             const aur_camera* cam, const aur_render_params* p, float* accum, int nthreads,
                             const float* TC, const aur_texture* tex, uint32_t ntex) {
    Scene sc;
    sc.V = V; sc.N = N; sc.S = S; sc.perm = perm; sc.count = count;
    sc.shaders = shaders; sc.nshaders = nshaders; sc.lights = lights; sc.nlights = nlights;
    sc.TC = TC; sc.tex = tex; sc.ntex = ntex;
    return render_scene(sc, cam, p, accum, nthreads);
}

/* cudaFilterPixelsKernel (kernels/utility.cu:231-252) over the inclusive
 * region (left, right, bottom, top), with the row below clamped to top
 * (the reference clamps it to bottom). in/out: width*height float4. */
void orc_filter_pixels(uint32_t width, const uint32_t* region, const float* in, float* out) {
    const uint32_t L = region[0], R = region[1], B = region[2], T = region[3];
    for (uint32_t y = B; y <= T; ++y)
        for (uint32_t x = L; x <= R; ++x) {
            const uint32_t xl = x > L ? x - 1 : L, xr = x < R ? x + 1 : R;
            const uint32_t yb = y > B ? y - 1 : B, yt = y < T ? y + 1 : T;
            const float* p00 = in + ((size_t)width * yb + xl) * 4; const float* p01 = in + ((size_t)width * yb + x) * 4;
            const float* p02 = in + ((size_t)width * yb + xr) * 4; const float* p10 = in + ((size_t)width * y + xl) * 4;
            const float* p11 = in + ((size_t)width * y + x) * 4;   const float* p12 = in + ((size_t)width * y + xr) * 4;
            const float* p20 = in + ((size_t)width * yt + xl) * 4; const float* p21 = in + ((size_t)width * yt + x) * 4;
            const float* p22 = in + ((size_t)width * yt + xr) * 4;
            float* o = out + ((size_t)width * y + x) * 4;
            for (int c = 0; c < 4; ++c)
                o[c] = p00[c] * 0.0625f + p01[c] * 0.125f + p02[c] * 0.0625f + p10[c] * 0.125f + p11[c] * 0.25f +
                       p12[c] * 0.125f + p20[c] * 0.0625f + p21[c] * 0.125f + p22[c] * 0.0625f;
        }
}

/* cudaCreateEmitters (kernels/emitter.cu:39-119) restated sequentially:
 * triangles of the NMH-ordered soup (V: count*9, S: 1-based shader ids)
 * whose shader has emission > 0, in order; area by Primitive3::area
 * (primitive.cuh:74-85), pdf = 1/area, power = emission colour; the CDF of
 * the emission weights summed in double and normalised, rounded to float.
 * Returns the number of emitters written to out. */
uint32_t orc_emitters(const float* V, const uint16_t* S, uint32_t count, const aur_shader* shaders, aur_emitter* out) {
    uint32_t m = 0;
    std::vector<double> w;
    for (uint32_t i = 0; i < count; ++i) {
        const aur_shader& sh = shaders[S[i] > 0 ? S[i] - 1 : 0];
        if (!(sh.emission > 0.0f)) continue;
        const float* v = V + (size_t)i * 9;
        const F3 v1 = mk3(v[0], v[3], v[6]), v2 = mk3(v[1], v[4], v[7]), v3 = mk3(v[2], v[5], v[8]);
        const F3 va = v1 - v2, vb = v1 - v3, vc = v2 - v3;
        const float a = dot(va, va), b = dot(vb, vb), c = dot(vc, vc);
        aur_emitter e;
        e.area = sqrtf((2 * a * b + 2 * b * c + 2 * c * a - a * a - b * b - c * c) / 16.0f);
        e.pdf = 1.0f / e.area;
        e.cdf = 0.0f;
        e.power = sh.emission_color;
        e.triangle_id = i;
        out[m++] = e;
        w.push_back((double)sh.emission);
    }
    double total = 0.0;
    for (double x : w) total += x;
    double run = 0.0;
    for (uint32_t j = 0; j < m; ++j) {
        run += w[j];
        out[j].cdf = (float)(run / total);
    }
    return m;
}

/* orc_render with everything optional: TC/tex (textures; ntex 0 for none)
 * and the AUR_MODE_PATH_MIS light-selection table (mis_pa per NMH triangle;
 * mis_count 0 for none). */
uint64_t orc_render_ex(const float* V, const float* N, const uint16_t* S, const uint32_t* perm, uint32_t count,
                       const aur_shader* shaders, uint32_t nshaders, const aur_light* lights, uint32_t nlights,
                       const aur_camera* cam, const aur_render_params* p, float* accum, int nthreads, const float* TC,
                       const aur_texture* tex, uint32_t ntex, const uint32_t* mis_tri, const float* mis_cdf,
                       const float* mis_pa, uint32_t mis_count) {
    Scene sc;
    sc.V = V; sc.N = N; sc.S = S; sc.perm = perm; sc.count = count;
    sc.shaders = shaders; sc.nshaders = nshaders; sc.lights = lights; sc.nlights = nlights;
    sc.TC = TC; sc.tex = tex; sc.ntex = ntex;
    sc.misTri = mis_tri; sc.misCdf = mis_cdf; sc.misPa = mis_pa; sc.misCount = mis_count;
    return render_scene(sc, cam, p, accum, nthreads);
}

/* orc_render, also returning the number of shading points (ray hits that
 * were shaded) in *shading_points: the units of the path-sampling roofline
 * (node fetches of the reference algorithm, normals and shader reads per
 * shading point, the accumulation per sample). */
uint64_t orc_render_counted(const float* V, const float* N, const uint16_t* S, const uint32_t* perm, uint32_t count,
                            const aur_shader* shaders, uint32_t nshaders, const aur_light* lights, uint32_t nlights,
                            const aur_camera* cam, const aur_render_params* p, float* accum, int nthreads,
                            uint64_t* shading_points) {
    Scene sc;
    sc.V = V; sc.N = N; sc.S = S; sc.perm = perm; sc.count = count;
    sc.shaders = shaders; sc.nshaders = nshaders; sc.lights = lights; sc.nlights = nlights;
    return render_scene(sc, cam, p, accum, nthreads, shading_points);
}

/* The light-selection table of AUR_MODE_PATH_MIS, sequentially: NMH
 * positions i (V: count*9 NMH-ordered, S: 1-based shader ids) whose shader
 * has emission > 0, whose area 0.5 |(v2 - v1) x (v3 - v1)| is positive and
 * which are not the even-padding copy (perm[i] >= input_count); weights
 * emission * area summed in double, cdf = (float)(running / total);
 * pa[i] = (cdf[k] - cdf[k-1]) / area for the k-th entry, 0 elsewhere.
 * tri and cdf need room for count entries. Returns the number of entries. */
uint32_t orc_mis_table(const float* V, const uint16_t* S, const uint32_t* perm, uint32_t count, uint32_t input_count,
                       const aur_shader* shaders, uint32_t* tri, float* cdf, float* pa) {
    std::vector<double> w;
    std::vector<float> area;
    uint32_t m = 0;
    for (uint32_t i = 0; i < count; ++i) {
        pa[i] = 0.0f;
        const aur_shader& sh = shaders[S[i] > 0 ? S[i] - 1 : 0];
        if (!(sh.emission > 0.0f) || perm[i] >= input_count) continue;
        F3 v1, v2, v3;
        triVerts(V, i, v1, v2, v3);
        const float a = 0.5f * length(cross(v2 - v1, v3 - v1));
        if (!(a > 0.0f)) continue;
        tri[m++] = i;
        w.push_back((double)sh.emission * (double)a);
        area.push_back(a);
    }
    double total = 0.0;
    for (double x : w) total += x;
    double run = 0.0;
    for (uint32_t k = 0; k < m; ++k) {
        run += w[k];
        cdf[k] = (float)(run / total);
    }
    for (uint32_t k = 0; k < m; ++k) pa[tri[k]] = (cdf[k] - (k > 0 ? cdf[k - 1] : 0.0f)) / area[k];
    return m;
}

/* BSDF sampling at hits (NMH-ordered V, N, S; hit i: ray rays8[8i..] =
 * origin, tmax, direction, pad; NMH triangle tri[i] (skipped when < 0);
 * t/u/v tuv[3i..]) with uniforms[2i], [2i+1]: the MIS mode's bsdfSample
 * (mis != 0) or the path-mode bounce; then bsdfPdf of the sampled direction
 * and of probes[3i..]. out, 6 floats per hit: wi.xyz, the sample's pdf,
 * pdf(wo, wi), pdf(wo, probe). */
void orc_bsdf_hits(const float* V, const float* N, const uint16_t* S, uint32_t count, const aur_shader* shaders,
                   uint32_t nshaders, const float* rays8, const int32_t* tri, const float* tuv, uint32_t n,
                   const float* uniforms, const float* probes, int mis, float* out) {
    Scene sc;
    sc.V = V; sc.N = N; sc.S = S; sc.perm = nullptr; sc.count = count;
    sc.shaders = shaders; sc.nshaders = nshaders; sc.lights = nullptr; sc.nlights = 0;
    for (uint32_t i = 0; i < n; ++i) {
        float* o = out + (size_t)i * 6;
        for (int q = 0; q < 6; ++q) o[q] = 0.0f;
        if (tri[i] < 0) continue;
        const float* r = rays8 + (size_t)i * 8;
        const F3 wo = -mk3(r[4], r[5], r[6]);
        const aur_shader& sh = shaders[S[tri[i]] > 0 ? S[tri[i]] - 1 : 0];
        const BSDF b = getBSDF(sc, sh, (uint32_t)tri[i], tuv[3 * i + 1], tuv[3 * i + 2]);
        float pdf;
        F3 wi;
        if (mis) {
            wi = bsdfSample(b, wo, uniforms[2 * i], uniforms[2 * i + 1], pdf);
        } else {   // the path-mode bounce: BSDF::samplef in the reference's frame
            const F3 lwo = worldToLocal(wo, b.N, b.S, b.T);
            F3 lwi = sampleHemisphereCosine(uniforms[2 * i], uniforms[2 * i + 1]);
            if (lwo.z < 0.0f) lwi.z *= -1.0f;
            pdf = (lwo.z * lwi.z > 0.0f) ? fabsf(lwi.z) * kInvPi : 0.0f;
            wi = localToWorld(lwi, b.N, b.S, b.T);
        }
        o[0] = wi.x; o[1] = wi.y; o[2] = wi.z;
        o[3] = pdf;
        o[4] = bsdfPdf(b, wo, wi);
        o[5] = bsdfPdf(b, wo, mk3(probes[3 * i], probes[3 * i + 1], probes[3 * i + 2]));
    }
}

/* The MIS weight of the oracle (and the GPU): 1 / (1 + (b / a)^2). */
float orc_mis_weight(float a, float b) { return misWeight(a, b); }

/* hitQuad against an area light's quad: 1 and the distance, else 0. */
int orc_hit_quad(const aur_light* l, const float* pos, const float* dir, float* t) {
    return hitQuad(mk3(pos[0], pos[1], pos[2]), mk3(dir[0], dir[1], dir[2]), from(l->position), from(l->e1),
                   from(l->e2), *t) ? 1 : 0;
}

/* The two uniforms the integrators draw at one RNG slot (draw2): u1, u2. */
void orc_draw2(uint32_t seed, uint32_t scene, uint32_t pixel, uint32_t sample, uint32_t ray, uint32_t slot,
               float* out2) {
    RngKey k;
    k.seed = seed;
    k.scene = scene;
    draw2(k, pixel, sample, ray, slot, out2[0], out2[1]);
}

/* The texture fetch alone: rgb[3i..] = texFetch(t, uv[2i], uv[2i+1]). */
void orc_texfetch(const aur_texture* t, const float* uv, uint32_t n, float* rgb) {
    for (uint32_t i = 0; i < n; ++i) {
        const F3 c = texFetch(*t, uv[2 * i], uv[2 * i + 1]);
        rgb[3 * i] = c.x; rgb[3 * i + 1] = c.y; rgb[3 * i + 2] = c.z;
    }
}

}  // extern "C"

static uint64_t render_scene(const Scene& sc, const aur_camera* cam, const aur_render_params* p, float* accum,
                             int nthreads, uint64_t* shading_points) {
    const uint32_t W = p->width, H = p->height;
    const uint32_t s0 = p->sample_begin, s1 = p->sample_end ? p->sample_end : p->spp;
    const float weight = 1.0f / (float)p->spp;
    // per worker: node fetches, shading points
    std::vector<uint64_t> tot(2 * (size_t)std::max(1, nthreads), 0);
    parallel_for(W * H, nthreads, [&](uint32_t pix, int w) {
        const uint32_t x = pix % W, y = pix / W;
        float* px = accum + (size_t)pix * 4;
        for (uint32_t s = s0; s < s1; ++s) {
            const Ray r = cameraRay(*cam, W, H, x, y, s, p->spp);
            PixelCtx pc;
            pc.key.seed = p->seed; pc.key.scene = p->scene_id;
            pc.pixel = pix; pc.sample = s; pc.ray = 0;
            const SampleOut o = integrate(sc, *p, r, pc, &tot[2 * (size_t)w]);
            if (o.hit) {
                px[0] += o.color.x * weight;
                px[1] += o.color.y * weight;
                px[2] += o.color.z * weight;
                px[3] += weight;
            }
        }
    });
    uint64_t s = 0, h = 0;
    for (size_t i = 0; i < tot.size(); i += 2) {
        s += tot[i];
        h += tot[i + 1];
    }
    if (shading_points) *shading_points = h;
    return s;
}

extern "C" {

/* cudaTransformKernel (kernels/utility.cu:96-124) with Transform::getPoint /
 * getNormal (kernels/lib/transform.cuh:8-24): triangle i uses the LAST object
 * in array order whose offset <= i (a linear scan, as the reference does);
 * triangles before every object are left untouched. */
void orc_transform(const float* sv, const float* sn, uint32_t count, const aur_object_transform* xf, uint32_t nobj,
                   float* dv, float* dn) {
    for (uint32_t i = 0; i < count; ++i) {
        const aur_object_transform* t = nullptr;
        for (uint32_t k = 0; k < nobj; ++k)
            if (xf[k].offset <= i) t = &xf[k];
        if (!t) continue;
        const float(*m)[4] = t->world_matrix;
        const float(*q)[4] = t->normal_matrix;
        for (int c = 0; c < 3; ++c) {
            const float px = sv[(size_t)i * 9 + c], py = sv[(size_t)i * 9 + 3 + c], pz = sv[(size_t)i * 9 + 6 + c];
            dv[(size_t)i * 9 + c] = m[0][0] * px + m[1][0] * py + m[2][0] * pz + m[3][0];
            dv[(size_t)i * 9 + 3 + c] = m[0][1] * px + m[1][1] * py + m[2][1] * pz + m[3][1];
            dv[(size_t)i * 9 + 6 + c] = m[0][2] * px + m[1][2] * py + m[2][2] * pz + m[3][2];
            const float nx = sn[(size_t)i * 9 + 3 * c], ny = sn[(size_t)i * 9 + 3 * c + 1], nz = sn[(size_t)i * 9 + 3 * c + 2];
            dn[(size_t)i * 9 + 3 * c] = q[0][0] * nx + q[1][0] * ny + q[2][0] * nz;
            dn[(size_t)i * 9 + 3 * c + 1] = q[0][1] * nx + q[1][1] * ny + q[2][1] * nz;
            dn[(size_t)i * 9 + 3 * c + 2] = q[0][2] * nx + q[1][2] * ny + q[2][2] * nz;
        }
    }
}

/* cudaGenerateTBKernel (kernels/utility.cu:136-167). */
void orc_generate_tb(const float* nrm, uint32_t count, float* tan, float* bit) {
    for (uint32_t i = 0; i < (size_t)count * 3; ++i) {
        F3 t, b;
        vertexTB(mk3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]), t, b);
        tan[3 * i] = t.x; tan[3 * i + 1] = t.y; tan[3 * i + 2] = t.z;
        bit[3 * i] = b.x; bit[3 * i + 1] = b.y; bit[3 * i + 2] = b.z;
    }
}

}  // extern "C"
