// aur_traverse.cuh — NMH traversal as a device function, shared by the
// batched trace kernels and the integrators.
//
// intersect() / intersectAny() (kernels/lib/intersect.cuh:36-152): depth
// first, near child first by the sign of the ray direction on the child's
// axis, range clipped cumulatively by each node's slab (ray.cuh:225-237),
// Moller-Trumbore with culling (ray.cuh:198-223), hits need
// Epsilon < t < best. Closest-hit ties in t go to the lower original prim id.
// Node k occupies recs[5k .. 5k+4]: (slab_lo, slab_hi, tri0.v1.xy),
// (tri0.v1.z, tri0.e1), (tri0.e2, tri1.v1.x), (tri1.v1.yz, tri1.e1.xy),
// (tri1.e1.z, tri1.e2). Children of node k are 2k+1, 2k+2; the axis of a node
// is its level mod 3 and rides in the top two bits of stack entries.
#pragma once

#include "aur_math.cuh"

namespace aur {

constexpr uint32_t kNoPrim = 0xFFFFFFFFu;

// A per-thread stack column in shared memory: entry e of thread t lives at
// [e * stride + t] of three arrays.
struct StackRef {
    uint32_t* idx;
    float* lo;
    float* hi;
    int stride;
    int cap;
};

__device__ __forceinline__ float sel3(uint32_t a, float x, float y, float z) { return a == 0 ? x : (a == 1 ? y : z); }

// Returns the NMH position of the hit (kNoPrim on a miss). For closest hit,
// best_t/bu/bv are updated; for any hit, best_t is the ray's tmax (read only).
template <bool kAny>
__device__ __forceinline__ uint32_t traverse(const float4* __restrict__ recs, uint32_t nodes,
                                             const uint32_t* __restrict__ perm, const f3& pos, const f3& dir,
                                             float& best_t, float& bu, float& bv, const StackRef& stk,
                                             uint32_t& visits, uint32_t* __restrict__ err) {
    uint32_t best = kNoPrim;
    uint32_t k = 0, a = 0;
    float lo = kEpsilon, hi = kInfinity;
    int sp = 0;
    for (;;) {
        bool descend = false;
        if (k < nodes) {
            ++visits;
            const float4 q0 = __ldg(recs + (size_t)k * 5);
            const float p = sel3(a, pos.x, pos.y, pos.z);
            const float d = sel3(a, dir.x, dir.y, dir.z);
            const float d0 = (q0.x - p) / d;
            const float d1 = (q0.y - p) / d;
            const float nlo = fmaxf(fminf(d0, d1), lo);
            const float nhi = fminf(fmaxf(d0, d1), hi);
            if (nlo <= nhi && nlo <= best_t) {
                const float4 q1 = __ldg(recs + (size_t)k * 5 + 1);
                const float4 q2 = __ldg(recs + (size_t)k * 5 + 2);
                const float4 q3 = __ldg(recs + (size_t)k * 5 + 3);
                const float4 q4 = __ldg(recs + (size_t)k * 5 + 4);
                float u, v, t;
                if (intersect_tri(pos, dir, mk3(q0.z, q0.w, q1.x), mk3(q1.y, q1.z, q1.w), mk3(q2.x, q2.y, q2.z), u, v,
                                  t) &&
                    t > kEpsilon) {
                    const uint32_t idx = 2 * k;
                    if (kAny) {
                        if (t < best_t) return idx;
                    } else if (t < best_t || (t == best_t && best != kNoPrim && perm[idx] < perm[best])) {
                        best_t = t; bu = u; bv = v; best = idx;
                    }
                }
                if (intersect_tri(pos, dir, mk3(q2.w, q3.x, q3.y), mk3(q3.z, q3.w, q4.x), mk3(q4.y, q4.z, q4.w), u, v,
                                  t) &&
                    t > kEpsilon) {
                    const uint32_t idx = 2 * k + 1;
                    if (kAny) {
                        if (t < best_t) return idx;
                    } else if (t < best_t || (t == best_t && best != kNoPrim && perm[idx] < perm[best])) {
                        best_t = t; bu = u; bv = v; best = idx;
                    }
                }
                const uint32_t na = a == 2 ? 0 : a + 1;
                const bool neg = sel3(na, dir.x, dir.y, dir.z) < 0.0f;
                const uint32_t near = neg ? 2 * k + 2 : 2 * k + 1;
                const uint32_t far = neg ? 2 * k + 1 : 2 * k + 2;
                if (sp < stk.cap) {
                    stk.idx[sp * stk.stride] = far | (na << 30);
                    stk.lo[sp * stk.stride] = nlo;
                    stk.hi[sp * stk.stride] = nhi;
                    ++sp;
                } else {
                    atomicOr(err, 1u);  // unreachable below 2^30 triangles: the stack holds one entry per level
                }
                k = near;
                a = na;
                lo = nlo;
                hi = nhi;
                descend = true;
            }
        }
        if (!descend) {
            if (sp == 0) break;
            --sp;
            const uint32_t e = stk.idx[sp * stk.stride];
            k = e & 0x3FFFFFFFu;
            a = e >> 30;
            lo = stk.lo[sp * stk.stride];
            hi = stk.hi[sp * stk.stride];
        }
    }
    return best;
}

}  // namespace aur
