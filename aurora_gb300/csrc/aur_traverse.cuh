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
// is its level mod 3.
#pragma once

#include "aur_math.cuh"

namespace aur {

constexpr uint32_t kNoPrim = 0xFFFFFFFFu;

// Per-thread storage of pending far-child ranges, one (lo, hi) pair per heap
// level, in shared memory: level L of thread t lives at [L * stride] of the
// two arrays (pointers already offset by t).
struct StackRef {
    float* lo;
    float* hi;
    int stride;
    int cap;   // levels + 1
};

__device__ __forceinline__ float sel3(uint32_t a, float x, float y, float z) { return a == 0 ? x : (a == 1 ? y : z); }

// Traversal state of one ray. The heap is implicit, so a pending far child
// needs no stored index: it is the sibling of the current node's ancestor on
// the far child's level, ((k+1) >> (lvl - L) ^ 1) - 1 in 0-based heap
// numbering. `trail` has bit L set while a far child waits on level L; its
// clipped range sits at stk[L]. Depth-first, near child first: the visit
// order of intersect() exactly.
struct TravState {
    uint32_t k, lvl, a, trail;
    float lo, hi;
};

__device__ __forceinline__ void trav_init(TravState& s) {
    s.k = 0; s.lvl = 0; s.a = 0; s.trail = 0;
    s.lo = kEpsilon; s.hi = kInfinity;
}

// Advances to the next node whose slab the ray crosses (slab test of
// ray.cuh:225-237 with the cumulative range). Returns false when the
// traversal is exhausted; otherwise q0 holds the node's first record word and
// nlo/nhi its clipped range.
__device__ __forceinline__ bool trav_next(TravState& s, const float4* __restrict__ recs, uint32_t nodes, const f3& pos,
                                          const f3& dir, float best_t, const StackRef& stk, float4& q0, float& nlo,
                                          float& nhi, uint32_t& visits) {
    for (;;) {
        if (s.k < nodes) {
            ++visits;
            q0 = __ldg(recs + (size_t)s.k * 5);
            const float p = sel3(s.a, pos.x, pos.y, pos.z);
            const float d = sel3(s.a, dir.x, dir.y, dir.z);
            const float d0 = (q0.x - p) / d;
            const float d1 = (q0.y - p) / d;
            nlo = fmaxf(fminf(d0, d1), s.lo);
            nhi = fminf(fmaxf(d0, d1), s.hi);
            if (nlo <= nhi && nlo <= best_t) return true;
        }
        if (s.trail == 0) return false;
        const uint32_t L = 31u - (uint32_t)__clz(s.trail);
        s.trail &= ~(1u << L);
        s.k = (((s.k + 1u) >> (s.lvl - L)) ^ 1u) - 1u;
        s.lvl = L;
        s.a = L % 3u;
        s.lo = stk.lo[L * stk.stride];
        s.hi = stk.hi[L * stk.stride];
    }
}

// Descends from the current node (whose slab was crossed) to its near child,
// leaving the far child pending on the child level.
__device__ __forceinline__ void trav_descend(TravState& s, const f3& dir, uint32_t nodes, const StackRef& stk, float nlo,
                                             float nhi) {
    const uint32_t na = s.a == 2 ? 0 : s.a + 1;
    const bool neg = sel3(na, dir.x, dir.y, dir.z) < 0.0f;
    const uint32_t near = neg ? 2 * s.k + 2 : 2 * s.k + 1;
    const uint32_t far = neg ? 2 * s.k + 1 : 2 * s.k + 2;
    const uint32_t L = s.lvl + 1;
    if (far < nodes) {
        stk.lo[L * stk.stride] = nlo;
        stk.hi[L * stk.stride] = nhi;
        s.trail |= 1u << L;
    }
    s.k = near;
    s.lvl = L;
    s.a = na;
    s.lo = nlo;
    s.hi = nhi;
}

// Tests the two triangles of node k (Moller-Trumbore with culling,
// ray.cuh:198-223) in order. Closest hit: ties in t go to the lower original
// prim id. Any hit: returns true on the first hit with Epsilon < t < best_t.
template <bool kAny>
__device__ __forceinline__ bool node_triangles(const float4* __restrict__ recs, uint32_t k, const float4& q0,
                                               const uint32_t* __restrict__ perm, const f3& pos, const f3& dir,
                                               float& best_t, float& bu, float& bv, uint32_t& best) {
    const float4 q1 = __ldg(recs + (size_t)k * 5 + 1);
    const float4 q2 = __ldg(recs + (size_t)k * 5 + 2);
    const float4 q3 = __ldg(recs + (size_t)k * 5 + 3);
    const float4 q4 = __ldg(recs + (size_t)k * 5 + 4);
    float u, v, t;
    if (intersect_tri(pos, dir, mk3(q0.z, q0.w, q1.x), mk3(q1.y, q1.z, q1.w), mk3(q2.x, q2.y, q2.z), u, v, t) &&
        t > kEpsilon) {
        const uint32_t idx = 2 * k;
        if (kAny) {
            if (t < best_t) { best = idx; return true; }
        } else if (t < best_t || (t == best_t && best != kNoPrim && perm[idx] < perm[best])) {
            best_t = t; bu = u; bv = v; best = idx;
        }
    }
    if (intersect_tri(pos, dir, mk3(q2.w, q3.x, q3.y), mk3(q3.z, q3.w, q4.x), mk3(q4.y, q4.z, q4.w), u, v, t) &&
        t > kEpsilon) {
        const uint32_t idx = 2 * k + 1;
        if (kAny) {
            if (t < best_t) { best = idx; return true; }
        } else if (t < best_t || (t == best_t && best != kNoPrim && perm[idx] < perm[best])) {
            best_t = t; bu = u; bv = v; best = idx;
        }
    }
    return false;
}

// Returns the NMH position of the hit (kNoPrim on a miss). For closest hit,
// best_t/bu/bv are updated; for any hit, best_t is the ray's tmax (read only).
// Structure: advance to the next crossed node (cheap, divergent), then test
// its triangles with the lanes that got there together ("while-while",
// Aila & Laine, HPG'09).
template <bool kAny>
__device__ __forceinline__ uint32_t traverse(const float4* __restrict__ recs, uint32_t nodes,
                                             const uint32_t* __restrict__ perm, const f3& pos, const f3& dir,
                                             float& best_t, float& bu, float& bv, const StackRef& stk,
                                             uint32_t& visits, uint32_t* __restrict__ err) {
    (void)err;
    uint32_t best = kNoPrim;
    TravState s;
    trav_init(s);
    float4 q0;
    float nlo, nhi;
    while (trav_next(s, recs, nodes, pos, dir, best_t, stk, q0, nlo, nhi, visits)) {
        if (node_triangles<kAny>(recs, s.k, q0, perm, pos, dir, best_t, bu, bv, best)) return best;
        trav_descend(s, dir, nodes, stk, nlo, nhi);
    }
    return best;
}

}  // namespace aur
