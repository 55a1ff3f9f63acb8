// aur_traverse.cuh — NMH traversal as a device function, shared by the
// batched trace kernels and the integrators.
//
// intersect() / intersectAny() (kernels/lib/intersect.cuh:36-152): depth
// first, near child first by the sign of the ray direction on the child's
// axis, range clipped cumulatively by each node's slab (ray.cuh:225-237),
// Moller-Trumbore with culling (ray.cuh:198-223), hits need
// Epsilon < t < best. Closest-hit ties in t go to the lower original prim id.
//
// Node k occupies the 128-byte record recs[8k .. 8k+7]:
//   [0] (slab_lo, slab_hi, tri0.v1.xy)   [1] (tri0.v1.z, tri0.e1)
//   [2] (tri0.e2, tri1.v1.x)             [3] (tri1.v1.yz, tri1.e1.xy)
//   [4] (tri1.e1.z, tri1.e2)
//   [5..7] padded subtree boxes of the children 2k+1 and 2k+2:
//          (c1.lo.xyz, c1.hi.x), (c1.hi.yz, c2.lo.xy), (c2.lo.z, c2.hi.xyz)
// The axis of a node is its level mod 3.
//
// Subtree-box pruning: before descending, each child's box is tested against
// the ray over (0, best t]; a child whose box the ray misses is neither
// fetched nor pushed. The boxes are padded (relative 1e-5 in space, 1e-4 in
// t) well beyond float rounding of both the box test and the triangle test,
// so a pruned subtree holds no triangle the unpruned traversal would accept:
// visit order, slab arithmetic and every accepted hit stay those of
// intersect(), only subtrees without an acceptable hit are skipped.
#pragma once

#include "aur_math.cuh"

namespace aur {

constexpr uint32_t kNoPrim = 0xFFFFFFFFu;
constexpr uint32_t kRecStride = 8;          // float4 per node record
// Set on TravState::k when the current node was pruned by its box: the node
// is not fetched, but its heap position still locates the pending far nodes.
constexpr uint32_t kSkipBit = 0x80000000u;
constexpr float kBoxNear = 0.9999f, kBoxFar = 1.0001f;

// Reciprocal direction for box tests; zero components become +-1e-30 so that
// no 0 * inf product (NaN) can occur.
__device__ __forceinline__ f3 box_inv(const f3& d) {
    return mk3(1.0f / copysignf(fmaxf(fabsf(d.x), 1e-30f), d.x), 1.0f / copysignf(fmaxf(fabsf(d.y), 1e-30f), d.y),
               1.0f / copysignf(fmaxf(fabsf(d.z), 1e-30f), d.z));
}

// The two slab distances (a0 / d, a1 / d) of the slab test (ray.cuh:225-237),
// equal bit for bit to the IEEE divisions. y is the ray's box reciprocal on
// the axis, which is RN(1/d) whenever |d| >= 1e-30 (box_inv). With
// y = RN(1/d), q = RN(a * y) is within an ulp of a / d, the remainder
// a - q * d is exact in one fused multiply-add, and RN(q + remainder * y) is
// the correctly rounded quotient (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990), provided nothing overflows or underflows: that holds when |y| is in
// [2^-40, 2^40] and the quotient's magnitude is in [2^-59, 2^100], which
// bounds |a| to [2^-100, 2^140]. Anything else (a zero or NaN quotient, a
// tiny or huge one, a near axis-parallel ray) takes the IEEE division.
// Checked against IEEE division on 6e8 pairs spanning subnormal to
// near-overflow numerators, and by the traversal parity tests.
__device__ __forceinline__ void slab_div(float a0, float a1, float d, float y, float& q0, float& q1) {
    float f0 = a0 * y, f1 = a1 * y;
    f0 = __fmaf_rn(__fmaf_rn(-f0, d, a0), y, f0);
    f1 = __fmaf_rn(__fmaf_rn(-f1, d, a1), y, f1);
    const float my = fabsf(y), m0 = fabsf(f0), m1 = fabsf(f1);
    if (my >= 0x1p-40f && my <= 0x1p40f && m0 >= 0x1p-59f && m0 <= 0x1p100f && m1 >= 0x1p-59f &&
        m1 <= 0x1p100f) {
        q0 = f0;
        q1 = f1;
    } else {
        q0 = a0 / d;
        q1 = a1 / d;
    }
}

// Conservative ray/box overlap over (0, tlimit]. poi = pos * inv per axis, so
// each slab distance is one fused multiply-add, (lo * inv - poi); its
// rounding, like that of (lo - pos) * inv, is far inside the box padding and
// the t margins, and a NaN (an overflowing poi with a 1e-30 component) can
// only drop an axis from the test, never prune.
__device__ __forceinline__ bool box_hit(float lx, float ly, float lz, float hx, float hy, float hz, const f3& poi,
                                        const f3& inv, float tlimit) {
    const float x0 = __fmaf_rn(lx, inv.x, -poi.x), x1 = __fmaf_rn(hx, inv.x, -poi.x);
    const float y0 = __fmaf_rn(ly, inv.y, -poi.y), y1 = __fmaf_rn(hy, inv.y, -poi.y);
    const float z0 = __fmaf_rn(lz, inv.z, -poi.z), z1 = __fmaf_rn(hz, inv.z, -poi.z);
    const float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), 0.0f));
    const float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tlimit));
    return tn * kBoxNear <= tf * kBoxFar;
}

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

// One 32-byte sector of a node record, read by a single 256-bit load
// (ld.global.nc.v8.f32; records are 128-byte aligned): half as many L1
// accesses per node as 16-byte loads, and the L1 data pipe is what bounds the
// traversal.
struct Sector {
    float4 a, b;
};
__device__ __forceinline__ Sector ld_sector(const float4* __restrict__ p) {
    Sector s;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(s.a.x), "=f"(s.a.y), "=f"(s.a.z), "=f"(s.a.w), "=f"(s.b.x), "=f"(s.b.y), "=f"(s.b.z), "=f"(s.b.w)
        : "l"(p));
    return s;
}

// The same sector through the texture path: two float4 texels of the records
// bound as a linear texture (texel index = float4 index in the records).
__device__ __forceinline__ Sector tex_sector(cudaTextureObject_t tex, size_t texel) {
    Sector s;
    s.a = tex1Dfetch<float4>(tex, (int)texel);
    s.b = tex1Dfetch<float4>(tex, (int)texel + 1);
    return s;
}

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
// traversal is exhausted; otherwise s0 holds the node's first record sector
// (words 0 and 1) and nlo/nhi its clipped range.
__device__ __forceinline__ bool trav_next(TravState& s, const float4* __restrict__ recs, uint32_t nodes, const f3& pos,
                                          const f3& dir, const f3& inv, float best_t, const StackRef& stk, Sector& s0,
                                          float& nlo, float& nhi, uint32_t& visits) {
    for (;;) {
        if (s.k < nodes) {
            ++visits;
            s0 = ld_sector(recs + (size_t)s.k * kRecStride);
            const float4& q0 = s0.a;
            const float p = sel3(s.a, pos.x, pos.y, pos.z);
            const float d = sel3(s.a, dir.x, dir.y, dir.z);
            float d0, d1;
            slab_div(q0.x - p, q0.y - p, d, sel3(s.a, inv.x, inv.y, inv.z), d0, d1);
            nlo = fmaxf(fminf(d0, d1), s.lo);
            nhi = fminf(fmaxf(d0, d1), s.hi);
            if (nlo <= nhi && nlo <= best_t) return true;
        }
        if (s.trail == 0) return false;
        const uint32_t L = 31u - (uint32_t)__clz(s.trail);
        s.trail &= ~(1u << L);
        s.k = ((((s.k & ~kSkipBit) + 1u) >> (s.lvl - L)) ^ 1u) - 1u;
        s.lvl = L;
        s.a = L % 3u;
        s.lo = stk.lo[L * stk.stride];
        s.hi = stk.hi[L * stk.stride];
    }
}

// Descends from the current node (whose slab was crossed) to its near child,
// leaving the far child pending on the child level. With kBoxes, children
// whose subtree box the ray misses within (0, tlimit] are dropped.
// q5 is record word 5 (first child's box lo.xyz, hi.x), already read with
// the triangles; words 6 and 7 are read here.
template <bool kBoxes = true>
__device__ __forceinline__ void trav_descend(TravState& s, const float4* __restrict__ recs, const float4& q5,
                                             const f3& pos, const f3& dir, const f3& inv, float tlimit,
                                             uint32_t nodes, const StackRef& stk, float nlo, float nhi) {
    const uint32_t na = s.a == 2 ? 0 : s.a + 1;
    const bool neg = sel3(na, dir.x, dir.y, dir.z) < 0.0f;
    const uint32_t c1 = 2 * s.k + 1;
    bool h1 = c1 < nodes, h2 = c1 + 1 < nodes;
    if (kBoxes && h1) {
        const Sector s3 = ld_sector(recs + (size_t)s.k * kRecStride + 6);
        const f3 poi = mk3(pos.x * inv.x, pos.y * inv.y, pos.z * inv.z);
        const float4& b1 = s3.a;
        const float4& b2 = s3.b;
        h1 = box_hit(q5.x, q5.y, q5.z, q5.w, b1.x, b1.y, poi, inv, tlimit);
        if (h2) h2 = box_hit(b1.z, b1.w, b2.x, b2.y, b2.z, b2.w, poi, inv, tlimit);
    }
    const bool near_ok = neg ? h2 : h1;
    const bool far_ok = neg ? h1 : h2;
    const uint32_t L = s.lvl + 1;
    if (far_ok) {
        stk.lo[L * stk.stride] = nlo;
        stk.hi[L * stk.stride] = nhi;
        s.trail |= 1u << L;
    }
    s.k = (neg ? c1 + 1 : c1) | (near_ok ? 0u : kSkipBit);
    s.lvl = L;
    s.a = na;
    s.lo = nlo;
    s.hi = nhi;
}

// Tests the two triangles of node k (Moller-Trumbore with culling,
// ray.cuh:198-223) in order. Closest hit: ties in t go to the lower original
// prim id. Any hit: returns true on the first hit with Epsilon < t < best_t.
// s0: record sector 0 (from trav_next); sectors 1 and 2 are read here, and
// word 5 (the tail of sector 2) is handed back in q5 for trav_descend. With
// kTex, sector 2 comes through the texture path (tex: the records as float4
// texels): with one of a node's four sectors there, the L1 load pipe, which
// bounds the traversal, and the texture pipe share the node's reads (+2.3 %
// on the traversal microbench; more sectors there, or others, measured slower).
template <bool kAny, bool kTex = false>
__device__ __forceinline__ bool node_triangles(const float4* __restrict__ recs, uint32_t k, const Sector& s0,
                                               const uint32_t* __restrict__ perm, const f3& pos, const f3& dir,
                                               float& best_t, float& bu, float& bv, uint32_t& best, float4& q5,
                                               cudaTextureObject_t tex = 0) {
    const Sector s1 = ld_sector(recs + (size_t)k * kRecStride + 2);
    const Sector s2 = kTex ? tex_sector(tex, (size_t)k * kRecStride + 4) : ld_sector(recs + (size_t)k * kRecStride + 4);
    const float4& q0 = s0.a;
    const float4& q1 = s0.b;
    const float4& q2 = s1.a;
    const float4& q3 = s1.b;
    const float4& q4 = s2.a;
    q5 = s2.b;
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
    const f3 inv = box_inv(dir);
    TravState s;
    trav_init(s);
    Sector s0;
    float4 q5;
    float nlo, nhi;
    while (trav_next(s, recs, nodes, pos, dir, inv, best_t, stk, s0, nlo, nhi, visits)) {
        if (node_triangles<kAny>(recs, s.k, s0, perm, pos, dir, best_t, bu, bv, best, q5)) return best;
        trav_descend(s, recs, q5, pos, dir, inv, best_t, nodes, stk, nlo, nhi);
    }
    return best;
}

// ------------------------------------------------------------ warp packets
// The 3-bit direction octant of a ray (bit a: dir[a] < 0, the comparison
// that picks the near child).
__device__ __forceinline__ uint32_t dir_octant(const f3& dir) {
    return (dir.x < 0.0f ? 1u : 0u) | (dir.y < 0.0f ? 2u : 0u) | (dir.z < 0.0f ? 4u : 0u);
}

// Largest side of the box around the valid lanes' ray origins (call with
// all 32 lanes). A packet pays for the union of its lanes' nodes, so it is
// only worth taking when the rays start close together (a camera's, or
// neighbouring points toward one light); this is that test's measure.
__device__ __forceinline__ float warp_origin_span(const f3& pos, bool valid) {
    float lx = valid ? pos.x : INFINITY, ly = valid ? pos.y : INFINITY, lz = valid ? pos.z : INFINITY;
    float hx = valid ? pos.x : -INFINITY, hy = valid ? pos.y : -INFINITY, hz = valid ? pos.z : -INFINITY;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
        ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
        lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
        hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
        hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
    }
    return fmaxf(fmaxf(hx - lx, hy - ly), hz - lz);
}

// All 32 lanes of a warp traverse together, one node at a time: the node
// sequence (k, level, axis) is the warp's, each lane keeps its own range,
// best hit and pending far children, and takes part in a node only where
// its own traversal would visit it. The rays must share their direction
// octant (`oct`): then every node's near child is the same for all lanes,
// the warp walks the depth-first, near-first order of intersect() over the
// union of the lanes' nodes, and each lane meets its own nodes in its own
// order with its own decisions (slab range, prune by best t, child boxes):
// its result is that of `traverse`, bit for bit. Node records are read at
// one address per warp (one L1 wavefront instead of one per lane), and
// lanes of coherent rays share most of their nodes. `valid`: the lane has a
// ray (false lanes never take part). Call with all 32 lanes.
template <bool kAny>
__device__ __forceinline__ uint32_t traverse_packet(const float4* __restrict__ recs, uint32_t nodes,
                                                    const uint32_t* __restrict__ perm, bool valid, uint32_t oct,
                                                    const f3& pos, const f3& dir, float& best_t, float& bu,
                                                    float& bv, const StackRef& stk) {
    const f3 inv = box_inv(dir);
    uint32_t best = kNoPrim;
    uint32_t k = 0, lvl = 0, ax = 0;   // the warp's node
    uint32_t trail = 0;                // this lane's pending far children, bit per level
    bool act = valid;                  // this lane visits node k
    float lo = kEpsilon, hi = kInfinity;
    for (;;) {
        if (__any_sync(0xffffffffu, act) && k < nodes) {
            const Sector s0 = ld_sector(recs + (size_t)k * kRecStride);
            bool crossed = false;
            float nlo = 0.0f, nhi = 0.0f;
            if (act) {
                const float p = sel3(ax, pos.x, pos.y, pos.z);
                const float d = sel3(ax, dir.x, dir.y, dir.z);
                float d0, d1;
                slab_div(s0.a.x - p, s0.a.y - p, d, sel3(ax, inv.x, inv.y, inv.z), d0, d1);
                nlo = fmaxf(fminf(d0, d1), lo);
                nhi = fminf(fmaxf(d0, d1), hi);
                crossed = nlo <= nhi && nlo <= best_t;
            }
            float4 q5 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (crossed && node_triangles<kAny>(recs, k, s0, perm, pos, dir, best_t, bu, bv, best, q5)) {
                crossed = false;   // any hit: this lane is done
                trail = 0;
            }
            const uint32_t c1 = 2 * k + 1;
            if (__any_sync(0xffffffffu, crossed) && c1 < nodes) {
                bool h1 = false, h2 = false;
                if (crossed) {
                    const Sector s3 = ld_sector(recs + (size_t)k * kRecStride + 6);
                    const f3 poi = mk3(pos.x * inv.x, pos.y * inv.y, pos.z * inv.z);
                    h1 = box_hit(q5.x, q5.y, q5.z, q5.w, s3.a.x, s3.a.y, poi, inv, best_t);
                    if (c1 + 1 < nodes)
                        h2 = box_hit(s3.a.z, s3.a.w, s3.b.x, s3.b.y, s3.b.z, s3.b.w, poi, inv, best_t);
                }
                const uint32_t na = ax == 2 ? 0 : ax + 1;
                const bool neg = (oct >> na) & 1u;
                const bool near_ok = neg ? h2 : h1;
                const bool far_ok = neg ? h1 : h2;
                const uint32_t L = lvl + 1;
                if (far_ok) {
                    stk.lo[L * stk.stride] = nlo;
                    stk.hi[L * stk.stride] = nhi;
                    trail |= 1u << L;
                }
                if (near_ok) { lo = nlo; hi = nhi; }
                act = near_ok;
                k = neg ? c1 + 1 : c1;
                lvl = L;
                ax = na;
                if (__any_sync(0xffffffffu, act)) continue;
            }
        }
        // Next: the deepest level where some lane has a pending far child
        // (the sibling of the warp's ancestor on that level).
        const uint32_t wt = __reduce_or_sync(0xffffffffu, trail);
        if (wt == 0) break;
        const uint32_t L = 31u - (uint32_t)__clz(wt);
        k = (((k + 1u) >> (lvl - L)) ^ 1u) - 1u;
        lvl = L;
        ax = L % 3u;
        act = (trail >> L) & 1u;
        if (act) {
            trail &= ~(1u << L);
            lo = stk.lo[L * stk.stride];
            hi = stk.hi[L * stk.stride];
        }
    }
    return best;
}

}  // namespace aur
