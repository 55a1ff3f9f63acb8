// trace.cu — closest-hit and any-hit traversal of the NMH pair-heap.
//
// Same visit order and arithmetic as intersect() / intersectAny()
// (kernels/lib/intersect.cuh:36-152): depth-first, near child first by the
// sign of the ray direction on the child's axis, range clipped cumulatively
// by each node's slab (ray.cuh:225-237), Moller-Trumbore with culling
// (ray.cuh:198-223). The node of the reference is 72 scattered bytes read
// with 24 scalar loads; here it is a 128-byte record (slab, two triangles as
// v1, e1, e2, and the subtree boxes of both children) read as one 16-byte
// load for the slab test, four more only when the slab is hit and three more
// for the children's boxes before descending. The traversal stack lives in
// shared memory: the near child is visited next, only the far child is
// pushed, so the stack never holds more entries than the heap has levels.
//
// A trace is two launches. k_trace_packets takes the rays in chunks of 32
// consecutive rays and traverses each chunk whose rays share a direction
// octant as one warp packet (one node at a time for the whole warp, each
// lane with its own decisions: coherent rays share the node fetches); the
// other chunks go to k_trace, which traverses one ray per lane. Results are
// the same bit for bit either way.
#include <algorithm>

#include "aur_internal.h"
#include "aur_math.cuh"
#include "aur_traverse.cuh"

namespace aur {
namespace {

constexpr int kTraceThreads = 128;
constexpr uint32_t kNoRay = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Stores a ray's result (hits: t, u, v, original prim id; occ: the
// occluder's original prim id) as intersect()/intersectAny() report it.
template <bool kAny>
__device__ __forceinline__ void store_result(uint32_t i, uint32_t best, float tmax, float best_t, float bu, float bv,
                                             const uint32_t* __restrict__ perm, float4* __restrict__ hits,
                                             uint32_t* __restrict__ occ) {
    if (kAny) {
        occ[i] = best == kNoPrim ? AUR_NO_HIT : perm[best];
    } else {
        float4 h;
        h.x = best == kNoPrim ? tmax : best_t;
        h.y = best == kNoPrim ? 0.0f : bu;
        h.z = best == kNoPrim ? 0.0f : bv;
        h.w = __uint_as_float(best == kNoPrim ? AUR_NO_HIT : perm[best]);
        hits[i] = h;
    }
}

// First pass of a trace: persistent warps take the rays in chunks of 32
// consecutive rays (one atomic per warp). A chunk whose rays share their
// direction octant and start within `packet_span` of each other is
// traversed as a warp packet (traverse_packet: coherent rays, such as a
// camera's, share node fetches and lanes); any other chunk goes to the
// deferred list for k_trace.
template <bool kAny>
__global__ void __launch_bounds__(kTraceThreads) k_trace_packets(const float4* __restrict__ recs, uint32_t nodes,
                                                                 const uint32_t* __restrict__ perm,
                                                                 const float4* __restrict__ rays, uint32_t n,
                                                                 float4* __restrict__ hits,
                                                                 uint32_t* __restrict__ occ,
                                                                 uint32_t* __restrict__ ctr,
                                                                 uint32_t* __restrict__ defer, int cap,
                                                                 float packet_span) {
    extern __shared__ uint32_t smem[];
    const int tid = threadIdx.x;
    const uint32_t lane = tid & 31;
    StackRef stk;
    stk.lo = reinterpret_cast<float*>(smem) + tid;
    stk.hi = reinterpret_cast<float*>(smem + cap * kTraceThreads) + tid;
    stk.stride = kTraceThreads;
    stk.cap = cap;
    const uint32_t chunks = (uint32_t)(((uint64_t)n + 31) >> 5);
    for (;;) {
        uint32_t c = 0;
        if (lane == 0) c = atomicAdd(ctr + 1, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= chunks) break;
        const uint32_t i = c * 32u + lane;
        const bool valid = i < n;       // lane 0 always has a ray
        f3 pos = mk3(0.0f), dir = mk3(0.0f);
        float tmax = 0.0f;
        if (valid) {
            const float4 r0 = rays[2 * (size_t)i];
            const float4 r1 = rays[2 * (size_t)i + 1];
            pos = mk3(r0.x, r0.y, r0.z);
            dir = mk3(r1.x, r1.y, r1.z);
            tmax = r0.w;
        }
        const uint32_t oct = dir_octant(dir);
        const uint32_t oct0 = __shfl_sync(0xffffffffu, oct, 0);
        if (!__all_sync(0xffffffffu, !valid || oct == oct0) || !(warp_origin_span(pos, valid) <= packet_span)) {
            if (lane == 0) defer[atomicAdd(ctr + 2, 1u)] = c;
            continue;
        }
        float best_t = tmax, bu = 0.0f, bv = 0.0f;
        const uint32_t best = traverse_packet<kAny>(recs, nodes, perm, valid, oct0, pos, dir, best_t, bu, bv, stk);
        if (valid) store_result<kAny>(i, best, tmax, best_t, bu, bv, perm, hits, occ);
    }
}

// Persistent traversal kernel with dynamic ray fetch: a lane whose ray is
// done takes the next unprocessed ray at once (one atomic per warp for all
// lanes asking together), so warps stay full until the ray pool is drained
// (Aila & Laine, "Understanding the efficiency of ray traversal on GPUs",
// HPG'09). Every ray is traversed as intersect()/intersectAny(); kBoxes adds
// the subtree-box pruning (off only to count the reference's own node visits).
// kCount adds up node fetches, slab crossings (triangle tests) and crossings
// of nodes with children (box loads) into counters[0..2].
// kTex: one sector of each node through the texture path (node_triangles).
// kDefer: the rays are those of the chunks k_trace_packets deferred
// (defer[0 .. ctr[2]), 32 consecutive rays each), else rays [0, n).
// ctr[0] is the ray fetch counter. Compiled for 9 blocks of 128 per SM (56
// registers): the deferred form otherwise takes 62 registers and 8 blocks,
// which measured slower.
template <bool kAny, bool kCount, bool kBoxes, bool kTex, bool kDefer>
__global__ void __launch_bounds__(kTraceThreads, 9) k_trace(const float4* __restrict__ recs, uint32_t nodes,
                                                         const uint32_t* __restrict__ perm,
                                                         const float4* __restrict__ rays, uint32_t n,
                                                         float4* __restrict__ hits, uint32_t* __restrict__ occ,
                                                         unsigned long long* __restrict__ counters,
                                                         uint32_t* __restrict__ ctr, int cap,
                                                         cudaTextureObject_t tex,
                                                         const uint32_t* __restrict__ defer) {
    extern __shared__ uint32_t smem[];
    const int tid = threadIdx.x;
    StackRef stk;
    stk.lo = reinterpret_cast<float*>(smem) + tid;
    stk.hi = reinterpret_cast<float*>(smem + cap * kTraceThreads) + tid;
    stk.stride = kTraceThreads;
    stk.cap = cap;
    uint32_t visits = 0, crossings = 0, inner = 0;
    // work items: the rays, or 32 per deferred chunk
    const uint32_t m = kDefer ? (uint32_t)min((unsigned long long)ctr[2] * 32ull, 0xFFFFFFFFull) : n;
    uint32_t i = kNoRay;
    f3 pos = mk3(0.0f), dir = mk3(0.0f), inv = mk3(0.0f);
    float tmax = 0.0f, best_t = 0.0f, bu = 0.0f, bv = 0.0f;
    uint32_t best = kNoPrim;
    TravState s;
    trav_init(s);
    for (;;) {
        if (i == kNoRay) {
            const uint32_t am = __activemask();
            const int leader = __ffs(am) - 1;
            uint32_t base = 0;
            if ((tid & 31) == leader) base = atomicAdd(ctr, (uint32_t)__popc(am));
            base = __shfl_sync(am, base, leader);
            i = base + __popc(am & lanemask_lt());
            if (i >= m) break;
            // A deferred chunk's positions past the last ray trace the last
            // ray again (the same result, stored twice).
            if (kDefer) i = min(defer[i >> 5] * 32u + (i & 31u), n - 1u);
            const float4 r0 = rays[2 * (size_t)i];
            const float4 r1 = rays[2 * (size_t)i + 1];
            pos = mk3(r0.x, r0.y, r0.z);
            dir = mk3(r1.x, r1.y, r1.z);
            inv = box_inv(dir);
            tmax = best_t = r0.w;
            bu = bv = 0.0f;
            best = kNoPrim;
            trav_init(s);
        }
        Sector s0;
        float4 q5;
        float nlo, nhi;
        bool done;
        if (trav_next(s, recs, nodes, pos, dir, inv, best_t, stk, s0, nlo, nhi, visits)) {
            if (kCount) {
                ++crossings;
                inner += 2 * s.k + 1 < nodes;
            }
            done = node_triangles<kAny, kTex>(recs, s.k, s0, perm, pos, dir, best_t, bu, bv, best, q5, tex);
            if (!done) trav_descend<kBoxes>(s, recs, q5, pos, dir, inv, best_t, nodes, stk, nlo, nhi);
        } else {
            done = true;
        }
        if (done) {
            store_result<kAny>(i, best, tmax, best_t, bu, bv, perm, hits, occ);
            i = kNoRay;
        }
    }
    if (kCount) {
        atomicAdd(counters, (unsigned long long)visits);
        atomicAdd(counters + 1, (unsigned long long)crossings);
        atomicAdd(counters + 2, (unsigned long long)inner);
    }
}

inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

// Largest origin spread of a warp packet: 1/64 of the soup's extent. Rays
// that start further apart visit mostly different nodes near their origins,
// and one ray per lane is faster for them.
inline float packet_span(const aur_nmh* nmh) { return nmh->extent * (1.0f / 64.0f); }

template <typename K>
aur_status persistent_grid(aur_ctx* ctx, K kernel, size_t smem, uint32_t n, uint32_t& grid) {
    int per_sm = 0;
    AUR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceThreads, smem));
    grid = std::max(1u, std::min<uint32_t>(cdiv(n, kTraceThreads), (uint32_t)(ctx->sm_count * per_sm)));
    return AUR_OK;
}

// The counting kernels (roofline accounting) trace every ray per lane and
// never read through the texture path; the shipped trace is two launches:
// k_trace_packets over all rays, then k_trace over the chunks it deferred.
template <bool kAny, bool kCount, bool kBoxes, bool kTex>
aur_status launch_kernel(aur_ctx* ctx, const aur_nmh* nmh, const float4* r, uint32_t n, float4* h, uint32_t* occ,
                         unsigned long long* counters, cudaStream_t stream, int slot) {
    const int cap = (int)nmh->levels + 1;
    const size_t smem = (size_t)2 * cap * kTraceThreads * sizeof(uint32_t);
    uint32_t* ctr = ctx->d_flags + 16 + 4 * slot;
    AUR_CUDA(cudaMemsetAsync(ctr, 0, 3 * sizeof(uint32_t), stream));
    uint32_t grid = 0;
    if constexpr (kCount) {
        aur_status st = persistent_grid(ctx, k_trace<kAny, kCount, kBoxes, kTex, false>, smem, n, grid);
        if (st != AUR_OK) return st;
        k_trace<kAny, kCount, kBoxes, kTex, false><<<grid, kTraceThreads, smem, stream>>>(
            nmh->node_recs, nmh->nodes, nmh->perm, r, n, h, occ, counters, ctr, cap, nmh->rec_tex, nullptr);
        AUR_CUDA(cudaGetLastError());
        return AUR_OK;
    }
    Scratch& d = ctx->defer[slot];
    const size_t need = (size_t)cdiv(n, 32) * sizeof(uint32_t);
    if (d.bytes < need) {
        if (d.ptr) cudaFreeAsync(d.ptr, stream);
        d.ptr = nullptr;
        d.bytes = 0;
        AUR_CHECK(::aur::dev_malloc_async(&d.ptr, need, stream) == cudaSuccess, AUR_ERR_OOM,
                  "trace: out of device memory for %u rays", n);
        d.bytes = need;
    }
    uint32_t* defer = static_cast<uint32_t*>(d.ptr);
    aur_status st = persistent_grid(ctx, k_trace_packets<kAny>, smem, n, grid);
    if (st != AUR_OK) return st;
    k_trace_packets<kAny><<<grid, kTraceThreads, smem, stream>>>(nmh->node_recs, nmh->nodes, nmh->perm, r, n, h, occ,
                                                                  ctr, defer, cap, packet_span(nmh));
    AUR_CUDA(cudaGetLastError());
    st = persistent_grid(ctx, k_trace<kAny, false, kBoxes, kTex, true>, smem, n, grid);
    if (st != AUR_OK) return st;
    k_trace<kAny, false, kBoxes, kTex, true><<<grid, kTraceThreads, smem, stream>>>(
        nmh->node_recs, nmh->nodes, nmh->perm, r, n, h, occ, nullptr, ctr, cap, nmh->rec_tex, defer);
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

// The shipped kernels read through the texture path when the NMH has its
// record texture; the counting kernels (roofline accounting) never do.
template <bool kAny, bool kCount, bool kBoxes = true>
aur_status launch_one(aur_ctx* ctx, const aur_nmh* nmh, const float4* r, uint32_t n, float4* h, uint32_t* occ,
                      unsigned long long* counters, cudaStream_t stream, int slot) {
    if (!kCount && nmh->rec_tex)
        return launch_kernel<kAny, kCount, kBoxes, true>(ctx, nmh, r, n, h, occ, counters, stream, slot);
    return launch_kernel<kAny, kCount, kBoxes, false>(ctx, nmh, r, n, h, occ, counters, stream, slot);
}

aur_status launch_trace(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, aur_hit* hits,
                        uint32_t* occluder, unsigned long long* counters, cudaStream_t stream, bool pruned,
                        int slot) {
    if (n == 0) return AUR_OK;
    const float4* r = reinterpret_cast<const float4*>(rays);
    float4* h = reinterpret_cast<float4*>(hits);
    if (counters && !pruned)
        return occluder ? launch_one<true, true, false>(ctx, nmh, r, n, nullptr, occluder, counters, stream, slot)
                        : launch_one<false, true, false>(ctx, nmh, r, n, h, nullptr, counters, stream, slot);
    if (counters)
        return occluder ? launch_one<true, true>(ctx, nmh, r, n, nullptr, occluder, counters, stream, slot)
                        : launch_one<false, true>(ctx, nmh, r, n, h, nullptr, counters, stream, slot);
    return occluder ? launch_one<true, false>(ctx, nmh, r, n, nullptr, occluder, nullptr, stream, slot)
                    : launch_one<false, false>(ctx, nmh, r, n, h, nullptr, nullptr, stream, slot);
}

}  // namespace aur

using namespace aur;

namespace {

aur_status check_trace_args(aur_ctx* ctx, const aur_nmh* nmh, const void* rays, uint32_t n, const void* out) {
    AUR_CHECK(ctx && nmh, AUR_ERR_INVALID, "trace: null context or NMH");
    AUR_CHECK(n == 0 || (rays && out), AUR_ERR_INVALID, "trace: null ray or result buffer for %u rays", n);
    AUR_CHECK(nmh->device == ctx->device, AUR_ERR_INVALID, "trace: NMH lives on device %d, context on %d",
              nmh->device, ctx->device);
    AUR_CHECK(((uintptr_t)rays & 15) == 0 && ((uintptr_t)out & 3) == 0, AUR_ERR_INVALID,
              "trace: rays must be 16-byte aligned");
    return AUR_OK;
}

// Host-buffer pipeline: chunks of rays alternate between two device slots
// and two launch streams (the context's and an internal one), so the H2D copy
// of chunk c+1 and the D2H copy of chunk c-1 overlap the traversal of c, and
// the traversal of c+1 starts while the last rays of c drain. Each slot has
// its own counters and deferred list, as its kernels may run concurrently
// with the other's. Chunks hold 8M rays, except a first chunk of 2M (its
// copy in waits for nothing to overlap) and, where the rays allow, a last
// chunk of 2M (its copy out likewise): 2^24 rays go as 2M, 8M, 4M, 2M, which
// measured 636 Mrays/s end to end against 605 for even chunks of 4M.
aur_status trace_host(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, void* out, bool any) {
    aur_status st = check_trace_args(ctx, nmh, rays, n, out);
    if (st != AUR_OK) return st;
    if (n == 0) return AUR_OK;
    AUR_CUDA(cudaSetDevice(ctx->device));
    const uint32_t chunk = 1u << 23;
    const size_t out_sz = any ? sizeof(uint32_t) : sizeof(aur_hit);
    for (int s = 0; s < 2; ++s) {
        const size_t need_in = (size_t)chunk * sizeof(aur_ray), need_out = (size_t)chunk * out_sz;
        if (ctx->pipe[s].bytes < need_in) {
            cudaFree(ctx->pipe[s].ptr);
            ctx->pipe[s].ptr = nullptr; ctx->pipe[s].bytes = 0;
            AUR_CHECK(::aur::dev_malloc(&ctx->pipe[s].ptr, need_in) == cudaSuccess, AUR_ERR_OOM, "trace_host: out of memory");
            ctx->pipe[s].bytes = need_in;
        }
        if (ctx->out[s].bytes < need_out) {
            cudaFree(ctx->out[s].ptr);
            ctx->out[s].ptr = nullptr; ctx->out[s].bytes = 0;
            AUR_CHECK(::aur::dev_malloc(&ctx->out[s].ptr, need_out) == cudaSuccess, AUR_ERR_OOM, "trace_host: out of memory");
            ctx->out[s].bytes = need_out;
        }
    }
    cudaEvent_t* in_done = ctx->ev;
    cudaEvent_t* comp_done = ctx->ev + 2;
    cudaEvent_t* out_done = ctx->ev + 4;
    // the copy and second launch streams start after work already queued on the launch stream
    AUR_CUDA(cudaEventRecord(ctx->ev[6], ctx->stream));
    AUR_CUDA(cudaStreamWaitEvent(ctx->copy_in, ctx->ev[6], 0));
    AUR_CUDA(cudaStreamWaitEvent(ctx->compute2, ctx->ev[6], 0));
    cudaStream_t const launch[2] = {ctx->stream, ctx->compute2};
    bool used[2] = {false, false};
    uint32_t m = 0;
    for (uint32_t c0 = 0, c = 0; c0 < n; c0 += m, ++c) {
        const int s = (int)(c & 1);
        // a quarter chunk first (the first copy is not overlapped) and last
        // (nor is the last copy back); full chunks between
        const uint32_t left = n - c0;
        uint32_t want = c == 0 ? chunk / 4 : chunk;
        if (c > 0 && left > chunk / 2 && left <= chunk + chunk / 4) want = left - chunk / 4;
        m = left < want ? left : want;
        if (used[s]) AUR_CUDA(cudaStreamWaitEvent(ctx->copy_in, out_done[s], 0));
        AUR_CUDA(cudaMemcpyAsync(ctx->pipe[s].ptr, rays + c0, (size_t)m * sizeof(aur_ray), cudaMemcpyHostToDevice,
                                 ctx->copy_in));
        AUR_CUDA(cudaEventRecord(in_done[s], ctx->copy_in));
        AUR_CUDA(cudaStreamWaitEvent(launch[s], in_done[s], 0));
        st = launch_trace(ctx, nmh, (const aur_ray*)ctx->pipe[s].ptr, m, any ? nullptr : (aur_hit*)ctx->out[s].ptr,
                          any ? (uint32_t*)ctx->out[s].ptr : nullptr, nullptr, launch[s], true, s);
        if (st != AUR_OK) return st;
        AUR_CUDA(cudaEventRecord(comp_done[s], launch[s]));
        AUR_CUDA(cudaStreamWaitEvent(ctx->copy_out, comp_done[s], 0));
        AUR_CUDA(cudaMemcpyAsync((char*)out + (size_t)c0 * out_sz, ctx->out[s].ptr, (size_t)m * out_sz,
                                 cudaMemcpyDeviceToHost, ctx->copy_out));
        AUR_CUDA(cudaEventRecord(out_done[s], ctx->copy_out));
        used[s] = true;
    }
    AUR_CUDA(cudaStreamSynchronize(ctx->copy_out));
    AUR_CUDA(cudaStreamSynchronize(ctx->compute2));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    return AUR_OK;
}

}  // namespace

extern "C" {

aur_status aur_trace_closest(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, aur_hit* hits) {
    AUR_RANGE("aur_trace_closest");
    aur_status st = check_trace_args(ctx, nmh, rays, n, hits);
    if (st != AUR_OK) return st;
    AUR_CUDA(cudaSetDevice(ctx->device));
    return launch_trace(ctx, nmh, rays, n, hits, nullptr, nullptr, ctx->stream, true);
}

aur_status aur_trace_any(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, uint32_t* occluder) {
    AUR_RANGE("aur_trace_any");
    aur_status st = check_trace_args(ctx, nmh, rays, n, occluder);
    if (st != AUR_OK) return st;
    AUR_CUDA(cudaSetDevice(ctx->device));
    return launch_trace(ctx, nmh, rays, n, nullptr, occluder, nullptr, ctx->stream, true);
}

aur_status aur_trace_closest_host(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, aur_hit* hits) {
    AUR_RANGE("aur_trace_closest_host");
    return trace_host(ctx, nmh, rays, n, hits, false);
}

aur_status aur_trace_any_host(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, uint32_t* occluder) {
    AUR_RANGE("aur_trace_any_host");
    return trace_host(ctx, nmh, rays, n, occluder, true);
}

namespace {

// Runs closest hit and any hit over n device rays with the counting kernels;
// out[0..2] closest (fetches, crossings, inner crossings), out[3..5] any hit.
aur_status count_work(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, bool pruned,
                      unsigned long long out[6]) {
    for (int q = 0; q < 6; ++q) out[q] = 0;
    if (n == 0) return AUR_OK;
    void* scratch = nullptr;
    const size_t bytes = 256 + (size_t)n * sizeof(aur_hit);
    AUR_CHECK(::aur::dev_malloc_async(&scratch, bytes, ctx->stream) == cudaSuccess, AUR_ERR_OOM,
              "trace counters: out of memory");
    unsigned long long* cnt = (unsigned long long*)scratch;
    aur_hit* hits = (aur_hit*)((char*)scratch + 256);
    cudaMemsetAsync(cnt, 0, 48, ctx->stream);
    aur_status st = launch_trace(ctx, nmh, rays, n, hits, nullptr, cnt, ctx->stream, pruned);
    if (st == AUR_OK) st = launch_trace(ctx, nmh, rays, n, nullptr, (uint32_t*)hits, cnt + 3, ctx->stream, pruned);
    unsigned long long host[6] = {0, 0, 0, 0, 0, 0};
    cudaMemcpyAsync(host, cnt, 48, cudaMemcpyDeviceToHost, ctx->stream);
    cudaFreeAsync(scratch, ctx->stream);
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    if (st != AUR_OK) return st;
    for (int q = 0; q < 6; ++q) out[q] = host[q];
    return AUR_OK;
}

}  // namespace

aur_status aur_trace_count_visits(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n,
                                  unsigned long long node_visits[2]) {
    AUR_RANGE("aur_trace_count_visits");
    AUR_CHECK(node_visits, AUR_ERR_INVALID, "aur_trace_count_visits: null output");
    aur_status st = check_trace_args(ctx, nmh, rays, n, rays);
    if (st != AUR_OK) return st;
    AUR_CUDA(cudaSetDevice(ctx->device));
    unsigned long long c[6];
    st = count_work(ctx, nmh, rays, n, false, c);
    node_visits[0] = c[0];
    node_visits[1] = c[3];
    return st;
}

aur_status aur_debug_trace_deferred(aur_ctx* ctx, uint32_t* chunks) {
    AUR_CHECK(ctx && chunks, AUR_ERR_INVALID, "aur_debug_trace_deferred: null argument");
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaMemcpyAsync(chunks, ctx->d_flags + 16 + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    return AUR_OK;
}

aur_status aur_trace_stats(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n,
                           aur_trace_work* closest, aur_trace_work* any) {
    AUR_RANGE("aur_trace_stats");
    AUR_CHECK(closest && any, AUR_ERR_INVALID, "aur_trace_stats: null output");
    aur_status st = check_trace_args(ctx, nmh, rays, n, rays);
    if (st != AUR_OK) return st;
    AUR_CUDA(cudaSetDevice(ctx->device));
    unsigned long long c[6];
    st = count_work(ctx, nmh, rays, n, true, c);
    closest->node_fetches = c[0];
    closest->slab_crossings = c[1];
    closest->box_loads = c[2];
    any->node_fetches = c[3];
    any->slab_crossings = c[4];
    any->box_loads = c[5];
    return st;
}

}  // extern "C"
