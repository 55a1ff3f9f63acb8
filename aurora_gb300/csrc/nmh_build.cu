// nmh_build.cu — GPU build of the NMH implicit pair-heap.
//
// Replaces cudaRebuildNMH (kernels/rebuilder.cu:311-450). The reference
// re-sorts all triangles twice per level with Thrust (sortTriangles, :262-289)
// and reads the split count back to the host every level (:255). Here:
//   1. per-triangle bounds and order-preserving integer keys (:72-91);
//   2. one stable LSD radix sort per axis of (min-key, prim id) — three
//      presorted lists;
//   3. per level, all on the device with closed-form segment offsets:
//      a. segmented arg-max of the max-key over the current axis' list gives
//         pair[1]; the first element of each segment is pair[0] (:93-151);
//      b. the next axis' list is compacted (pairs removed); its position
//         within the remainder decides left/right (calcPartition sizes,
//         :40-50, :189-215);
//      c. the other two lists are stably partitioned left/right.
//      Stable partitions are warp-ballot scans over 4096-element tiles in a
//      single pass, the tile prefixes by decoupled look-back;
//   3'. once every node's segment fits 2048 triangles, one block per node
//      finishes its subtree in shared memory (k_local_finish).
//   4. each pair is ordered by the last level's axis key (the reference's
//      final sort, :381-385), then vertices are gathered into NMH order
//      (applyIndices, :217-245) and traversal node records are written.
// Every ordering ties by the lower original prim id.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "aur_internal.h"
#include "aur_math.cuh"
#include "aur_traverse.cuh"

namespace aur {
namespace {

constexpr uint32_t kDone = 0xFFFFFFFFu;
constexpr int kThreads = 256;
constexpr int kTileItems = 16;                       // per thread, scan tiles
constexpr uint32_t kTile = kThreads * kTileItems;     // 4096
constexpr int kSelectItems = 16;                     // per thread, k_select (a multiple of 4)
constexpr int kSortItems = 8;
constexpr uint32_t kSortTile = kThreads * kSortItems; // 2048

__device__ __forceinline__ uint32_t orderable(float f) {
    if (f == 0.0f) f = 0.0f;  // -0 and +0 compare equal in the reference's float sorts
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__host__ __device__ __forceinline__ uint32_t level_of(uint32_t k) {
#ifdef __CUDA_ARCH__
    return 31u - (uint32_t)__clz(k + 1u);
#else
    return 31u - (uint32_t)__builtin_clz(k + 1u);
#endif
}

// Nodes in the subtree of node k of a complete heap of n nodes.
__host__ __device__ __forceinline__ uint64_t subtree_nodes(uint64_t k, uint64_t n) {
    uint64_t s = 0;
    for (uint64_t f = k, w = 1; f < n; f = 2 * f + 1, w <<= 1) s += (w < n - f) ? w : n - f;
    return s;
}

// Triangle offset of node k's segment among the active triangles of its
// level (L0 = first node of the level): twice the subtree sizes of the nodes
// left of k on the level.
__host__ __device__ __forceinline__ uint64_t segment_start(uint64_t k, uint64_t L0, uint64_t n) {
    const uint64_t M = k - L0;
    uint64_t s = 0;
    for (uint64_t f = L0, w = 1; f < n; f = 2 * f + 1, w <<= 1) s += (M * w < n - f) ? M * w : n - f;
    return 2 * s;
}

// Triangles that go to left children among the nodes left of k on its level:
// sum over k' in [L0, k) of 2 * subtree_nodes(2k'+1).
__host__ __device__ __forceinline__ uint64_t left_base(uint64_t k, uint64_t L0, uint64_t n) {
    const uint64_t M = k - L0;
    uint64_t s = 0;
    for (uint64_t g = 2 * L0 + 1, w = 1; g < n; g = 2 * g + 1, w <<= 1) {
        const uint64_t r = n - g, step = 2 * w;
        uint64_t full = 0;
        if (r >= w) { full = (r - w) / step + 1; if (full > M) full = M; }
        s += full * w;
        if (full < M && r > full * step) {
            const uint64_t rem = r - full * step;
            s += rem < w ? rem : w;
        }
    }
    return 2 * s;
}

// ------------------------------------------------------------ kernels

// Bounds and sort keys (computeTriangleBounds, rebuilder.cu:72-91). Position
// i >= count_in is the even-padding duplicate of the last triangle.
// A coordinate that is NaN or infinite sets bit 8 of *err: the reference's
// float sorts have no defined order for NaN, so the build refuses such soups.
__global__ void k_bounds(const float* __restrict__ V, uint32_t N, size_t S, uint32_t count_in,
                         float* __restrict__ mn, float* __restrict__ mx, uint32_t* __restrict__ keys,
                         uint32_t* __restrict__ vals, uint32_t* __restrict__ err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint32_t src = i < count_in ? i : count_in - 1;
    const float* v = V + (size_t)src * 9;
    float c[9];
    bool finite = true;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        c[q] = v[q];
        finite = finite && isfinite(c[q]);
    }
    if (!finite) atomicOr(err, 8u);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float lo = fminf(fminf(c[3 * a], c[3 * a + 1]), c[3 * a + 2]);
        const float hi = fmaxf(fmaxf(c[3 * a], c[3 * a + 1]), c[3 * a + 2]);
        mn[a * S + i] = lo;
        mx[a * S + i] = hi;
        keys[a * S + i] = orderable(lo);
        vals[a * S + i] = i;
    }
}

// Radix sort, pass histogram: hist[(axis*256 + digit) * nb + block].
__global__ void k_radix_hist(const uint32_t* __restrict__ keys, uint32_t N, size_t S, int shift,
                             uint32_t* __restrict__ hist, uint32_t nb) {
    __shared__ uint32_t h[256];
    const uint32_t axis = blockIdx.y;
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t* k = keys + axis * S;
    const uint32_t base = blockIdx.x * kSortTile;
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t idx = base + i * kThreads + threadIdx.x;
        if (idx < N) atomicAdd(&h[(k[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[((size_t)axis * 256 + threadIdx.x) * nb + blockIdx.x] = h[threadIdx.x];
}

// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[nw - 1];
    const uint32_t r = x - v + (warp > 0 ? s_warp[warp - 1] : 0);
    __syncthreads();
    return r;
}

// Exclusive scan of each (axis, digit) row of the histogram over blocks;
// totals[axis*256 + digit] = row sum.
__global__ void k_radix_scan_rows(uint32_t* __restrict__ hist, uint32_t nb, uint32_t* __restrict__ totals) {
    __shared__ uint32_t s_warp[32];
    const size_t row = (size_t)blockIdx.y * 256 + blockIdx.x;
    uint32_t* h = hist + row * nb;
    uint32_t carry = 0;
    for (uint32_t b = 0; b < nb; b += blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const uint32_t v = i < nb ? h[i] : 0;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(v, s_warp, tot);
        if (i < nb) h[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[row] = carry;
}

// Stable scatter of one radix pass.
__global__ void __launch_bounds__(kThreads) k_radix_scatter(const uint32_t* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin,
                                                            uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                            uint32_t N, size_t S, int shift,
                                                            const uint32_t* __restrict__ hist,
                                                            const uint32_t* __restrict__ totals, uint32_t nb,
                                                            uint32_t* __restrict__ err) {
    __shared__ uint32_t s_off[256];
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_wc[kThreads / 32][256];
    __shared__ uint32_t s_warp[32];
    const uint32_t axis = blockIdx.y;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    {
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(totals[axis * 256 + t], s_warp, tot);
        s_off[t] = ex + hist[((size_t)axis * 256 + t) * nb + blockIdx.x];
        s_base[t] = 0;
    }
    const uint32_t* ki = kin + axis * S;
    const uint32_t* vi = vin + axis * S;
    uint32_t* ko = kout + axis * S;
    uint32_t* vo = vout + axis * S;
    const uint32_t base = blockIdx.x * kSortTile;
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t idx = base + i * kThreads + t;
        const bool valid = idx < N;
        const uint32_t key = valid ? ki[idx] : 0xFFFFFFFFu;
        const uint32_t val = valid ? vi[idx] : 0u;
        const uint32_t d = valid ? ((key >> shift) & 255u) : 256u;
#pragma unroll
        for (int q = 0; q < 256 / 32; ++q) s_wc[warp][q * 32 + lane] = 0;
        __syncthreads();
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lanemask_lt());
        if (valid && rank == 0) s_wc[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = s_base[t];
#pragma unroll
            for (int w = 0; w < kThreads / 32; ++w) {
                const uint32_t c = s_wc[w][t];
                s_wc[w][t] = run;
                run += c;
            }
            s_base[t] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t dst = s_off[d] + s_wc[warp][d] + rank;
            if (dst < N) {
                ko[dst] = key;
                vo[dst] = val;
            } else {
                atomicOr(err, 4u);
            }
        }
        __syncthreads();
    }
}

// Per-node layout table: segment start, left-child triangle count and
// left base, for every node of the heap.
__global__ void k_node_table(uint32_t n, uint32_t* __restrict__ nstart, uint32_t* __restrict__ nnuml,
                             uint32_t* __restrict__ nlbase) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t L0 = (1u << level_of(k)) - 1u;
    nstart[k] = (uint32_t)segment_start(k, L0, n);
    nnuml[k] = (2u * k + 1u < n) ? (uint32_t)(2 * subtree_nodes(2u * k + 1u, n)) : 0u;
    nlbase[k] = (uint32_t)left_base(k, L0, n);
}

// Bit 16 of the error word: a look-back wait gave up. The lists of that
// level then have positions nobody wrote, so every later kernel of the build
// returns at once instead of reading ids out of them; the build reports
// AUR_ERR_TIMEOUT and its outputs are not used.
constexpr uint32_t kErrLookback = 16u;
__device__ __forceinline__ bool build_aborted(const uint32_t* err) {
    return (*reinterpret_cast<const volatile uint32_t*>(err) & kErrLookback) != 0u;
}

// Segmented arg-max of (max-key, lowest prim id) over each node's segment,
// excluding the segment's first element, which is recorded as pair[0]
// (swapMaxTriangleTPS/TPT, rebuilder.cu:93-151). Each thread owns
// kSelectItems consecutive list positions.
__global__ void __launch_bounds__(kThreads) k_select(const uint32_t* __restrict__ list, uint32_t M,
                                                     const float* __restrict__ mxa,
                                                     const uint32_t* __restrict__ node_of,
                                                     const uint32_t* __restrict__ nstart, uint32_t L0,
                                                     unsigned long long* __restrict__ best,
                                                     uint32_t* __restrict__ pair0, const uint32_t* err) {
    if (build_aborted(err)) return;       // whole blocks: the word does not change during this launch
    const uint32_t base = (blockIdx.x * kThreads + threadIdx.x) * kSelectItems;
    const int lane = threadIdx.x & 31;
    uint32_t cur = kDone;
    unsigned long long cur_key = 0;
    bool first_run = true;
    if (base < M) {
        const int cnt = (M - base) < (uint32_t)kSelectItems ? (int)(M - base) : kSelectItems;
        uint32_t pid[kSelectItems];
        if (cnt == kSelectItems) {
            const uint4* p = reinterpret_cast<const uint4*>(list + base);
#pragma unroll
            for (int q = 0; q < kSelectItems / 4; ++q) {
                const uint4 v = p[q];
                pid[4 * q] = v.x; pid[4 * q + 1] = v.y; pid[4 * q + 2] = v.z; pid[4 * q + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int i = 0; i < kSelectItems; ++i) pid[i] = i < cnt ? list[base + i] : 0u;
        }
        uint32_t nd[kSelectItems];
#pragma unroll
        for (int i = 0; i < kSelectItems; ++i) nd[i] = i < cnt ? node_of[pid[i]] : kDone;
#pragma unroll
        for (int i = 0; i < kSelectItems; ++i) {
            if (i >= cnt) break;
            const uint32_t k = nd[i];
            unsigned long long key;
            if (base + i == nstart[k]) {
                pair0[k - L0] = pid[i];
                key = 0ull;
            } else {
                key = ((unsigned long long)orderable(mxa[pid[i]]) << 32) | (unsigned long long)(0xFFFFFFFFu - pid[i]);
            }
            if (k != cur) {
                if (cur != kDone) {
                    if (first_run) atomicMax(&best[cur - L0], cur_key);
                    else best[cur - L0] = cur_key;       // run wholly inside this thread's range
                    first_run = false;
                }
                cur = k;
                cur_key = key;
            } else if (key > cur_key) {
                cur_key = key;
            }
        }
    }
    // The last run may continue into the next lanes: segmented max across the
    // warp (equal node ids are contiguous), heads publish.
    uint32_t node = cur;
    unsigned long long key = cur_key;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t on = __shfl_down_sync(0xffffffffu, node, o);
        const unsigned long long ok = __shfl_down_sync(0xffffffffu, key, o);
        if (lane + o < 32 && on == node && ok > key) key = ok;
    }
    const uint32_t prev = __shfl_up_sync(0xffffffffu, node, 1);
    if (node != kDone && (lane == 0 || prev != node)) atomicMax(&best[node - L0], key);
}

// Writes each level node's pair into the heap and retires its triangles.
__global__ void k_emit_pairs(uint32_t L0, uint32_t L1, unsigned long long* __restrict__ best,
                             const uint32_t* __restrict__ pair0, uint32_t* __restrict__ heap,
                             uint32_t* __restrict__ node_of, const uint32_t* err) {
    const uint32_t k = L0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L1 || build_aborted(err)) return;
    const uint32_t p0 = pair0[k - L0];
    const uint32_t p1 = 0xFFFFFFFFu - (uint32_t)(best[k - L0] & 0xFFFFFFFFull);
    best[k - L0] = 0ull;
    heap[2 * k] = p0;
    heap[2 * k + 1] = p1;
    node_of[p0] = kDone;
    node_of[p1] = kDone;
}

struct ListSet {
    const uint32_t* in[2];
    uint32_t* out[2];
};

// Flags of list position j: D = retired (pair), L = goes to a left child.
template <bool kPart>
__device__ __forceinline__ void flags_of(uint32_t nd, bool& D, bool& Lf) {
    D = nd == kDone;
    Lf = kPart && !D && (nd & 1u);
}

// Single-pass tile prefix (decoupled look-back, D. Merrill and M. Garland,
// "Single-pass Parallel Prefix Scan with Decoupled Look-back", NVIDIA
// NVR-2016-002): each tile publishes its (D, L) counts, then walks back over
// its predecessors' words until one holds an inclusive prefix. A status word
// packs the state (bits 62-63: 0 not ready, 1 counts of the tile, 2
// inclusive prefix) with the D count (bits 31-61) and the L count (bits
// 0-30), so one 64-bit store publishes all of it. Tiles are taken in launch
// order from a counter, so every tile a block waits for belongs to a block
// that is already running; the wait is still bounded, and a block that gives
// up sets bit 16 of *err and publishes what it has. `test` != 0 is a test
// hook (aur_debug_lookback_timeout): every tile after the first then waits
// on its predecessor as on a word that nothing sets, for `test` spins, so
// that the give-up path runs on purpose.
constexpr unsigned long long kStTile = 1ull << 62, kStPrefix = 2ull << 62;
constexpr uint32_t kLookbackSpins = 1u << 22;

__device__ __forceinline__ unsigned long long st_word(unsigned long long state, uint64_t d, uint64_t l) {
    return state | ((d & 0x7FFFFFFFull) << 31) | (l & 0x7FFFFFFFull);
}

// One thread: exclusive (D, L) prefix of `tile` given its own counts.
__device__ uint2 tile_lookback(unsigned long long* status, uint32_t tile, uint32_t cd, uint32_t cl,
                               uint32_t* err, uint32_t test) {
    if (tile == 0) {
        atomicExch(status, st_word(kStPrefix, cd, cl));
        return make_uint2(0u, 0u);
    }
    atomicExch(status + tile, st_word(kStTile, cd, cl));
    uint64_t ed = 0, el = 0;
    uint32_t spins = 0;
    const uint32_t limit = test ? test : kLookbackSpins;
    for (int64_t p = (int64_t)tile - 1; p >= 0;) {
        const unsigned long long w = atomicAdd(status + p, 0ull);   // coherent read
        const unsigned long long state = test ? 0ull : w >> 62;
        if (state == 0) {
            if (++spins > limit) {
                atomicOr(err, kErrLookback);
                break;
            }
            __nanosleep(32);
            continue;
        }
        ed += (w >> 31) & 0x7FFFFFFFull;
        el += w & 0x7FFFFFFFull;
        if (state == 2) break;
        --p;
    }
    atomicExch(status + tile, st_word(kStPrefix, ed + cd, el + cl));
    return make_uint2((uint32_t)ed, (uint32_t)el);
}

// Per-tile scan helper: the block takes the next tile, and for each of a
// warp's 16 items gets the exclusive global counts of D and L flags before
// position j (tile prefix by look-back).
template <bool kPart>
struct TileScan {
    uint32_t pid[kTileItems];
    uint32_t nd[kTileItems];
    uint32_t dmask[kTileItems], lmask[kTileItems];
    uint32_t wd, wl;  // warp offsets within the tile + tile prefix
    uint32_t tile;
};

template <bool kPart>
__device__ __forceinline__ void tile_scan(const uint32_t* __restrict__ list, uint32_t M,
                                          const uint32_t* __restrict__ node_of, unsigned long long* status,
                                          uint32_t* tile_counter, uint32_t* err, uint32_t test,
                                          TileScan<kPart>& s) {
    __shared__ uint32_t s_d[kThreads / 32], s_l[kThreads / 32];
    __shared__ uint32_t s_tile;
    __shared__ uint2 s_pre;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
    __syncthreads();
    s.tile = s_tile;
    const uint32_t wbase = s.tile * kTile + warp * 32 * kTileItems;
#pragma unroll
    for (int i = 0; i < kTileItems; ++i) {
        const uint32_t j = wbase + i * 32 + lane;
        s.pid[i] = j < M ? list[j] : 0u;
    }
    uint32_t cd = 0, cl = 0;
#pragma unroll
    for (int i = 0; i < kTileItems; ++i) {
        const uint32_t j = wbase + i * 32 + lane;
        s.nd[i] = j < M ? node_of[s.pid[i]] : kDone;
        bool D = false, Lf = false;
        if (j < M) flags_of<kPart>(s.nd[i], D, Lf);
        s.dmask[i] = __ballot_sync(0xffffffffu, D);
        s.lmask[i] = __ballot_sync(0xffffffffu, Lf);
        cd += __popc(s.dmask[i]);
        cl += __popc(s.lmask[i]);
    }
    if (lane == 0) { s_d[warp] = cd; s_l[warp] = cl; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t td = 0, tl = 0;
        for (int w = 0; w < kThreads / 32; ++w) { td += s_d[w]; tl += s_l[w]; }
        s_pre = tile_lookback(status, s.tile, td, tl, err, test);
    }
    __syncthreads();
    uint32_t od = s_pre.x, ol = s_pre.y;
    for (int w = 0; w < warp; ++w) { od += s_d[w]; ol += s_l[w]; }
    s.wd = od;
    s.wl = ol;
}

// Next-axis list: drop retired triangles, classify the rest left/right by
// their rank in the remainder of their node (rpos < numL -> left child).
__global__ void __launch_bounds__(kThreads) k_split_next(ListSet ls, uint32_t M, uint32_t* __restrict__ node_of,
                                                         const uint32_t* __restrict__ nstart,
                                                         const uint32_t* __restrict__ nnuml, uint32_t L0,
                                                         unsigned long long* __restrict__ status,
                                                         uint32_t* __restrict__ tile_counter,
                                                         uint32_t* __restrict__ err, uint32_t test) {
    // Blocks of this launch may see the word change (a tile that gives up),
    // so the decision is made block-wide. A block that leaves takes no tile;
    // the tiles after it then give up too, within their bounded wait.
    if (__syncthreads_or(build_aborted(err))) return;
    TileScan<false> s;
    tile_scan<false>(ls.in[0], M, node_of, status, tile_counter, err, test, s);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t wbase = s.tile * kTile + warp * 32 * kTileItems;
    const uint32_t lt = lanemask_lt();
    uint32_t gd = s.wd;
    uint32_t* out = ls.out[0];
#pragma unroll
    for (int i = 0; i < kTileItems; ++i) {
        const uint32_t j = wbase + i * 32 + lane;
        const uint32_t GP = gd + __popc(s.dmask[i] & lt);
        gd += __popc(s.dmask[i]);
        if (j < M && s.nd[i] != kDone) {
            const uint32_t k = s.nd[i];
            const uint32_t rpos = (j - nstart[k]) - (GP - 2u * (k - L0));
            node_of[s.pid[i]] = rpos < nnuml[k] ? 2u * k + 1u : 2u * k + 2u;
            out[j - GP] = s.pid[i];
        }
    }
}

// The other two lists: stable partition into left then right child segments.
__global__ void __launch_bounds__(kThreads) k_partition(ListSet ls, uint32_t M, const uint32_t* __restrict__ node_of,
                                                        const uint32_t* __restrict__ nstart,
                                                        const uint32_t* __restrict__ nnuml,
                                                        const uint32_t* __restrict__ nlbase, uint32_t L0,
                                                        unsigned long long* __restrict__ status, uint32_t ntiles,
                                                        uint32_t* __restrict__ tile_counter, uint32_t m_next,
                                                        uint32_t* __restrict__ err, uint32_t test) {
    if (__syncthreads_or(build_aborted(err))) return;      // see k_split_next
    TileScan<true> s;
    tile_scan<true>(ls.in[blockIdx.y], M, node_of, status + (size_t)blockIdx.y * ntiles, tile_counter + blockIdx.y,
                    err, test, s);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t wbase = s.tile * kTile + warp * 32 * kTileItems;
    const uint32_t lt = lanemask_lt();
    uint32_t gd = s.wd, gl = s.wl;
    uint32_t* out = ls.out[blockIdx.y];
#pragma unroll
    for (int i = 0; i < kTileItems; ++i) {
        const uint32_t j = wbase + i * 32 + lane;
        const uint32_t GP = gd + __popc(s.dmask[i] & lt);
        const uint32_t GL = gl + __popc(s.lmask[i] & lt);
        gd += __popc(s.dmask[i]);
        gl += __popc(s.lmask[i]);
        if (j < M && s.nd[i] != kDone) {
            const uint32_t c = s.nd[i];
            const uint32_t k = (c - 1u) >> 1;
            const uint32_t lb = nlbase[k];
            uint32_t dst;
            if (c & 1u) {
                dst = (nstart[k] - 2u * (k - L0)) + GL - lb;
            } else {
                const uint32_t GR = j - GL - GP;
                dst = nnuml[k] + GR + lb;
            }
            if (dst < m_next) out[dst] = s.pid[i];
            else atomicOr(err, 4u);
        }
    }
}

// ------------------------------------------------ subtree finish in shared memory
// Once every node segment of a level holds at most kLocalMax triangles, one
// block per node of that level finishes its whole subtree with the same
// per-level steps (select, emit, split, partition) on shared-memory copies of
// the three lists, instead of 8 launches per remaining level over the whole
// soup. Triangles get block-local ids (their position in the first list);
// lists hold local ids, the global node_of array is reused as the pid ->
// local id map while the block loads its segment.
constexpr uint32_t kLocalMax = 2048;
constexpr int kLocalThreads = 512;
constexpr int kLocalPer = (int)kLocalMax / kLocalThreads;   // elements per thread in block scans
constexpr uint16_t kLocalDone = 0xFFFFu;

// 53.6 KB: four blocks fit an SM, so the 512 subtrees of a 1M-triangle
// build run as one wave on 152 SMs.
struct LocalSmem {
    uint16_t list[2][3][kLocalMax];       // local ids, double-buffered, per axis
    uint16_t node[kLocalMax];             // local node index at the current depth, kLocalDone once paired
    uint8_t right[kLocalMax];             // 1: goes to the right child at the next depth
    union {                               // select / emit use best, split / partition the scans
        struct {
            uint16_t pre0[kLocalMax];     // block-scan outputs (exclusive prefix counts)
            uint16_t pre1[kLocalMax];
        };
        unsigned long long best[kLocalMax / 2];
    };
    uint32_t pid[kLocalMax];              // global prim id of each local id
    uint16_t off[kLocalMax / 2 + 1];      // segment offsets of the depth's nodes (+ end)
    uint16_t numl[kLocalMax / 2];         // triangles going to the left child
    uint16_t p0[kLocalMax / 2];           // pair[0] (local id) per node
    uint32_t warp_tot[kLocalThreads / 32][2];
};

// Exclusive prefix counts of two flags over positions [0, m) (each thread a
// contiguous chunk of kLocalPer), written to out0 and (if not null) out1;
// returns the totals.
template <typename F>
__device__ __forceinline__ void local_scan2(LocalSmem& s, uint32_t m, F flags, uint16_t* out0, uint16_t* out1,
                                            uint32_t& tot0, uint32_t& tot1) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t b = (uint32_t)t * kLocalPer;
    uint32_t f0[kLocalPer], f1[kLocalPer];
    uint32_t c0 = 0, c1 = 0;
#pragma unroll
    for (int i = 0; i < kLocalPer; ++i) {
        f0[i] = f1[i] = 0;
        if (b + i < m) flags(b + i, f0[i], f1[i]);
        c0 += f0[i];
        c1 += f1[i];
    }
    uint32_t x0 = c0, x1 = c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y0 = __shfl_up_sync(0xffffffffu, x0, o), y1 = __shfl_up_sync(0xffffffffu, x1, o);
        if (lane >= o) { x0 += y0; x1 += y1; }
    }
    if (lane == 31) { s.warp_tot[warp][0] = x0; s.warp_tot[warp][1] = x1; }
    __syncthreads();
    uint32_t w0 = 0, w1 = 0, a0 = 0, a1 = 0;
    for (int w = 0; w < kLocalThreads / 32; ++w) {
        if (w < warp) { w0 += s.warp_tot[w][0]; w1 += s.warp_tot[w][1]; }
        a0 += s.warp_tot[w][0];
        a1 += s.warp_tot[w][1];
    }
    uint32_t r0 = w0 + x0 - c0, r1 = w1 + x1 - c1;
#pragma unroll
    for (int i = 0; i < kLocalPer; ++i) {
        if (b + i < m) {
            out0[b + i] = (uint16_t)r0;
            if (out1) out1[b + i] = (uint16_t)r1;
        }
        r0 += f0[i];
        r1 += f1[i];
    }
    tot0 = a0;
    tot1 = a1;
    __syncthreads();
}

// Finishes the subtree of node L0 + blockIdx.x (levels lv0 .. levels-1).
// Lists: the level-lv0 lists (axis x at list + x * S), node segments in heap
// order. Writes heap[2g], heap[2g+1] for every node g of the subtree.
__global__ void __launch_bounds__(kLocalThreads) k_local_finish(const uint32_t* __restrict__ list, size_t S,
                                                                 const float* __restrict__ mn,
                                                                 const float* __restrict__ mx, uint32_t n,
                                                                 uint32_t lv0, uint32_t L0,
                                                                 const uint32_t* __restrict__ nstart,
                                                                 uint32_t npids, uint32_t* __restrict__ lid_of,
                                                                 uint32_t* __restrict__ heap,
                                                                 float* __restrict__ sbox,
                                                                 uint32_t* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LocalSmem& s = *reinterpret_cast<LocalSmem*>(smem_raw);
    if (build_aborted(err)) return;       // whole blocks: the word does not change during this launch
    const uint32_t k = L0 + blockIdx.x;
    const int t = threadIdx.x;
    const uint32_t seg0 = nstart[k];
    const uint32_t len = (uint32_t)(2 * subtree_nodes(k, n));
    if (len > kLocalMax) {   // the host chose lv0 so that this cannot happen
        if (t == 0) atomicOr(err, 4u);
        return;
    }
    const uint32_t a0 = lv0 % 3u;
    // local ids: positions in the select axis' list
    for (uint32_t j = t; j < len; j += kLocalThreads) {
        const uint32_t gp = list[a0 * S + seg0 + j];
        s.pid[j] = gp;
        s.list[0][a0][j] = (uint16_t)j;
        s.node[j] = 0;
        lid_of[gp] = j;
    }
    __syncthreads();
    for (uint32_t j = t; j < len; j += kLocalThreads) {
#pragma unroll
        for (uint32_t x = 0; x < 3; ++x)
            if (x != a0) s.list[0][x][j] = (uint16_t)lid_of[list[x * S + seg0 + j]];
    }
    int cur = 0;
    uint32_t depth_last = 0;
    for (uint32_t d = 0;; ++d) {
        depth_last = d;
        const uint32_t lv = lv0 + d;
        const uint64_t G0 = (uint64_t)(k + 1) * (1ull << d) - 1ull;
        if (G0 >= n) break;
        const uint64_t avail = (uint64_t)n - G0;
        const uint32_t nd = (uint32_t)((1ull << d) < avail ? (1ull << d) : avail);
        const uint32_t a = lv % 3u, b = (lv + 1) % 3u, c = (lv + 2) % 3u;
        // node table of this depth: segment lengths and left sizes, offsets by a scan
        {
            uint32_t tot0, tot1;
            local_scan2(
                s, nd,
                [&](uint32_t r, uint32_t& f0, uint32_t& f1) {
                    const uint64_t g = G0 + r;
                    f0 = (uint32_t)(2 * subtree_nodes(g, n));
                    f1 = 0;
                    s.numl[r] = (uint16_t)((2 * g + 1 < n) ? 2 * subtree_nodes(2 * g + 1, n) : 0);
                },
                s.off, nullptr, tot0, tot1);
            if (t == 0) s.off[nd] = (uint16_t)tot0;
            __syncthreads();
        }
        const uint32_t m = s.off[nd];
        for (uint32_t r = t; r < nd; r += kLocalThreads) s.best[r] = 0ull;   // shares storage with the scans
        __syncthreads();
        // select: pair[0] = first of the segment on axis a, pair[1] = arg-max
        // of (max-key, lowest prim id) over the rest (k_select)
        for (uint32_t j = t; j < m; j += kLocalThreads) {
            const uint16_t lid = s.list[cur][a][j];
            const uint32_t r = lid < len ? s.node[lid] : kLocalDone;
            if (r >= nd) {   // consistency check: every listed triangle belongs to a node of this depth
                atomicOr(err, 4u);
                continue;
            }
            if (j == s.off[r]) {
                s.p0[r] = lid;
            } else {
                const uint32_t gp = s.pid[lid];
                const unsigned long long key =
                    ((unsigned long long)orderable(mx[a * S + gp]) << 32) | (unsigned long long)(0xFFFFFFFFu - gp);
                atomicMax(&s.best[r], key);
            }
        }
        __syncthreads();
        // emit (k_emit_pairs)
        for (uint32_t r = t; r < nd; r += kLocalThreads) {
            const uint32_t g = (uint32_t)(G0 + r);
            const uint32_t q0 = s.p0[r];
            const uint32_t p1 = 0xFFFFFFFFu - (uint32_t)(s.best[r] & 0xFFFFFFFFull);
            const uint32_t q1 = p1 < npids ? lid_of[p1] : kLocalMax;
            if (q0 >= len || q1 >= len) {
                atomicOr(err, 4u);
                continue;
            }
            heap[2 * g] = s.pid[q0];
            heap[2 * g + 1] = p1;
            s.node[q0] = kLocalDone;
            s.node[q1] = kLocalDone;
        }
        __syncthreads();
        if (2 * G0 + 1 >= n) break;   // no node below this depth
        const int nxt = cur ^ 1;
        // split the next axis' list: drop the pairs, rank within the node's
        // remainder decides left / right (k_split_next)
        {
            uint32_t td, tu;
            local_scan2(
                s, m,
                [&](uint32_t j, uint32_t& f0, uint32_t& f1) {
                    const uint16_t lid = s.list[cur][b][j];
                    f0 = lid < len && s.node[lid] == kLocalDone;
                    f1 = 0;
                },
                s.pre0, nullptr, td, tu);
            for (uint32_t j = t; j < m; j += kLocalThreads) {
                const uint16_t lid = s.list[cur][b][j];
                const uint32_t r = lid < len ? s.node[lid] : kLocalDone;
                if (r == kLocalDone) continue;
                if (r >= nd) {
                    atomicOr(err, 4u);
                    continue;
                }
                const uint32_t db = s.pre0[j];
                const uint32_t rpos = (j - s.off[r]) - (db - 2u * r);
                s.right[lid] = rpos < s.numl[r] ? 0 : 1;
                s.list[nxt][b][j - db] = lid;
            }
            __syncthreads();
        }
        // stable partition of the other two lists into left then right child
        // segments (k_partition)
        for (int which = 0; which < 2; ++which) {
            const uint32_t x = which == 0 ? a : c;
            uint32_t td, tl;
            local_scan2(
                s, m,
                [&](uint32_t j, uint32_t& f0, uint32_t& f1) {
                    const uint16_t lid = s.list[cur][x][j];
                    const bool done = lid >= len || s.node[lid] == kLocalDone;
                    f0 = done;
                    f1 = !done && !s.right[lid];
                },
                s.pre0, s.pre1, td, tl);
            for (uint32_t j = t; j < m; j += kLocalThreads) {
                const uint16_t lid = s.list[cur][x][j];
                const uint32_t r = lid < len ? s.node[lid] : kLocalDone;
                if (r == kLocalDone) continue;
                if (r >= nd) {
                    atomicOr(err, 4u);
                    continue;
                }
                const uint32_t o = s.off[r];
                const uint32_t base = o - 2u * r;                 // left child's segment at the next depth
                const uint32_t lb = s.pre1[j] - s.pre1[o];        // left elements of this node before j
                const uint32_t db = s.pre0[j] - s.pre0[o];        // retired elements of this node before j
                uint32_t dst;
                if (!s.right[lid]) dst = base + lb;
                else dst = base + s.numl[r] + ((j - o) - lb - db);
                if (dst < m - 2u * nd) s.list[nxt][x][dst] = lid;
                else atomicOr(err, 4u);
            }
            __syncthreads();
        }
        for (uint32_t j = t; j < len; j += kLocalThreads)
            if (s.node[j] != kLocalDone) s.node[j] = (uint16_t)(2u * s.node[j] + s.right[j]);
        __syncthreads();
        cur = nxt;
    }
    // subtree boxes of the subtree's nodes, bottom-up: the pair's bounds
    // (k_bounds' per-triangle min / max) and the children's subtree boxes,
    // written by this block one depth earlier
    for (int d = (int)depth_last; d >= 0; --d) {
        const uint64_t G0 = (uint64_t)(k + 1) * (1ull << d) - 1ull;
        const uint64_t avail = (uint64_t)n - G0;
        const uint32_t nd = (uint32_t)((1ull << d) < avail ? (1ull << d) : avail);
        for (uint32_t r = t; r < nd; r += kLocalThreads) {
            const uint32_t g = (uint32_t)(G0 + r);
            const uint32_t p = heap[2 * g], q = heap[2 * g + 1];
            float b[6];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                b[ax] = fminf(mn[ax * S + p], mn[ax * S + q]);
                b[3 + ax] = fmaxf(mx[ax * S + p], mx[ax * S + q]);
            }
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const uint32_t c = 2 * g + 1 + j;
                if (c < n) {
#pragma unroll
                    for (int ax = 0; ax < 3; ++ax) {
                        b[ax] = fminf(b[ax], sbox[6 * (size_t)c + ax]);
                        b[3 + ax] = fmaxf(b[3 + ax], sbox[6 * (size_t)c + 3 + ax]);
                    }
                }
            }
#pragma unroll
            for (int q6 = 0; q6 < 6; ++q6) sbox[6 * (size_t)g + q6] = b[q6];
        }
        __syncthreads();
    }
}

// Orders each pair by (min-key on the last level's axis, prim id).
__global__ void k_pair_order(uint32_t n, const uint32_t* __restrict__ heap, const float* __restrict__ mn_last,
                             uint32_t* __restrict__ perm, const uint32_t* err) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || build_aborted(err)) return;
    uint32_t p = heap[2 * k], q = heap[2 * k + 1];
    const float kp = mn_last[p], kq = mn_last[q];
    if (kq < kp || (kq == kp && q < p)) { const uint32_t t = p; p = q; q = t; }
    perm[2 * k] = p;
    perm[2 * k + 1] = q;
}

// applyIndices (rebuilder.cu:217-245) for the vertices, plus the traversal
// record of each node: slab of the pair on the node's axis
// (intersect.cuh:106-111) and both triangles as (v1, e1, e2). The bounding
// box of the pair goes to box[6k..6k+5] (lo.xyz, hi.xyz) for k_node_boxes.
__global__ void k_emit_nodes(const float* __restrict__ V, uint32_t count_in, const uint32_t* __restrict__ perm,
                             uint32_t n, float* __restrict__ verts, float4* __restrict__ recs,
                             float* __restrict__ box, const uint32_t* err) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || build_aborted(err)) return;
    const int a = (int)(level_of(k) % 3u);
    float c[2][9];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const uint32_t pid = perm[2 * k + t];
        const uint32_t src = pid < count_in ? pid : count_in - 1;
        const float* v = V + (size_t)src * 9;
        float* o = verts + (size_t)(2 * k + t) * 9;
#pragma unroll
        for (int q = 0; q < 9; ++q) { c[t][q] = v[q]; o[q] = c[t][q]; }
    }
    float blo[3], bhi[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        blo[ax] = fminf(fminf(fminf(c[0][3 * ax], c[0][3 * ax + 1]), c[0][3 * ax + 2]),
                        fminf(fminf(c[1][3 * ax], c[1][3 * ax + 1]), c[1][3 * ax + 2]));
        bhi[ax] = fmaxf(fmaxf(fmaxf(c[0][3 * ax], c[0][3 * ax + 1]), c[0][3 * ax + 2]),
                        fmaxf(fmaxf(c[1][3 * ax], c[1][3 * ax + 1]), c[1][3 * ax + 2]));
        box[6 * (size_t)k + ax] = blo[ax];
        box[6 * (size_t)k + 3 + ax] = bhi[ax];
    }
    float r[20];
    r[0] = a == 0 ? blo[0] : (a == 1 ? blo[1] : blo[2]);
    r[1] = a == 0 ? bhi[0] : (a == 1 ? bhi[1] : bhi[2]);
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        // layout [x1 x2 x3 y1 y2 y3 z1 z2 z3]: v1 = (c0, c3, c6), v2 = (c1, c4, c7), v3 = (c2, c5, c8)
        float* o = r + 2 + 9 * t;
        o[0] = c[t][0]; o[1] = c[t][3]; o[2] = c[t][6];
        o[3] = c[t][1] - c[t][0]; o[4] = c[t][4] - c[t][3]; o[5] = c[t][7] - c[t][6];
        o[6] = c[t][2] - c[t][0]; o[7] = c[t][5] - c[t][3]; o[8] = c[t][8] - c[t][6];
    }
    float4* rec = recs + (size_t)k * kRecStride;
#pragma unroll
    for (int q = 0; q < 5; ++q) rec[q] = make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
}

// Box padding: relative 1e-5 of the coordinates' magnitude, far above the
// rounding of the triangle test and of the box test.
__device__ __forceinline__ void pad_interval(float lo, float hi, float& plo, float& phi) {
    const float p = 1e-5f * (fabsf(lo) + fabsf(hi)) + 1e-30f;
    plo = lo - p;
    phi = hi + p;
}

// Nodes [L0, L1) (kUnion: one heap level, bottom-up): with kUnion, sbox[k]
// becomes the bounding box of node k's subtree (its pair's box pbox[k] and
// its children's subtree boxes, computed one launch earlier); in both forms
// the padded subtree boxes of the children go into record words 5..7 of
// node k (an empty box where a child does not exist).
template <bool kUnion>
__global__ void k_node_boxes(uint32_t L0, uint32_t L1, uint32_t n, const float* __restrict__ pbox,
                             float* __restrict__ box, float4* __restrict__ recs, const uint32_t* err) {
    const uint32_t k = L0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L1 || build_aborted(err)) return;
    float b[6];
    if (kUnion) {
#pragma unroll
        for (int q = 0; q < 6; ++q) b[q] = pbox[6 * (size_t)k + q];
    }
    float cb[2][6];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const uint32_t c = 2 * k + 1 + j;
        if (c < n) {
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                const float lo = box[6 * (size_t)c + ax], hi = box[6 * (size_t)c + 3 + ax];
                b[ax] = fminf(b[ax], lo);
                b[3 + ax] = fmaxf(b[3 + ax], hi);
                pad_interval(lo, hi, cb[j][ax], cb[j][3 + ax]);
            }
        } else {
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) { cb[j][ax] = 1.0f; cb[j][3 + ax] = -1.0f; }
        }
    }
    if (kUnion) {
#pragma unroll
        for (int q = 0; q < 6; ++q) box[6 * (size_t)k + q] = b[q];
    }
    float4* rec = recs + (size_t)k * kRecStride + 5;
    rec[0] = make_float4(cb[0][0], cb[0][1], cb[0][2], cb[0][3]);
    rec[1] = make_float4(cb[0][4], cb[0][5], cb[1][0], cb[1][1]);
    rec[2] = make_float4(cb[1][2], cb[1][3], cb[1][4], cb[1][5]);
}

inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

uint32_t log2i(uint32_t x) {
    uint32_t r = (uint32_t)(-1);
    while (x) { x >>= 1; r++; }
    return r;
}

// Look-back scratch: per list (the split list and the two partitioned ones)
// one status word per tile, then the three tile counters.
constexpr size_t lookback_bytes(size_t ntiles) { return 3 * ntiles * sizeof(unsigned long long) + 16; }

// ------------------------------------------------------------ launch sequence
//
// The launches of one build go through a Seq, which either issues them on a
// stream, or records them as a linear chain of CUDA graph nodes, or replays
// the same sequence against such a recording and writes into its
// instantiated graph only the arguments that differ (another vertex array,
// other output buffers: the next build of the same size). A build makes six
// launches per global level plus 20 (74 at 1M triangles); recorded once and
// then launched as one graph they no longer wait on the host's per-launch
// cost.
struct NodeRec {
    cudaGraphNode_t node = nullptr;
    const void* func = nullptr;          // null for a memset node
    dim3 grid, block;
    unsigned smem = 0;
    std::vector<unsigned char> args;     // packed kernel arguments, or (target, bytes) of a memset
};

class Seq {
public:
    enum Mode { kDirect, kRecord, kPatch };

    static Seq direct(cudaStream_t st) { Seq q; q.mode_ = kDirect; q.st_ = st; return q; }
    static Seq record(cudaGraph_t g, std::vector<NodeRec>* nodes) {
        Seq q; q.mode_ = kRecord; q.g_ = g; q.nodes_ = nodes; nodes->clear(); return q;
    }
    static Seq patch(cudaGraphExec_t exec, std::vector<NodeRec>* nodes) {
        Seq q; q.mode_ = kPatch; q.exec_ = exec; q.nodes_ = nodes; return q;
    }

    template <typename... P, typename... A>
    void launch(void (*k)(P...), dim3 grid, dim3 block, size_t smem, A... a) {
        static_assert(sizeof...(P) == sizeof...(A), "kernel argument count");
        if (err_ != cudaSuccess) return;
        if (mode_ == kDirect) {
            k<<<grid, block, smem, st_>>>(static_cast<P>(a)...);
            return;
        }
        std::vector<unsigned char> buf;
        size_t offs[sizeof...(P) + 1];
        size_t i = 0;
        (put<P>(buf, offs[i++], static_cast<P>(a)), ...);
        void* ptrs[sizeof...(P) + 1];
        for (size_t j = 0; j < sizeof...(P); ++j) ptrs[j] = buf.data() + offs[j];
        cudaKernelNodeParams p = {};
        p.func = (void*)k;
        p.gridDim = grid;
        p.blockDim = block;
        p.sharedMemBytes = (unsigned)smem;
        p.kernelParams = ptrs;
        if (mode_ == kRecord) {
            NodeRec r;
            err_ = cudaGraphAddKernelNode(&r.node, g_, last_ ? &last_ : nullptr, last_ ? 1 : 0, &p);
            if (err_ != cudaSuccess) return;
            last_ = r.node;
            r.func = p.func; r.grid = grid; r.block = block; r.smem = p.sharedMemBytes;
            r.args = std::move(buf);
            nodes_->push_back(std::move(r));
            return;
        }
        if (next_ >= nodes_->size()) { err_ = cudaErrorInvalidValue; return; }
        NodeRec& r = (*nodes_)[next_++];
        if (r.func != p.func || !same(r.grid, grid) || !same(r.block, block) || r.smem != p.sharedMemBytes ||
            r.args.size() != buf.size()) {
            err_ = cudaErrorInvalidValue;
            return;
        }
        if (r.args != buf) {
            err_ = cudaGraphExecKernelNodeSetParams(exec_, r.node, &p);
            if (err_ == cudaSuccess) r.args = std::move(buf);
        }
    }

    // Zeroes `bytes` (a multiple of 4) at p.
    void memset(void* p, size_t bytes) {
        if (err_ != cudaSuccess) return;
        if (mode_ == kDirect) {
            err_ = cudaMemsetAsync(p, 0, bytes, st_);
            return;
        }
        cudaMemsetParams m = {};
        m.dst = p;
        m.value = 0;
        m.elementSize = 4;
        m.width = bytes / 4;
        m.height = 1;
        std::vector<unsigned char> key(sizeof(void*) + sizeof(size_t));
        std::memcpy(key.data(), &p, sizeof(void*));
        std::memcpy(key.data() + sizeof(void*), &bytes, sizeof(size_t));
        if (mode_ == kRecord) {
            NodeRec r;
            err_ = cudaGraphAddMemsetNode(&r.node, g_, last_ ? &last_ : nullptr, last_ ? 1 : 0, &m);
            if (err_ != cudaSuccess) return;
            last_ = r.node;
            r.args = std::move(key);
            nodes_->push_back(std::move(r));
            return;
        }
        if (next_ >= nodes_->size() || (*nodes_)[next_].func != nullptr) { err_ = cudaErrorInvalidValue; return; }
        NodeRec& r = (*nodes_)[next_++];
        if (r.args != key) {
            err_ = cudaGraphExecMemsetNodeSetParams(exec_, r.node, &m);
            if (err_ == cudaSuccess) r.args = std::move(key);
        }
    }

    // First error of the sequence: a failed launch or node call, or (when
    // patching) a sequence that does not match the recording.
    cudaError_t finish() {
        if (err_ == cudaSuccess && mode_ == kDirect) err_ = cudaGetLastError();
        if (err_ == cudaSuccess && mode_ == kPatch && next_ != nodes_->size()) err_ = cudaErrorInvalidValue;
        return err_;
    }

private:
    template <typename T>
    static void put(std::vector<unsigned char>& b, size_t& off, const T& v) {
        off = (b.size() + alignof(T) - 1) & ~(alignof(T) - 1);
        b.resize(off + sizeof(T));
        std::memcpy(b.data() + off, &v, sizeof(T));
    }
    static bool same(const dim3& a, const dim3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

    Mode mode_ = kDirect;
    cudaStream_t st_ = nullptr;
    cudaGraph_t g_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    cudaGraphNode_t last_ = nullptr;
    std::vector<NodeRec>* nodes_ = nullptr;
    size_t next_ = 0;
    cudaError_t err_ = cudaSuccess;
};

// One level's split of the next axis' list and partition of the other two,
// each a single pass with look-back tile prefixes; the status words and
// tile counters are cleared first.
void split_and_partition(Seq& q, const ListSet& sb, const ListSet& sac, uint32_t M, uint32_t mt, uint32_t ntiles,
                         uint32_t* node_of, const uint32_t* ns, const uint32_t* nl, const uint32_t* nlb, uint32_t L0,
                         uint32_t m_next, unsigned long long* lb, uint32_t* err, uint32_t test) {
    uint32_t* counters = reinterpret_cast<uint32_t*>(lb + 3 * (size_t)ntiles);
    q.memset(lb, lookback_bytes(ntiles));
    q.launch(k_split_next, dim3(mt), dim3(kThreads), 0, sb, M, node_of, ns, nl, L0, lb, counters, err, test);
    q.launch(k_partition, dim3(mt, 2), dim3(kThreads), 0, sac, M, node_of, ns, nl, nlb, L0, lb + ntiles, ntiles,
             counters + 1, m_next, err, test);
}

// First level whose node segments all fit k_local_finish (the leftmost
// subtree of a level of a complete heap is its largest).
uint32_t local_level(uint32_t n, uint32_t levels) {
    for (uint32_t lv = 0; lv < levels; ++lv)
        if (2 * subtree_nodes((1ull << lv) - 1ull, n) <= kLocalMax) return lv;
    return levels;
}

// The remaining levels lv0 .. levels-1, one block per node of level lv0.
void finish_local(Seq& q, const uint32_t* list, size_t S, const float* mn, const float* mx, uint32_t n, uint32_t lv0,
                  const uint32_t* nstart, uint32_t* node_of, uint32_t* heap, float* sbox, uint32_t* err) {
    const uint32_t L0 = (1u << lv0) - 1u;
    const uint32_t L1 = ((2u << lv0) - 1u) < n ? ((2u << lv0) - 1u) : n;
    q.launch(k_local_finish, dim3(L1 - L0), dim3(kLocalThreads), sizeof(LocalSmem), list, S, mn, mx, n, lv0, L0,
             nstart, 2 * n, node_of, heap, sbox, err);
}

// Node records: pairs and slabs, then the children's subtree boxes. The
// subtree boxes of levels >= lv0 are in sbox already (k_local_finish); the
// levels above are unions, level by level from the bottom, of the pair boxes
// (pbox, written by k_emit_nodes) and the children's subtree boxes.
// pbox and sbox: 6 floats per node of scratch each.
void emit_records(Seq& q, const float* V, uint32_t count, const uint32_t* perm, uint32_t n, uint32_t lv0,
                  float* verts, float4* recs, float* pbox, float* sbox, const uint32_t* err) {
    q.launch(k_emit_nodes, dim3(cdiv(n, 128)), dim3(128), 0, V, count, perm, n, verts, recs, pbox, err);
    const uint32_t Lb = (1u << lv0) - 1u;   // first node of level lv0
    if (Lb < n)
        q.launch(k_node_boxes<false>, dim3(cdiv(n - Lb, 256)), dim3(256), 0, Lb, n, n, pbox, sbox, recs, err);
    for (int lv = (int)lv0 - 1; lv >= 0; --lv) {
        const uint32_t L0 = (1u << lv) - 1u;
        const uint32_t L1 = ((2u << lv) - 1u) < n ? ((2u << lv) - 1u) : n;
        q.launch(k_node_boxes<true>, dim3(cdiv(L1 - L0, 256)), dim3(256), 0, L0, L1, n, pbox, sbox, recs, err);
    }
}

constexpr size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// Byte offsets of the scratch regions of a build of N (even) triangles; the
// per-axis arrays use a stride S that keeps every axis 256-byte aligned.
struct ScratchLayout {
    size_t S, flags, mn, mx, keys, vals, k2, v2, nodeof, heap, pair0, best, ns, nl, nlb, tiles, hist, tot, end;
};

constexpr ScratchLayout scratch_layout(size_t N) {
    ScratchLayout L{};
    const size_t n = N / 2;
    const size_t nb = (N + kSortTile - 1) / kSortTile;
    const size_t ntiles = (N + kTile - 1) / kTile;
    L.S = (N + 63) & ~(size_t)63;
    size_t off = 0;
    L.flags = off; off += round256(4);
    L.mn = off; off += round256(3 * L.S * 4);
    L.mx = off; off += round256(3 * L.S * 4);
    L.keys = off; off += round256(3 * L.S * 4);
    L.vals = off; off += round256(3 * L.S * 4);
    L.k2 = off; off += round256(3 * L.S * 4);
    L.v2 = off; off += round256(3 * L.S * 4);
    L.nodeof = off; off += round256(N * 4);
    L.heap = off; off += round256(N * 4);
    L.pair0 = off; off += round256(n * 4);
    L.best = off; off += round256(n * 8);
    L.ns = off; off += round256(n * 4);
    L.nl = off; off += round256(n * 4);
    L.nlb = off; off += round256(n * 4);
    L.tiles = off; off += round256(lookback_bytes(ntiles));
    L.hist = off; off += round256(3 * 256 * nb * 4);
    L.tot = off; off += round256(3 * 256 * 4);
    L.end = off;
    return L;
}

// Everything one build reads and writes.
struct BuildArgs {
    const float* V;
    uint32_t count;            // input triangles; N = count rounded up to even
    float4* recs;
    uint32_t* perm;
    float* verts;
    unsigned char* scratch;    // scratch_layout(N).end bytes
    uint32_t* flags;           // error bits 4 (internal check), 8 (non-finite vertex), 16 (look-back timeout)
    uint32_t lookback_test = 0;  // test hook: nonzero makes the look-back waits run out (see tile_lookback)
};

// The whole build of a non-empty soup: bounds and keys, three radix sorts,
// the global levels, the per-subtree finish, pair order and node records.
void enqueue_build(Seq& q, const BuildArgs& b) {
    const uint32_t N = b.count + (b.count & 1u);
    const uint32_t n = N / 2;
    const uint32_t levels = log2i(n) + 1;
    const ScratchLayout L = scratch_layout(N);
    const size_t S = L.S;
    unsigned char* base = b.scratch;
    float* mn = (float*)(base + L.mn);
    float* mx = (float*)(base + L.mx);
    uint32_t* keys = (uint32_t*)(base + L.keys);
    uint32_t* vals = (uint32_t*)(base + L.vals);
    uint32_t* k2 = (uint32_t*)(base + L.k2);
    uint32_t* v2 = (uint32_t*)(base + L.v2);
    uint32_t* node_of = (uint32_t*)(base + L.nodeof);
    uint32_t* heap = (uint32_t*)(base + L.heap);
    uint32_t* pair0 = (uint32_t*)(base + L.pair0);
    unsigned long long* best = (unsigned long long*)(base + L.best);
    uint32_t* ns = (uint32_t*)(base + L.ns);
    uint32_t* nl = (uint32_t*)(base + L.nl);
    uint32_t* nlb = (uint32_t*)(base + L.nlb);
    unsigned long long* tiles = (unsigned long long*)(base + L.tiles);
    uint32_t* hist = (uint32_t*)(base + L.hist);
    uint32_t* tot = (uint32_t*)(base + L.tot);
    const uint32_t nb = cdiv(N, kSortTile);
    const uint32_t ntiles = cdiv(N, kTile);

    q.memset(node_of, (size_t)N * 4);
    q.memset(best, (size_t)n * 8);
    q.launch(k_bounds, dim3(cdiv(N, 256)), dim3(256), 0, b.V, N, S, b.count, mn, mx, keys, vals, b.flags);
    // three stable LSD radix sorts of (min-key, prim id); result in keys/vals
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = pass * 8;
        uint32_t* kin = (pass & 1) ? k2 : keys;
        uint32_t* vin = (pass & 1) ? v2 : vals;
        uint32_t* kout = (pass & 1) ? keys : k2;
        uint32_t* vout = (pass & 1) ? vals : v2;
        q.launch(k_radix_hist, dim3(nb, 3), dim3(kThreads), 0, kin, N, S, shift, hist, nb);
        q.launch(k_radix_scan_rows, dim3(256, 3), dim3(1024), 0, hist, nb, tot);
        q.launch(k_radix_scatter, dim3(nb, 3), dim3(kThreads), 0, kin, vin, kout, vout, N, S, shift, hist, tot, nb,
                 b.flags);
    }
    // lists: vals = sorted pids per axis (buffer A), v2 = buffer B
    uint32_t* listA = vals;
    uint32_t* listB = v2;
    q.launch(k_node_table, dim3(cdiv(n, 256)), dim3(256), 0, n, ns, nl, nlb);

    // levels above lv0 over the whole soup, the rest per subtree in shared memory
    const uint32_t lv0 = local_level(n, levels);
    for (uint32_t lv = 0; lv < lv0; ++lv) {
        const uint32_t L0 = (1u << lv) - 1u;
        const uint32_t L1 = ((2u << lv) - 1u) < n ? ((2u << lv) - 1u) : n;
        const uint32_t M = N - 2u * L0;
        const int a = (int)(lv % 3), bx = (int)((lv + 1) % 3), c = (int)((lv + 2) % 3);
        const uint32_t mt = cdiv(M, kTile);
        // each node's pair: its segment's first entry and the entry of largest max-key (k_select),
        // written to the heap (k_emit_pairs)
        q.launch(k_select, dim3(cdiv(M, (uint32_t)kThreads * kSelectItems)), dim3(kThreads), 0, listA + a * S, M,
                 mx + a * S, node_of, ns, L0, best, pair0, b.flags);
        q.launch(k_emit_pairs, dim3(cdiv(L1 - L0, 256)), dim3(256), 0, L0, L1, best, pair0, heap, node_of, b.flags);
        if (lv + 1 == levels) break;
        ListSet sb;
        sb.in[0] = listA + bx * S; sb.out[0] = listB + bx * S;
        sb.in[1] = nullptr; sb.out[1] = nullptr;
        ListSet sac;
        sac.in[0] = listA + a * S; sac.out[0] = listB + a * S;
        sac.in[1] = listA + c * S; sac.out[1] = listB + c * S;
        split_and_partition(q, sb, sac, M, mt, ntiles, node_of, ns, nl, nlb, L0, M - 2u * (L1 - L0), tiles, b.flags,
                            b.lookback_test);
        uint32_t* t = listA; listA = listB; listB = t;
    }
    if (lv0 < levels) finish_local(q, listA, S, mn, mx, n, lv0, ns, node_of, heap, (float*)k2, b.flags);
    const int al = (int)((levels - 1) % 3);
    q.launch(k_pair_order, dim3(cdiv(n, 256)), dim3(256), 0, n, heap, mn + al * S, b.perm, b.flags);
    // mx and k2 are free once the levels are placed: 3*S >= 6*n floats each for the boxes
    emit_records(q, b.V, b.count, b.perm, n, lv0, b.verts, b.recs, mx, (float*)k2, b.flags);
}

// Error bits of a finished build, read back on `st`.
aur_status build_flags(const char* who, uint32_t* d_flags, cudaStream_t st, bool clear) {
    uint32_t flags = 0;
    AUR_CUDA(cudaMemcpyAsync(&flags, d_flags, 4, cudaMemcpyDeviceToHost, st));
    AUR_CUDA(cudaStreamSynchronize(st));
    if (!(flags & (4u | 8u | 16u))) return AUR_OK;
    if (clear) {
        cudaMemsetAsync(d_flags, 0, 4, st);
        cudaStreamSynchronize(st);
    }
    if (flags & 8u) return fail(AUR_ERR_INVALID, "%s: a vertex coordinate is NaN or infinite", who);
    if (flags & 16u) return fail(AUR_ERR_TIMEOUT, "%s: a tile prefix wait gave up (flags 0x%x)", who, flags);
    return fail(AUR_ERR_CUDA, "%s: internal partition check failed (flags 0x%x)", who, flags);
}

cudaError_t set_local_smem() {
    return cudaFuncSetAttribute(k_local_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(LocalSmem));
}

}  // namespace

// A context's cached build: its scratch, and the launch sequences of up to
// kCachedGraphs sizes recorded as CUDA graphs. The first build of a size
// launches directly; a size built again (as when cudaRebuildNMH runs every
// frame) is recorded, and later builds of it launch the graph with the
// changed arguments patched in. Soups of at most kGraphMaxTriangles use the
// cache; larger ones (whose kernels dwarf the launch cost) launch directly
// with stream-ordered scratch that is released after the build.
constexpr uint32_t kGraphMaxTriangles = 1u << 24;
constexpr int kCachedGraphs = 4;
constexpr int kSeenSizes = 8;

struct BuildGraph {
    uint32_t N = 0;                        // size the graph was recorded for
    uint64_t used = 0;                     // last use, for eviction
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<NodeRec> nodes;

    void drop() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        nodes.clear();
        N = 0;
        used = 0;
    }
};

struct BuildCache {
    std::mutex mutex;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    BuildGraph graphs[kCachedGraphs];
    uint32_t seen[kSeenSizes] = {};        // sizes built directly, most recent last written
    int seen_next = 0;
    uint64_t clock = 0;
    cudaEvent_t done = nullptr;            // recorded after each build launched from the cache
};

void free_build_cache(aur_ctx* ctx) {
    BuildCache* bc = ctx->build;
    if (!bc) return;
    if (bc->done) {
        cudaEventSynchronize(bc->done);
        cudaEventDestroy(bc->done);
    }
    for (BuildGraph& g : bc->graphs) g.drop();
    cudaFree(bc->scratch);
    delete bc;
    ctx->build = nullptr;
}

namespace {

// Runs the build from the context's cache: the recorded graph of this size,
// patched; or a new recording, when the size was built before; or direct
// launches on the cached scratch.
aur_status build_cached(aur_ctx* ctx, const BuildArgs& a0, uint32_t N, cudaStream_t st) {
    if (!ctx->build) ctx->build = new BuildCache();
    BuildCache& bc = *ctx->build;
    std::lock_guard<std::mutex> lock(bc.mutex);
    if (!bc.done) AUR_CUDA(cudaEventCreateWithFlags(&bc.done, cudaEventDisableTiming));
    const size_t need = scratch_layout(N).end;
    if (bc.scratch_bytes < need) {
        AUR_CUDA(cudaEventSynchronize(bc.done));   // the last build may still use the old scratch
        cudaFree(bc.scratch);
        bc.scratch = nullptr;
        bc.scratch_bytes = 0;
        if (::aur::dev_malloc(&bc.scratch, need) != cudaSuccess) {
            cudaGetLastError();
            return fail(AUR_ERR_OOM, "aur_nmh_build: out of device memory for %zu bytes of scratch", need);
        }
        bc.scratch_bytes = need;
    }
    BuildArgs a = a0;
    a.scratch = (unsigned char*)bc.scratch;
    AUR_CUDA(cudaStreamWaitEvent(st, bc.done, 0));
    AUR_CUDA(set_local_smem());
    BuildGraph* g = nullptr;
    for (BuildGraph& c : bc.graphs)
        if (c.exec && c.N == N) g = &c;
    if (g) {
        Seq q = Seq::patch(g->exec, &g->nodes);
        enqueue_build(q, a);
        if (q.finish() != cudaSuccess) {
            cudaGetLastError();
            g->drop();
            g = nullptr;
        }
    } else {
        bool seen = false;
        for (uint32_t x : bc.seen) seen = seen || x == N;
        if (!seen) {
            bc.seen[bc.seen_next] = N;
            bc.seen_next = (bc.seen_next + 1) % kSeenSizes;
            Seq q = Seq::direct(st);
            enqueue_build(q, a);
            AUR_CUDA(q.finish());
            AUR_CUDA(cudaEventRecord(bc.done, st));
            return AUR_OK;
        }
    }
    if (!g) {
        g = &bc.graphs[0];
        for (BuildGraph& c : bc.graphs)
            if (c.used < g->used) g = &c;
        g->drop();
        AUR_CUDA(cudaGraphCreate(&g->graph, 0));
        Seq q = Seq::record(g->graph, &g->nodes);
        enqueue_build(q, a);
        cudaError_t e = q.finish();
        if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (e != cudaSuccess) {
            cudaGetLastError();
            g->drop();
            return cuda_fail(e, "aur_nmh_build (recording the build graph)", __FILE__, __LINE__);
        }
        g->N = N;
    }
    g->used = ++bc.clock;
    AUR_CUDA(cudaGraphLaunch(g->exec, st));
    AUR_CUDA(cudaEventRecord(bc.done, st));
    return AUR_OK;
}

}  // namespace

// Largest side of the box around the root's two triangles (v1, v1 + e1,
// v1 + e2) and its children's padded subtree boxes: the whole soup's bounds,
// up to the padding and the rounding of v1 + e.
static float record_extent(const float* r, uint32_t nodes) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    auto add = [&](int a, float v) {
        if (v == v) { lo[a] = std::min(lo[a], v); hi[a] = std::max(hi[a], v); }
    };
    for (int t = 0; t < 2; ++t) {
        const float* q = r + 2 + 9 * t;    // v1, e1, e2
        for (int a = 0; a < 3; ++a) {
            add(a, q[a]);
            add(a, q[a] + q[3 + a]);
            add(a, q[a] + q[6 + a]);
        }
    }
    for (uint32_t j = 0; j < 2; ++j)
        if (1 + j < nodes)
            for (int a = 0; a < 3; ++a) {
                add(a, r[20 + 6 * j + a]);
                add(a, r[20 + 6 * j + 3 + a]);
            }
    float e = 0.0f;
    for (int a = 0; a < 3; ++a)
        if (hi[a] >= lo[a]) e = std::max(e, hi[a] - lo[a]);
    return std::isfinite(e) ? e : 0.0f;
}

aur_status nmh_build_impl(aur_ctx* ctx, const float* V, uint32_t count, aur_nmh** out) {
    AUR_CHECK(ctx && out, AUR_ERR_INVALID, "aur_nmh_build: null context or output pointer");
    AUR_CHECK(count == 0 || V, AUR_ERR_INVALID, "aur_nmh_build: null vertices for %u triangles", count);
    AUR_CHECK(count < kMaxTriangles, AUR_ERR_INVALID, "aur_nmh_build: %u triangles exceed the limit of %u", count,
              kMaxTriangles - 1);
    AUR_CUDA(cudaSetDevice(ctx->device));
    const uint32_t N = count + (count & 1u);
    const uint32_t n = N / 2;
    aur_nmh* nmh = new aur_nmh();
    nmh->device = ctx->device;
    nmh->count = N;
    nmh->input_count = count;
    nmh->nodes = n;
    nmh->levels = n ? log2i(n) + 1 : 0;
    if (N == 0) { *out = nmh; return AUR_OK; }

    auto cleanup = [&]() {
        cudaFree(nmh->mem);
        delete nmh;
    };
    // records, permutation and vertices in one allocation (records first: 128-byte aligned)
    const size_t b_recs = ((size_t)n * kRecStride * sizeof(float4) + 255) & ~(size_t)255;
    const size_t b_perm = ((size_t)N * sizeof(uint32_t) + 255) & ~(size_t)255;
    if (::aur::dev_malloc(&nmh->mem, b_recs + b_perm + (size_t)N * 9 * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return fail(AUR_ERR_OOM, "aur_nmh_build: out of device memory for %u triangles", N);
    }
    nmh->node_recs = (float4*)nmh->mem;
    nmh->perm = (uint32_t*)((char*)nmh->mem + b_recs);
    nmh->verts = (float*)((char*)nmh->mem + b_recs + b_perm);

    cudaStream_t st = ctx->stream;
    BuildArgs a{V, count, nmh->node_recs, nmh->perm, nmh->verts, nullptr, ctx->d_flags};
    a.lookback_test = ctx->lookback_test;     // armed for this one build only
    ctx->lookback_test = 0;
    if (N <= kGraphMaxTriangles) {
        const aur_status s = build_cached(ctx, a, N, st);
        if (s != AUR_OK) {
            cleanup();
            return s;
        }
    } else {
        const size_t need = scratch_layout(N).end;
        if (::aur::dev_malloc_async((void**)&a.scratch, need, st) != cudaSuccess) {
            cudaGetLastError();
            cleanup();
            return fail(AUR_ERR_OOM, "aur_nmh_build: out of device memory for %zu bytes of scratch", need);
        }
        cudaError_t e = set_local_smem();
        if (e == cudaSuccess) {
            Seq q = Seq::direct(st);
            enqueue_build(q, a);
            e = q.finish();
        }
        cudaFreeAsync(a.scratch, st);
        if (e != cudaSuccess) {
            cleanup();
            return cuda_fail(e, "aur_nmh_build kernels", __FILE__, __LINE__);
        }
    }
    float root[32];    // the root's record, read back with the flags (build_flags synchronizes the stream)
    AUR_CUDA(cudaMemcpyAsync(root, nmh->node_recs, sizeof(root), cudaMemcpyDeviceToHost, st));
    const aur_status s = build_flags("aur_nmh_build", ctx->d_flags, st, true);
    if (s != AUR_OK) {
        cudaGetLastError();
        cleanup();
        return s;
    }
    nmh->extent = record_extent(root, n);
    // the records as a linear float4 texture for k_trace (when they fit one);
    // without it k_trace reads every sector with plain loads
    int max_linear = 0;
    if (cudaDeviceGetAttribute(&max_linear, cudaDevAttrMaxTexture1DLinearWidth, ctx->device) == cudaSuccess &&
        (uint64_t)n * kRecStride <= (uint64_t)max_linear) {
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeLinear;
        rd.res.linear.devPtr = nmh->node_recs;
        rd.res.linear.desc = cudaCreateChannelDesc<float4>();
        rd.res.linear.sizeInBytes = (size_t)n * kRecStride * sizeof(float4);
        cudaTextureDesc td = {};
        td.readMode = cudaReadModeElementType;
        if (cudaCreateTextureObject(&nmh->rec_tex, &rd, &td, nullptr) != cudaSuccess) {
            cudaGetLastError();
            nmh->rec_tex = 0;
        }
    }
    *out = nmh;
    return AUR_OK;
}


// ------------------------------------------------ allocation-free variant
//
// aur_nmh_build_noalloc runs the same kernels as aur_nmh_build, but takes all
// of its scratch from one file-scope device array sized for
// kNoAllocMaxTriangles triangles, and writes into buffers the caller owns.
// It exists for callers that cannot allocate device memory themselves: a
// plug-in whose host application owns the GPU's memory budget and hands out
// fixed buffers, or a render loop that must not pay for cudaMalloc/cudaFree
// (which can synchronize the whole device). The array is part of the loaded
// library, so every GPU that loads the library holds it until the process
// exits.
namespace {

constexpr uint32_t kNoAllocMaxTriangles = 1u << 16;
constexpr size_t kNoAllocScratchBytes = scratch_layout(kNoAllocMaxTriangles).end;

// Shared by every call on a device; see aur_nmh_build_noalloc.
static __device__ __align__(256) unsigned char g_nmh_scratch[kNoAllocScratchBytes];

// Device address of g_nmh_scratch per device, looked up once per device with
// that device current (the host-side name of the array is not a device
// address). A cudaDeviceReset of the device makes the kept address stale; the
// header tells callers not to use this entry point on a device after a reset.
constexpr int kMaxDevices = 64;
unsigned char* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

aur_status noalloc_scratch(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_nmh_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_nmh_scratch)", __FILE__, __LINE__);
        g_scratch_addr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[device];
    return AUR_OK;
}

}  // namespace

aur_status nmh_build_noalloc_impl(const float* V, uint32_t count, cudaStream_t st, float4* recs, uint32_t* perm,
                                  float* verts, uint32_t* levels_out) {
    AUR_CHECK(count == 0 || (V && recs && perm && verts), AUR_ERR_INVALID,
              "aur_nmh_build_noalloc: null vertex or output pointer for %u triangles", count);
    AUR_CHECK(count <= kNoAllocMaxTriangles, AUR_ERR_INVALID,
              "aur_nmh_build_noalloc: %u triangles exceed this entry point's fixed scratch for %u triangles; "
              "use aur_nmh_build for larger soups", count, kNoAllocMaxTriangles);
    AUR_CHECK(((uintptr_t)recs & 31) == 0, AUR_ERR_INVALID, "aur_nmh_build_noalloc: node_records must be 32-byte aligned");
    const uint32_t N = count + (count & 1u);
    const uint32_t n = N / 2;
    const uint32_t levels = n ? log2i(n) + 1 : 0;
    if (levels_out) *levels_out = levels;
    if (N == 0) return AUR_OK;
    int device = 0;
    AUR_CUDA(cudaGetDevice(&device));
    AUR_CHECK(device >= 0 && device < kMaxDevices, AUR_ERR_INVALID, "aur_nmh_build_noalloc: device %d", device);
    unsigned char* base = nullptr;
    aur_status stt = noalloc_scratch(device, &base);
    if (stt != AUR_OK) return stt;
    uint32_t* flags = (uint32_t*)(base + scratch_layout(N).flags);
    // The array keeps the previous call's contents: the flags must start at
    // zero (enqueue_build clears the rest that must).
    AUR_CUDA(cudaMemsetAsync(flags, 0, 4, st));
    AUR_CUDA(set_local_smem());
    Seq q = Seq::direct(st);
    enqueue_build(q, BuildArgs{V, count, recs, perm, verts, base, flags});
    const cudaError_t e = q.finish();
    if (e != cudaSuccess) {
        cudaGetLastError();     // a failed launch leaves a non-sticky error behind, as in aur_nmh_build
        return cuda_fail(e, "aur_nmh_build_noalloc kernels", __FILE__, __LINE__);
    }
    return build_flags("aur_nmh_build_noalloc", flags, st, false);
}

}  // namespace aur

extern "C" {

/* Layout helper exposed for host-side tests of the closed forms:
 * out[0] = segment start, out[1] = left-child triangles, out[2] = left base
 * of node k in a heap of n nodes. Pure host code, no device needed. */
aur_status aur_debug_nmh_layout(uint32_t n, uint32_t k, uint32_t out[3]) {
    if (!out || k >= n) return aur::fail(AUR_ERR_INVALID, "aur_debug_nmh_layout: k >= n");
    const uint32_t L0 = (1u << aur::level_of(k)) - 1u;
    out[0] = (uint32_t)aur::segment_start(k, L0, n);
    out[1] = (2u * k + 1u < n) ? (uint32_t)(2 * aur::subtree_nodes(2u * k + 1u, n)) : 0u;
    out[2] = (uint32_t)aur::left_base(k, L0, n);
    return AUR_OK;
}

/* Test hook: the next aur_nmh_build on ctx makes its look-back waits run out. */
aur_status aur_debug_lookback_timeout(aur_ctx* ctx, uint32_t spins) {
    aur::clear_error();
    AUR_CHECK(ctx, AUR_ERR_INVALID, "aur_debug_lookback_timeout: null context");
    ctx->lookback_test = spins;
    return AUR_OK;
}

/* Allocation-free NMH build; see include/aurora_gb300.h. */
aur_status aur_nmh_build_noalloc(const float* vertices, uint32_t count, void* cuda_stream, float* node_records,
                                 uint32_t* perm, float* nmh_vertices, uint32_t* levels) {
    aur::clear_error();
    return aur::nmh_build_noalloc_impl(vertices, count, (cudaStream_t)cuda_stream,
                                       reinterpret_cast<float4*>(node_records), perm, nmh_vertices, levels);
}

}  // extern "C"
