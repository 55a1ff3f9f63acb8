// emitters.cu — the emissive-triangle table of a scene (cudaCreateEmitters,
// kernels/emitter.cu:39-119): every triangle whose shader has emission > 0,
// in NMH order, with its area, pdf = 1 / area, power = the shader's
// emission colour, and a CDF over the emission weights normalised to 1.
//
// Three passes over tiles of kEmTile elements, deterministic throughout:
// compaction (tile counts, one-block scan of the counts, ordered scatter,
// as thrust::copy_if keeps order), then the emitter records, then an
// inclusive scan of the weights in double (tile sums, one-block scan,
// per-tile apply) rounded to float after normalisation.
#include "aur_internal.h"
#include "aur_math.cuh"

namespace aur {
namespace {

constexpr uint32_t kEmThreads = 256;
constexpr uint32_t kEmPer = 16;                       // elements per thread
constexpr uint32_t kEmTile = kEmThreads * kEmPer;     // elements per tile

inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

__device__ __forceinline__ bool emissive(const uint16_t* sids, const aur_shader* shaders, uint32_t i) {
    const uint32_t sid = sids[i];
    return shaders[sid > 0 ? sid - 1 : 0].emission > 0.0f;   // ValidEmitterPredicate, emitter.cu:20-24
}

// Block-wide exclusive scan of one value per thread (kEmThreads threads).
template <typename T>
__device__ T block_exclusive_scan(T v, T* sh, T& total) {
    const uint32_t t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (uint32_t d = 1; d < kEmThreads; d <<= 1) {
        const T add = t >= d ? sh[t - d] : T(0);
        __syncthreads();
        sh[t] += add;
        __syncthreads();
    }
    total = sh[kEmThreads - 1];
    const T incl = sh[t];
    __syncthreads();
    return incl - v;
}

__global__ void k_em_count(const uint16_t* __restrict__ sids, const aur_shader* __restrict__ shaders, uint32_t n,
                           uint32_t* __restrict__ tile_counts) {
    __shared__ uint32_t sh[kEmThreads];
    const uint32_t base = blockIdx.x * kEmTile + threadIdx.x * kEmPer;
    uint32_t c = 0;
    for (uint32_t k = 0; k < kEmPer; ++k) c += base + k < n && emissive(sids, shaders, base + k);
    uint32_t total;
    block_exclusive_scan<uint32_t>(c, sh, total);
    if (threadIdx.x == 0) tile_counts[blockIdx.x] = total;
}

// Exclusive scan of `m` values in place with one block; writes the total to
// *total. Each thread scans a contiguous chunk sequentially.
template <typename T>
__global__ void k_em_scan_tiles(T* __restrict__ v, uint32_t m, T* __restrict__ total) {
    __shared__ T sh[kEmThreads];
    const uint32_t per = (m + kEmThreads - 1) / kEmThreads;
    const uint32_t b0 = min(m, threadIdx.x * per), b1 = min(m, b0 + per);
    T s = T(0);
    for (uint32_t i = b0; i < b1; ++i) s += v[i];
    T all;
    T run = block_exclusive_scan<T>(s, sh, all);
    for (uint32_t i = b0; i < b1; ++i) {
        const T x = v[i];
        v[i] = run;
        run += x;
    }
    if (threadIdx.x == 0) *total = all;
}

__global__ void k_em_scatter(const uint16_t* __restrict__ sids, const aur_shader* __restrict__ shaders,
                             const float* __restrict__ verts, uint32_t n, const uint32_t* __restrict__ tile_off,
                             aur_emitter* __restrict__ out, double* __restrict__ weight) {
    __shared__ uint32_t sh[kEmThreads];
    const uint32_t base = blockIdx.x * kEmTile + threadIdx.x * kEmPer;
    uint32_t c = 0;
    for (uint32_t k = 0; k < kEmPer; ++k) c += base + k < n && emissive(sids, shaders, base + k);
    uint32_t total;
    uint32_t j = tile_off[blockIdx.x] + block_exclusive_scan<uint32_t>(c, sh, total);
    for (uint32_t k = 0; k < kEmPer; ++k) {
        const uint32_t i = base + k;
        if (i >= n || !emissive(sids, shaders, i)) continue;
        const uint32_t sid = sids[i];
        const aur_shader& s = shaders[sid > 0 ? sid - 1 : 0];
        // Primitive3::area (primitive.cuh:74-85)
        const float* v = verts + (size_t)i * 9;
        const f3 v1 = mk3(v[0], v[3], v[6]), v2 = mk3(v[1], v[4], v[7]), v3 = mk3(v[2], v[5], v[8]);
        const f3 va = v1 - v2, vb = v1 - v3, vc = v2 - v3;
        const float a = dot(va, va), b = dot(vb, vb), cc = dot(vc, vc);
        const float area = sqrtf((2 * a * b + 2 * b * cc + 2 * cc * a - a * a - b * b - cc * cc) / 16.0f);
        aur_emitter e;
        e.area = area;
        e.pdf = 1.0f / area;                  // cudaCalculateEmittersCDF, emitter.cu:49-61
        e.cdf = 0.0f;
        e.power = s.emission_color;
        e.triangle_id = i;
        out[j] = e;
        weight[j] = (double)s.emission;       // the CDF's weight: the shader's emission
        ++j;
    }
}

__global__ void k_em_tile_sums(const double* __restrict__ w, uint32_t m, double* __restrict__ tile_sums) {
    __shared__ double sh[kEmThreads];
    const uint32_t base = blockIdx.x * kEmTile + threadIdx.x * kEmPer;
    double s = 0.0;
    for (uint32_t k = 0; k < kEmPer; ++k)
        if (base + k < m) s += w[base + k];
    double total;
    block_exclusive_scan<double>(s, sh, total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Inclusive scan, normalised by the total (cudaNormalizeEmittersCDF, emitter.cu:63-71).
__global__ void k_em_cdf(const double* __restrict__ w, uint32_t m, const double* __restrict__ tile_off,
                         const double* __restrict__ total, aur_emitter* __restrict__ out) {
    __shared__ double sh[kEmThreads];
    const uint32_t base = blockIdx.x * kEmTile + threadIdx.x * kEmPer;
    double s = 0.0;
    for (uint32_t k = 0; k < kEmPer; ++k)
        if (base + k < m) s += w[base + k];
    double all;
    double run = tile_off[blockIdx.x] + block_exclusive_scan<double>(s, sh, all);
    const double tot = *total;
    for (uint32_t k = 0; k < kEmPer; ++k) {
        if (base + k >= m) break;
        run += w[base + k];
        out[base + k].cdf = (float)(run / tot);
    }
}

}  // namespace
}  // namespace aur

using namespace aur;

extern "C" {

aur_status aur_scene_emitters(aur_ctx* ctx, const aur_scene* sc, aur_emitter* emitters, uint32_t* num_emitters) {
    AUR_RANGE("aur_scene_emitters");
    clear_error();
    AUR_CHECK(ctx && sc && num_emitters, AUR_ERR_INVALID, "aur_scene_emitters: null argument");
    *num_emitters = 0;
    const uint32_t n = sc->nmh->count;
    if (n == 0) return AUR_OK;
    AUR_CHECK(emitters, AUR_ERR_INVALID, "aur_scene_emitters: null emitter buffer");
    AUR_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const uint32_t tiles = cdiv(n, kEmTile);
    // scratch: tile counts (+ total), weights, tile sums (+ total)
    const size_t o_cnt = 0, o_w = ((size_t)(tiles + 1) * 4 + 255) & ~(size_t)255;
    const size_t o_ts = o_w + (((size_t)n * 8 + 255) & ~(size_t)255);
    const size_t bytes = o_ts + (size_t)(tiles + 1) * 8;
    char* scratch = nullptr;
    AUR_CHECK(::aur::dev_malloc_async((void**)&scratch, bytes, s) == cudaSuccess, AUR_ERR_OOM,
              "aur_scene_emitters: out of device memory");
    uint32_t* cnt = (uint32_t*)(scratch + o_cnt);
    double* w = (double*)(scratch + o_w);
    double* ts = (double*)(scratch + o_ts);
    k_em_count<<<tiles, kEmThreads, 0, s>>>(sc->shader_ids, sc->shaders, n, cnt);
    k_em_scan_tiles<uint32_t><<<1, kEmThreads, 0, s>>>(cnt, tiles, cnt + tiles);
    k_em_scatter<<<tiles, kEmThreads, 0, s>>>(sc->shader_ids, sc->shaders, sc->nmh->verts, n, cnt, emitters, w);
    uint32_t m = 0;
    cudaMemcpyAsync(&m, cnt + tiles, 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && m > 0) {
        const uint32_t mt = cdiv(m, kEmTile);
        k_em_tile_sums<<<mt, kEmThreads, 0, s>>>(w, m, ts);
        k_em_scan_tiles<double><<<1, kEmThreads, 0, s>>>(ts, mt, ts + mt);
        k_em_cdf<<<mt, kEmThreads, 0, s>>>(w, m, ts, ts + mt, emitters);
        e = cudaGetLastError();
    }
    cudaFreeAsync(scratch, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "aur_scene_emitters", __FILE__, __LINE__);
    *num_emitters = m;
    return AUR_OK;
}

}  // extern "C"
