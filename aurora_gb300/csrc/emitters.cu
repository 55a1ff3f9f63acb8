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
#include <mutex>

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

// ------------------------------------------- light-selection table (MIS)
// The emitters AUR_MODE_PATH_MIS samples: emission > 0, positive area
// 0.5 |(v2 - v1) x (v3 - v1)|, and not the even-padding copy of the last
// triangle (perm >= the input count), so that every emitting surface is in
// the table once; weight emission * area.

__device__ __forceinline__ float mis_area(const float* __restrict__ verts, uint32_t i) {
    const float* v = verts + (size_t)i * 9;
    const f3 v1 = mk3(v[0], v[3], v[6]), v2 = mk3(v[1], v[4], v[7]), v3 = mk3(v[2], v[5], v[8]);
    return 0.5f * length(cross(v2 - v1, v3 - v1));
}

__device__ __forceinline__ bool mis_valid(const uint16_t* sids, const aur_shader* shaders, const float* verts,
                                          const uint32_t* perm, uint32_t input_count, uint32_t i) {
    return emissive(sids, shaders, i) && perm[i] < input_count && mis_area(verts, i) > 0.0f;
}

__global__ void k_mis_count(const uint16_t* __restrict__ sids, const aur_shader* __restrict__ shaders,
                            const float* __restrict__ verts, const uint32_t* __restrict__ perm, uint32_t input_count,
                            uint32_t n, uint32_t* __restrict__ tile_counts) {
    __shared__ uint32_t sh[kEmThreads];
    const uint32_t base = blockIdx.x * kEmTile + threadIdx.x * kEmPer;
    uint32_t c = 0;
    for (uint32_t k = 0; k < kEmPer; ++k)
        c += base + k < n && mis_valid(sids, shaders, verts, perm, input_count, base + k);
    uint32_t total;
    block_exclusive_scan<uint32_t>(c, sh, total);
    if (threadIdx.x == 0) tile_counts[blockIdx.x] = total;
}

__global__ void k_mis_scatter(const uint16_t* __restrict__ sids, const aur_shader* __restrict__ shaders,
                              const float* __restrict__ verts, const uint32_t* __restrict__ perm, uint32_t input_count,
                              uint32_t n, const uint32_t* __restrict__ tile_off, uint32_t* __restrict__ tri,
                              double* __restrict__ weight) {
    __shared__ uint32_t sh[kEmThreads];
    const uint32_t base = blockIdx.x * kEmTile + threadIdx.x * kEmPer;
    uint32_t c = 0;
    for (uint32_t k = 0; k < kEmPer; ++k)
        c += base + k < n && mis_valid(sids, shaders, verts, perm, input_count, base + k);
    uint32_t total;
    uint32_t j = tile_off[blockIdx.x] + block_exclusive_scan<uint32_t>(c, sh, total);
    for (uint32_t k = 0; k < kEmPer; ++k) {
        const uint32_t i = base + k;
        if (i >= n || !mis_valid(sids, shaders, verts, perm, input_count, i)) continue;
        const uint32_t sid = sids[i];
        tri[j] = i;
        weight[j] = (double)shaders[sid > 0 ? sid - 1 : 0].emission * (double)mis_area(verts, i);
        ++j;
    }
}

__global__ void k_mis_cdf(const double* __restrict__ w, uint32_t m, const double* __restrict__ tile_off,
                          const double* __restrict__ total, float* __restrict__ cdf) {
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
        cdf[base + k] = (float)(run / tot);
    }
}

// pa[tri] = (cdf[k] - cdf[k-1]) / area: the density, per unit area, of the
// points the emitter sample draws on that triangle.
__global__ void k_mis_pa(const uint32_t* __restrict__ tri, const float* __restrict__ cdf, uint32_t m,
                         const float* __restrict__ verts, float* __restrict__ pa) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const float psel = cdf[k] - (k > 0 ? cdf[k - 1] : 0.0f);
    const uint32_t i = tri[k];
    pa[i] = psel / mis_area(verts, i);
}

// Guards the lazily built tables: renders of one scene from several threads
// (each on its own context) may ask for the table at the same time.
std::mutex g_mis_mutex;

void free_mis_table_locked(const aur_scene* sc) {
    cudaFree(sc->mis_tri);
    cudaFree(sc->mis_cdf);
    cudaFree(sc->mis_pa);
    sc->mis_tri = nullptr;
    sc->mis_cdf = nullptr;
    sc->mis_pa = nullptr;
    sc->mis_count = 0;
    sc->mis_ready = false;
}

}  // namespace

void free_mis_table(const aur_scene* sc) {
    std::lock_guard<std::mutex> lock(g_mis_mutex);
    free_mis_table_locked(sc);
}

aur_status build_mis_table(aur_ctx* ctx, const aur_scene* sc) {
    std::lock_guard<std::mutex> lock(g_mis_mutex);
    if (sc->mis_ready) return AUR_OK;
    free_mis_table_locked(sc);
    const uint32_t n = sc->nmh->count;
    if (n == 0) {
        sc->mis_ready = true;
        return AUR_OK;
    }
    cudaStream_t s = ctx->stream;
    const uint32_t tiles = cdiv(n, kEmTile);
    // scratch: tile counts (+ total), triangle ids, weights, tile sums (+ total)
    const size_t o_tri = ((size_t)(tiles + 1) * 4 + 255) & ~(size_t)255;
    const size_t o_w = o_tri + (((size_t)n * 4 + 255) & ~(size_t)255);
    const size_t o_ts = o_w + (((size_t)n * 8 + 255) & ~(size_t)255);
    const size_t bytes = o_ts + (size_t)(tiles + 1) * 8;
    char* scratch = nullptr;
    AUR_CHECK(::aur::dev_malloc_async((void**)&scratch, bytes, s) == cudaSuccess, AUR_ERR_OOM,
              "render: out of device memory (light-selection table)");
    uint32_t* cnt = (uint32_t*)scratch;
    uint32_t* tri = (uint32_t*)(scratch + o_tri);
    double* w = (double*)(scratch + o_w);
    double* ts = (double*)(scratch + o_ts);
    const uint32_t* perm = sc->nmh->perm;
    const float* verts = sc->nmh->verts;
    const uint32_t nin = sc->nmh->input_count;
    k_mis_count<<<tiles, kEmThreads, 0, s>>>(sc->shader_ids, sc->shaders, verts, perm, nin, n, cnt);
    k_em_scan_tiles<uint32_t><<<1, kEmThreads, 0, s>>>(cnt, tiles, cnt + tiles);
    k_mis_scatter<<<tiles, kEmThreads, 0, s>>>(sc->shader_ids, sc->shaders, verts, perm, nin, n, cnt, tri, w);
    uint32_t m = 0;
    cudaMemcpyAsync(&m, cnt + tiles, 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    aur_status st = AUR_OK;
    if (e == cudaSuccess) {
        if (::aur::dev_malloc(&sc->mis_pa, (size_t)n * 4) != cudaSuccess ||
            (m > 0 && (::aur::dev_malloc(&sc->mis_tri, (size_t)m * 4) != cudaSuccess ||
                       ::aur::dev_malloc(&sc->mis_cdf, (size_t)m * 4) != cudaSuccess))) {
            cudaGetLastError();
            st = fail(AUR_ERR_OOM, "render: out of device memory (light-selection table)");
        }
    }
    if (e == cudaSuccess && st == AUR_OK) {
        cudaMemsetAsync(sc->mis_pa, 0, (size_t)n * 4, s);
        if (m > 0) {
            const uint32_t mt = cdiv(m, kEmTile);
            cudaMemcpyAsync(sc->mis_tri, tri, (size_t)m * 4, cudaMemcpyDeviceToDevice, s);
            k_em_tile_sums<<<mt, kEmThreads, 0, s>>>(w, m, ts);
            k_em_scan_tiles<double><<<1, kEmThreads, 0, s>>>(ts, mt, ts + mt);
            k_mis_cdf<<<mt, kEmThreads, 0, s>>>(w, m, ts, ts + mt, sc->mis_cdf);
            k_mis_pa<<<cdiv(m, 256), 256, 0, s>>>(sc->mis_tri, sc->mis_cdf, m, verts, sc->mis_pa);
        }
        e = cudaGetLastError();
    }
    cudaFreeAsync(scratch, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_fail(e, "render (light-selection table)", __FILE__, __LINE__);
    if (st != AUR_OK) {
        free_mis_table_locked(sc);
        return st;
    }
    sc->mis_count = m;
    sc->mis_ready = true;
    return AUR_OK;
}

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

aur_status aur_scene_mis_table(aur_ctx* ctx, const aur_scene* sc, uint32_t* triangles, float* cdf, float* pa,
                               uint32_t* count) {
    AUR_RANGE("aur_scene_mis_table");
    clear_error();
    AUR_CHECK(ctx && sc && count, AUR_ERR_INVALID, "aur_scene_mis_table: null argument");
    AUR_CUDA(cudaSetDevice(ctx->device));
    const aur_status st = build_mis_table(ctx, sc);
    if (st != AUR_OK) return st;
    const uint32_t m = sc->mis_count;
    *count = m;
    cudaStream_t s = ctx->stream;
    if (triangles && m) AUR_CUDA(cudaMemcpyAsync(triangles, sc->mis_tri, (size_t)m * 4, cudaMemcpyDefault, s));
    if (cdf && m) AUR_CUDA(cudaMemcpyAsync(cdf, sc->mis_cdf, (size_t)m * 4, cudaMemcpyDefault, s));
    if (pa && sc->nmh->count)
        AUR_CUDA(cudaMemcpyAsync(pa, sc->mis_pa, (size_t)sc->nmh->count * 4, cudaMemcpyDefault, s));
    AUR_CUDA(cudaStreamSynchronize(s));
    return AUR_OK;
}

}  // extern "C"
