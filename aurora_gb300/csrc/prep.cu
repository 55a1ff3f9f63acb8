// prep.cu — scene preparation kernels of the reference's renderer helpers.
//
// aur_transform: cudaTransform (kernels/utility.cu:96-134). The reference
// scans every object per triangle to find the last one whose offset is <=
// the triangle index; with non-decreasing offsets that is an upper-bound
// binary search, done here in O(log objects).
// aur_generate_tb: cudaGenerateTBKernel (kernels/utility.cu:136-167).
#include <vector>

#include "aur_integrate.cuh"
#include "aur_internal.h"

namespace aur {
namespace {

// transform.cuh:8-24, row-vector convention, left-to-right sums.
__device__ __forceinline__ f3 xform_point(const aur_object_transform& t, const f3& p) {
    const float(*m)[4] = t.world_matrix;
    return mk3(m[0][0] * p.x + m[1][0] * p.y + m[2][0] * p.z + m[3][0],
               m[0][1] * p.x + m[1][1] * p.y + m[2][1] * p.z + m[3][1],
               m[0][2] * p.x + m[1][2] * p.y + m[2][2] * p.z + m[3][2]);
}

__device__ __forceinline__ f3 xform_normal(const aur_object_transform& t, const f3& n) {
    const float(*m)[4] = t.normal_matrix;
    return mk3(m[0][0] * n.x + m[1][0] * n.y + m[2][0] * n.z, m[0][1] * n.x + m[1][1] * n.y + m[2][1] * n.z,
               m[0][2] * n.x + m[1][2] * n.y + m[2][2] * n.z);
}

// Blocks of kPrepTris triangles stage their 9-float records through shared
// memory: global loads and stores walk consecutive words (a warp moves 128
// contiguous bytes per access), and the 9-float stride of the per-triangle
// arithmetic falls on shared memory, where it is free of bank conflicts (9 is
// coprime with 32 banks).
constexpr uint32_t kPrepTris = 256;
constexpr uint32_t kPrepWords = 9 * kPrepTris;

// Loads words [9 * t0, 9 * t0 + 9 * n) of src into s (coalesced).
__device__ __forceinline__ void stage_in(float* __restrict__ s, const float* __restrict__ src, size_t t0, uint32_t n) {
    const float* g = src + 9 * t0;
    for (uint32_t j = threadIdx.x; j < 9 * n; j += kPrepTris) s[j] = g[j];
}

__global__ void __launch_bounds__(kPrepTris) k_transform(const float* __restrict__ sv, const float* __restrict__ sn,
                                                         uint32_t count, const aur_object_transform* __restrict__ xf,
                                                         uint32_t nobj, float* __restrict__ dv,
                                                         float* __restrict__ dn) {
    __shared__ float s_v[kPrepWords], s_n[kPrepWords];
    __shared__ uint8_t s_keep[kPrepTris];
    const size_t t0 = (size_t)blockIdx.x * kPrepTris;
    const uint32_t n = (uint32_t)min((size_t)kPrepTris, count - t0);
    stage_in(s_v, sv, t0, n);
    stage_in(s_n, sn, t0, n);
    __syncthreads();
    const uint32_t k = threadIdx.x;
    if (k < n) {
        const uint32_t i = (uint32_t)t0 + k;
        // last object with offset <= i
        uint32_t lo = 0, hi = nobj;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (xf[mid].offset <= i) lo = mid + 1; else hi = mid;
        }
        s_keep[k] = lo == 0;                // before the first object: left untouched
        if (lo != 0) {
            const aur_object_transform& t = xf[lo - 1];
            float* v = s_v + 9 * k;
            // readPoints / writePoints: [x1 x2 x3 y1 y2 y3 z1 z2 z3]
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const f3 p = xform_point(t, mk3(v[c], v[3 + c], v[6 + c]));
                v[c] = p.x; v[3 + c] = p.y; v[6 + c] = p.z;
            }
            float* m = s_n + 9 * k;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const f3 q = xform_normal(t, mk3(m[3 * c], m[3 * c + 1], m[3 * c + 2]));
                m[3 * c] = q.x; m[3 * c + 1] = q.y; m[3 * c + 2] = q.z;
            }
        }
    }
    __syncthreads();
    float* ov = dv + 9 * t0;
    float* on = dn + 9 * t0;
    for (uint32_t j = threadIdx.x; j < 9 * n; j += kPrepTris) {
        if (s_keep[j / 9]) continue;
        ov[j] = s_v[j];
        on[j] = s_n[j];
    }
}

__global__ void __launch_bounds__(kPrepTris) k_generate_tb(const float* __restrict__ nrm, uint32_t count,
                                                           float* __restrict__ tan, float* __restrict__ bit) {
    __shared__ float s_n[kPrepWords], s_t[kPrepWords], s_b[kPrepWords];
    const size_t t0 = (size_t)blockIdx.x * kPrepTris;
    const uint32_t n = (uint32_t)min((size_t)kPrepTris, count - t0);
    stage_in(s_n, nrm, t0, n);
    __syncthreads();
    const uint32_t k = threadIdx.x;
    if (k < n) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* m = s_n + 9 * k + 3 * c;
            f3 t, b;
            vertex_tb(mk3(m[0], m[1], m[2]), t, b);
            float* to = s_t + 9 * k + 3 * c;
            float* bo = s_b + 9 * k + 3 * c;
            to[0] = t.x; to[1] = t.y; to[2] = t.z;
            bo[0] = b.x; bo[1] = b.y; bo[2] = b.z;
        }
    }
    __syncthreads();
    float* ot = tan + 9 * t0;
    float* ob = bit + 9 * t0;
    for (uint32_t j = threadIdx.x; j < 9 * n; j += kPrepTris) {
        ot[j] = s_t[j];
        ob[j] = s_b[j];
    }
}

}  // namespace
}  // namespace aur

using namespace aur;

extern "C" {

aur_status aur_transform(aur_ctx* ctx, const float* src_vertices, const float* src_normals, uint32_t count,
                         const aur_object_transform* transforms, uint32_t num_objects, float* dst_vertices,
                         float* dst_normals) {
    AUR_RANGE("aur_transform");
    clear_error();
    AUR_CHECK(ctx, AUR_ERR_INVALID, "aur_transform: null context");
    AUR_CHECK(count == 0 || (src_vertices && src_normals && dst_vertices && dst_normals), AUR_ERR_INVALID,
              "aur_transform: null soup pointer");
    AUR_CHECK(num_objects == 0 || transforms, AUR_ERR_INVALID, "aur_transform: null transform table");
    for (uint32_t i = 1; i < num_objects; ++i)
        AUR_CHECK(transforms[i].offset >= transforms[i - 1].offset, AUR_ERR_INVALID,
                  "aur_transform: object offsets must be non-decreasing (object %u)", i);
    if (count == 0 || num_objects == 0) return AUR_OK;
    AUR_CUDA(cudaSetDevice(ctx->device));
    aur_object_transform* dxf = nullptr;
    AUR_CHECK(::aur::dev_malloc_async(&dxf, sizeof(aur_object_transform) * num_objects, ctx->stream) == cudaSuccess, AUR_ERR_OOM,
              "aur_transform: out of device memory");
    AUR_CUDA(cudaMemcpyAsync(dxf, transforms, sizeof(aur_object_transform) * num_objects, cudaMemcpyHostToDevice, ctx->stream));
    k_transform<<<(count + kPrepTris - 1) / kPrepTris, kPrepTris, 0, ctx->stream>>>(
        src_vertices, src_normals, count, dxf, num_objects, dst_vertices, dst_normals);
    cudaFreeAsync(dxf, ctx->stream);
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));   // the host table is released to the caller on return
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

aur_status aur_generate_tb(aur_ctx* ctx, const float* normals, uint32_t count, float* tangents, float* bitangents) {
    AUR_RANGE("aur_generate_tb");
    clear_error();
    AUR_CHECK(ctx && (count == 0 || (normals && tangents && bitangents)), AUR_ERR_INVALID,
              "aur_generate_tb: null argument");
    if (count == 0) return AUR_OK;
    AUR_CUDA(cudaSetDevice(ctx->device));
    k_generate_tb<<<(count + kPrepTris - 1) / kPrepTris, kPrepTris, 0, ctx->stream>>>(normals, count, tangents,
                                                                                     bitangents);
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

}  // extern "C"
