// abi.cu — contexts, errors, NMH and scene objects of the C ABI.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "aur_integrate.cuh"
#include "aur_internal.h"
#include "aur_math.cuh"

namespace aur {

namespace {
thread_local char g_error[512] = "";
}

aur_status fail(aur_status st, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
    return st;
}

aur_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    const aur_status st = (e == cudaErrorMemoryAllocation) ? AUR_ERR_OOM
                          : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? AUR_ERR_NO_DEVICE
                                                                                          : AUR_ERR_CUDA;
    const char* base = strrchr(file, '/');
    return fail(st, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), base ? base + 1 : file, line);
}

void clear_error() { g_error[0] = 0; }

namespace {
// Allocation fault injection: 0 = off; k > 0 = the k-th allocation from now fails.
std::atomic<uint32_t> g_fail_countdown{0};

bool injected_failure() {
    uint32_t k = g_fail_countdown.load();
    while (k > 0)
        if (g_fail_countdown.compare_exchange_weak(k, k - 1)) return k == 1;
    return false;
}
}  // namespace

cudaError_t alloc_device(void** p, size_t bytes) {
    if (injected_failure()) { *p = nullptr; return cudaErrorMemoryAllocation; }
    return cudaMalloc(p, bytes);
}

cudaError_t alloc_device_async(void** p, size_t bytes, cudaStream_t s) {
    if (injected_failure()) { *p = nullptr; return cudaErrorMemoryAllocation; }
    return cudaMallocAsync(p, bytes, s);
}

cudaError_t alloc_pinned(void** p, size_t bytes) {
    if (injected_failure()) { *p = nullptr; return cudaErrorMemoryAllocation; }
    return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

Range::Range(const char* name) { nvtxRangePushA(name); }
Range::~Range() { nvtxRangePop(); }

namespace {

// Reorders per-triangle attributes into NMH order; odd inputs read their
// padding duplicate from the last triangle.
__global__ void k_permute_attrs(const uint32_t* __restrict__ perm, uint32_t N, uint32_t count_in,
                                const float* __restrict__ nin, const uint16_t* __restrict__ sin,
                                float* __restrict__ nout, uint16_t* __restrict__ sout) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    uint32_t src = perm[i];
    if (src >= count_in) src = count_in - 1;
#pragma unroll
    for (int q = 0; q < 9; ++q) nout[(size_t)i * 9 + q] = nin[(size_t)src * 9 + q];
    sout[i] = sin[src];
}

// applyIndices for an attribute of `words` 16-bit words per triangle.
__global__ void k_apply(const uint32_t* __restrict__ perm, uint32_t N, uint32_t count_in,
                        const uint16_t* __restrict__ src, uint32_t words, uint16_t* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    uint32_t p = perm[i];
    if (p >= count_in) p = count_in - 1;
    for (uint32_t w = 0; w < words; ++w) dst[(size_t)i * words + w] = src[(size_t)p * words + w];
}

void free_textures(aur_scene* sc) {
    cudaFree(sc->texels);
    cudaFree(sc->tex_info);
    cudaFree(sc->texcoords);
    sc->texels = nullptr;
    sc->tex_info = nullptr;
    sc->texcoords = nullptr;
    sc->num_textures = 0;
}

__global__ void k_texfetch(SceneView sv, uint32_t texture, const float* __restrict__ uv, uint32_t n,
                           float* __restrict__ rgb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 c = texfetch(sv, texture - 1, uv[2 * i], uv[2 * i + 1]);
    rgb[3 * i] = c.x;
    rgb[3 * i + 1] = c.y;
    rgb[3 * i + 2] = c.z;
}

}  // namespace
}  // namespace aur

using namespace aur;

extern "C" {

const char* aur_last_error(void) { return g_error; }

const char* aur_version(void) { return "aurora_gb300 0.1 (sm_103a)"; }

aur_status aur_ctx_create(int device, aur_ctx** out) {
    clear_error();
    AUR_CHECK(out, AUR_ERR_INVALID, "aur_ctx_create: null output");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(AUR_ERR_NO_DEVICE, "aur_ctx_create: no CUDA device (%s)", cudaGetErrorString(e));
    }
    AUR_CHECK(device >= 0 && device < ndev, AUR_ERR_INVALID, "aur_ctx_create: device %d of %d", device, ndev);
    cudaDeviceProp prop;
    AUR_CUDA(cudaGetDeviceProperties(&prop, device));
    AUR_CHECK(prop.major == 10 && prop.minor == 3, AUR_ERR_NO_DEVICE,
              "aur_ctx_create: device %d is sm_%d%d; this build targets sm_103a", device, prop.major, prop.minor);
    AUR_CUDA(cudaSetDevice(device));
    aur_ctx* c = new aur_ctx();
    c->device = device;
    c->sm_count = prop.multiProcessorCount;
    // keep the first failing call's own code (not the sticky last error)
    e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->compute2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = ::aur::dev_malloc(&c->d_flags, 256);
    if (e == cudaSuccess) e = cudaMemset(c->d_flags, 0, 256);
    if (e != cudaSuccess) {
        cudaGetLastError();
        aur_ctx_destroy(c);
        return cuda_fail(e, "aur_ctx_create", __FILE__, __LINE__);
    }
    for (auto& ev : c->ev) {
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaGetLastError();
            aur_ctx_destroy(c);
            return cuda_fail(e, "aur_ctx_create events", __FILE__, __LINE__);
        }
    }
    c->stream = c->own_stream;
    *out = c;
    return AUR_OK;
}

aur_status aur_debug_fail_allocation(uint32_t k) {
    g_fail_countdown.store(k);
    return AUR_OK;
}

aur_status aur_ctx_destroy(aur_ctx* ctx) {
    if (!ctx) return AUR_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    ::aur::free_build_cache(ctx);
    for (auto& s : ctx->pipe) cudaFree(s.ptr);
    for (auto& s : ctx->out) cudaFree(s.ptr);
    for (auto& s : ctx->defer) cudaFree(s.ptr);
    for (auto& ev : ctx->ev) if (ev) cudaEventDestroy(ev);
    cudaFree(ctx->d_flags);
    if (ctx->copy_in) cudaStreamDestroy(ctx->copy_in);
    if (ctx->copy_out) cudaStreamDestroy(ctx->copy_out);
    if (ctx->compute2) cudaStreamDestroy(ctx->compute2);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return AUR_OK;
}

aur_status aur_ctx_set_stream(aur_ctx* ctx, void* cuda_stream) {
    AUR_CHECK(ctx, AUR_ERR_INVALID, "aur_ctx_set_stream: null context");
    ctx->stream = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_stream;
    return AUR_OK;
}

aur_status aur_ctx_get_stream(aur_ctx* ctx, void** cuda_stream) {
    AUR_CHECK(ctx && cuda_stream, AUR_ERR_INVALID, "aur_ctx_get_stream: null argument");
    *cuda_stream = (void*)ctx->stream;
    return AUR_OK;
}

aur_status aur_ctx_synchronize(aur_ctx* ctx) {
    AUR_CHECK(ctx, AUR_ERR_INVALID, "aur_ctx_synchronize: null context");
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    uint32_t flags = 0;
    AUR_CUDA(cudaMemcpy(&flags, ctx->d_flags, 4, cudaMemcpyDeviceToHost));
    if (flags) {
        cudaMemset(ctx->d_flags, 0, 4);
        return fail(AUR_ERR_OVERFLOW, "a device-side stack would have overflowed (flags 0x%x)", flags);
    }
    return AUR_OK;
}

aur_status aur_ctx_sm_count(aur_ctx* ctx, int* sm_count) {
    AUR_CHECK(ctx && sm_count, AUR_ERR_INVALID, "aur_ctx_sm_count: null argument");
    *sm_count = ctx->sm_count;
    return AUR_OK;
}

// ------------------------------------------------------------------ NMH

aur_status aur_nmh_build(aur_ctx* ctx, const float* vertices, uint32_t count, aur_nmh** out) {
    AUR_RANGE("aur_nmh_build");
    clear_error();
    return nmh_build_impl(ctx, vertices, count, out);
}

aur_status aur_nmh_destroy(aur_nmh* nmh) {
    if (!nmh) return AUR_OK;
    cudaSetDevice(nmh->device);
    if (nmh->rec_tex) {
        cudaDeviceSynchronize();   // no traversal may still read through the texture
        cudaDestroyTextureObject(nmh->rec_tex);
    }
    cudaFree(nmh->mem);
    delete nmh;
    return AUR_OK;
}

aur_status aur_debug_nmh_drop_texture(aur_nmh* nmh) {
    AUR_CHECK(nmh, AUR_ERR_INVALID, "aur_debug_nmh_drop_texture: null NMH");
    AUR_CUDA(cudaSetDevice(nmh->device));
    if (nmh->rec_tex) {
        AUR_CUDA(cudaDeviceSynchronize());   // no launch may still read through it
        AUR_CUDA(cudaDestroyTextureObject(nmh->rec_tex));
        nmh->rec_tex = 0;
    }
    return AUR_OK;
}

aur_status aur_nmh_info(const aur_nmh* nmh, uint32_t* count, uint32_t* levels) {
    AUR_CHECK(nmh, AUR_ERR_INVALID, "aur_nmh_info: null NMH");
    if (count) *count = nmh->count;
    if (levels) *levels = nmh->levels;
    return AUR_OK;
}

aur_status aur_nmh_export(aur_ctx* ctx, const aur_nmh* nmh, uint32_t* perm, float* vertices) {
    AUR_CHECK(ctx && nmh, AUR_ERR_INVALID, "aur_nmh_export: null context or NMH");
    AUR_CUDA(cudaSetDevice(ctx->device));
    if (nmh->count == 0) return AUR_OK;
    if (perm)
        AUR_CUDA(cudaMemcpyAsync(perm, nmh->perm, (size_t)nmh->count * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (vertices)
        AUR_CUDA(cudaMemcpyAsync(vertices, nmh->verts, (size_t)nmh->count * 36, cudaMemcpyDeviceToHost, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    return AUR_OK;
}

aur_status aur_nmh_apply(aur_ctx* ctx, const aur_nmh* nmh, const void* src, uint32_t bytes_per_triangle, void* dst) {
    AUR_RANGE("aur_nmh_apply");
    clear_error();
    AUR_CHECK(ctx && nmh, AUR_ERR_INVALID, "aur_nmh_apply: null context or NMH");
    AUR_CHECK(bytes_per_triangle > 0 && bytes_per_triangle % 2 == 0, AUR_ERR_INVALID,
              "aur_nmh_apply: bytes_per_triangle must be a positive multiple of 2");
    if (nmh->count == 0) return AUR_OK;
    AUR_CHECK(src && dst, AUR_ERR_INVALID, "aur_nmh_apply: null buffer");
    AUR_CUDA(cudaSetDevice(ctx->device));
    k_apply<<<(nmh->count + 255) / 256, 256, 0, ctx->stream>>>(nmh->perm, nmh->count, nmh->input_count,
                                                              (const uint16_t*)src, bytes_per_triangle / 2,
                                                              (uint16_t*)dst);
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

// --------------------------------------------------------------- memory

aur_status aur_malloc(aur_ctx* ctx, size_t bytes, int policy, void** out) {
    clear_error();
    AUR_CHECK(ctx && out, AUR_ERR_INVALID, "aur_malloc: null argument");
    *out = nullptr;
    if (bytes == 0) return AUR_OK;
    if (policy == AUR_HOST_MEMORY) {
        *out = std::malloc(bytes);
        AUR_CHECK(*out, AUR_ERR_OOM, "aur_malloc: out of host memory (%zu bytes)", bytes);
        return AUR_OK;
    }
    AUR_CUDA(cudaSetDevice(ctx->device));
    cudaError_t e;
    if (policy == AUR_DEVICE_MEMORY) e = ::aur::dev_malloc(out, bytes);
    else if (policy == AUR_PINNED_MEMORY) e = alloc_pinned(out, bytes);
    else return fail(AUR_ERR_INVALID, "aur_malloc: unknown memory policy %d", policy);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return fail(AUR_ERR_OOM, "aur_malloc: %zu bytes: %s", bytes, cudaGetErrorString(e));
    }
    return AUR_OK;
}

aur_status aur_free(aur_ctx* ctx, void* ptr, int policy) {
    AUR_CHECK(ctx, AUR_ERR_INVALID, "aur_free: null context");
    if (!ptr) return AUR_OK;
    if (policy == AUR_HOST_MEMORY) { std::free(ptr); return AUR_OK; }
    AUR_CUDA(cudaSetDevice(ctx->device));
    if (policy == AUR_DEVICE_MEMORY) AUR_CUDA(cudaFree(ptr));
    else if (policy == AUR_PINNED_MEMORY) AUR_CUDA(cudaFreeHost(ptr));
    else return fail(AUR_ERR_INVALID, "aur_free: unknown memory policy %d", policy);
    return AUR_OK;
}

aur_status aur_memzero(aur_ctx* ctx, void* ptr, size_t bytes, int policy) {
    AUR_CHECK(ctx && (ptr || bytes == 0), AUR_ERR_INVALID, "aur_memzero: null argument");
    if (bytes == 0) return AUR_OK;
    if (policy != AUR_DEVICE_MEMORY) { std::memset(ptr, 0, bytes); return AUR_OK; }
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaMemsetAsync(ptr, 0, bytes, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    return AUR_OK;
}

aur_status aur_memupload(aur_ctx* ctx, void* dst, const void* src, size_t bytes, int policy) {
    AUR_CHECK(ctx && ((dst && src) || bytes == 0), AUR_ERR_INVALID, "aur_memupload: null argument");
    if (bytes == 0) return AUR_OK;
    if (policy != AUR_DEVICE_MEMORY) { std::memcpy(dst, src, bytes); return AUR_OK; }
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    return AUR_OK;
}

aur_status aur_memdownload(aur_ctx* ctx, void* dst, const void* src, size_t bytes) {
    AUR_CHECK(ctx && ((dst && src) || bytes == 0), AUR_ERR_INVALID, "aur_memdownload: null argument");
    if (bytes == 0) return AUR_OK;
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    return AUR_OK;
}

aur_status aur_nmh_perm_device(const aur_nmh* nmh, const uint32_t** perm) {
    AUR_CHECK(nmh && perm, AUR_ERR_INVALID, "aur_nmh_perm_device: null argument");
    *perm = nmh->perm;
    return AUR_OK;
}

// ---------------------------------------------------------------- scene

static aur_status validate_materials(const aur_shader* shaders, uint32_t ns, const aur_light* lights, uint32_t nl) {
    AUR_CHECK(ns >= 1 && shaders, AUR_ERR_INVALID, "scene: at least one shader is required (id 0 selects shader 0)");
    AUR_CHECK(nl == 0 || lights, AUR_ERR_INVALID, "scene: null light table");
    for (uint32_t i = 0; i < ns; ++i) {
        AUR_CHECK(shaders[i].type == AUR_SHADER_LAMBERT || shaders[i].type == AUR_SHADER_PHONG, AUR_ERR_INVALID,
                  "scene: shader %u has unknown type %d", i, shaders[i].type);
    }
    for (uint32_t i = 0; i < nl; ++i) {
        AUR_CHECK(lights[i].type >= AUR_LIGHT_AMBIENT && lights[i].type <= AUR_LIGHT_AREA, AUR_ERR_INVALID,
                  "scene: light %u has unknown type %d", i, lights[i].type);
        AUR_CHECK(lights[i].type != AUR_LIGHT_AREA || lights[i].samples >= 1, AUR_ERR_INVALID,
                  "scene: area light %u needs samples >= 1", i);
    }
    return AUR_OK;
}

static uint32_t max_texture_id(const aur_shader* shaders, uint32_t n) {
    uint32_t m = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (shaders[i].texture <= AUR_MAX_TEXTURES && shaders[i].texture > m) m = shaders[i].texture;
    return m;
}

aur_status aur_scene_create(aur_ctx* ctx, const float* vertices, const float* normals, const uint16_t* shader_ids,
                            uint32_t count, const aur_shader* shaders, uint32_t num_shaders, const aur_light* lights,
                            uint32_t num_lights, aur_scene** out) {
    AUR_RANGE("aur_scene_create");
    clear_error();
    AUR_CHECK(ctx && out, AUR_ERR_INVALID, "aur_scene_create: null context or output");
    AUR_CHECK(count == 0 || vertices, AUR_ERR_INVALID, "aur_scene_create: null vertices");
    AUR_CHECK(count < kMaxTriangles, AUR_ERR_INVALID, "aur_scene_create: too many triangles (%u)", count);
    aur_status st = validate_materials(shaders, num_shaders, lights, num_lights);
    if (st != AUR_OK) return st;
    if (shader_ids)
        for (uint32_t i = 0; i < count; ++i)
            AUR_CHECK(shader_ids[i] <= num_shaders, AUR_ERR_INVALID, "aur_scene_create: triangle %u has shader id %u > %u",
                      i, shader_ids[i], num_shaders);
    AUR_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    aur_scene* sc = new aur_scene();
    auto bail = [&](aur_status e) {
        aur_scene_destroy(sc);
        return e;
    };
    // host-side normals when absent: the face normal at all three vertices
    std::vector<float> fn;
    if (!normals && count) {
        fn.resize((size_t)count * 9);
        for (uint32_t i = 0; i < count; ++i) {
            const float* v = vertices + (size_t)i * 9;
            const f3 p1 = mk3(v[0], v[3], v[6]), p2 = mk3(v[1], v[4], v[7]), p3 = mk3(v[2], v[5], v[8]);
            f3 n = cross(p2 - p1, p3 - p1);
            const float l = length(n);
            n = l > 0.0f ? n / l : mk3(0.0f, 1.0f, 0.0f);
            for (int q = 0; q < 3; ++q) { fn[(size_t)i * 9 + 3 * q] = n.x; fn[(size_t)i * 9 + 3 * q + 1] = n.y; fn[(size_t)i * 9 + 3 * q + 2] = n.z; }
        }
        normals = fn.data();
    }
    std::vector<uint16_t> zeros;
    if (!shader_ids && count) { zeros.assign(count, 0); shader_ids = zeros.data(); }
    float* dv = nullptr; float* dn = nullptr; uint16_t* ds = nullptr;
    if (count) {
        if (::aur::dev_malloc_async(&dv, (size_t)count * 36, s) != cudaSuccess || ::aur::dev_malloc_async(&dn, (size_t)count * 36, s) != cudaSuccess ||
            ::aur::dev_malloc_async(&ds, (size_t)count * 2, s) != cudaSuccess) {
            cudaGetLastError();
            cudaFreeAsync(dv, s); cudaFreeAsync(dn, s); cudaFreeAsync(ds, s);
            return bail(fail(AUR_ERR_OOM, "aur_scene_create: out of device memory"));
        }
        cudaMemcpyAsync(dv, vertices, (size_t)count * 36, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dn, normals, (size_t)count * 36, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(ds, shader_ids, (size_t)count * 2, cudaMemcpyHostToDevice, s);
    }
    st = nmh_build_impl(ctx, dv, count, &sc->nmh);
    if (st != AUR_OK) {
        cudaFreeAsync(dv, s); cudaFreeAsync(dn, s); cudaFreeAsync(ds, s);
        return bail(st);
    }
    const uint32_t N = sc->nmh->count;
    if (N) {
        if (::aur::dev_malloc(&sc->normals, (size_t)N * 36) != cudaSuccess || ::aur::dev_malloc(&sc->shader_ids, (size_t)N * 2) != cudaSuccess) {
            cudaGetLastError();
            cudaFreeAsync(dv, s); cudaFreeAsync(dn, s); cudaFreeAsync(ds, s);
            return bail(fail(AUR_ERR_OOM, "aur_scene_create: out of device memory"));
        }
        k_permute_attrs<<<(N + 255) / 256, 256, 0, s>>>(sc->nmh->perm, N, count, dn, ds, sc->normals, sc->shader_ids);
    }
    cudaFreeAsync(dv, s); cudaFreeAsync(dn, s); cudaFreeAsync(ds, s);
    if (::aur::dev_malloc(&sc->shaders, sizeof(aur_shader) * num_shaders) != cudaSuccess ||
        (num_lights && ::aur::dev_malloc(&sc->lights, sizeof(aur_light) * num_lights) != cudaSuccess)) {
        cudaGetLastError();
        return bail(fail(AUR_ERR_OOM, "aur_scene_create: out of device memory"));
    }
    sc->num_shaders = num_shaders;
    sc->num_lights = num_lights;
    sc->max_texture = max_texture_id(shaders, num_shaders);
    for (uint32_t i = 0; i < num_shaders; ++i)
        sc->has_specular |= shaders[i].reflectivity > 0.0f || shaders[i].translucence > 0.0f;
    cudaMemcpyAsync(sc->shaders, shaders, sizeof(aur_shader) * num_shaders, cudaMemcpyHostToDevice, s);
    if (num_lights) cudaMemcpyAsync(sc->lights, lights, sizeof(aur_light) * num_lights, cudaMemcpyHostToDevice, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return bail(cuda_fail(e, "aur_scene_create", __FILE__, __LINE__));
    *out = sc;
    return AUR_OK;
}

aur_status aur_scene_destroy(aur_scene* sc) {
    if (!sc) return AUR_OK;
    if (sc->nmh) cudaSetDevice(sc->nmh->device);
    cudaFree(sc->normals);
    cudaFree(sc->shader_ids);
    cudaFree(sc->shaders);
    cudaFree(sc->lights);
    free_mis_table(sc);
    free_textures(sc);
    aur_nmh_destroy(sc->nmh);
    delete sc;
    return AUR_OK;
}

aur_status aur_scene_nmh(const aur_scene* sc, const aur_nmh** nmh) {
    AUR_CHECK(sc && nmh, AUR_ERR_INVALID, "aur_scene_nmh: null argument");
    *nmh = sc->nmh;
    return AUR_OK;
}

aur_status aur_scene_set_shaders(aur_ctx* ctx, aur_scene* sc, const aur_shader* shaders, uint32_t n) {
    AUR_CHECK(ctx && sc, AUR_ERR_INVALID, "aur_scene_set_shaders: null argument");
    AUR_CHECK(n == sc->num_shaders, AUR_ERR_INVALID, "aur_scene_set_shaders: %u shaders, scene has %u", n,
              sc->num_shaders);
    aur_status st = validate_materials(shaders, n, nullptr, 0);
    if (st != AUR_OK) return st;
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaMemcpyAsync(sc->shaders, shaders, sizeof(aur_shader) * n, cudaMemcpyHostToDevice, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    sc->has_specular = false;
    for (uint32_t i = 0; i < n; ++i)
        sc->has_specular |= shaders[i].reflectivity > 0.0f || shaders[i].translucence > 0.0f;
    sc->max_texture = max_texture_id(shaders, n);
    free_mis_table(sc);   // emission may have changed
    return AUR_OK;
}

aur_status aur_scene_set_textures(aur_ctx* ctx, aur_scene* sc, const float* texcoords, const aur_texture* textures,
                                  uint32_t n) {
    AUR_RANGE("aur_scene_set_textures");
    clear_error();
    AUR_CHECK(ctx && sc, AUR_ERR_INVALID, "aur_scene_set_textures: null argument");
    AUR_CHECK(n <= AUR_MAX_TEXTURES, AUR_ERR_INVALID, "aur_scene_set_textures: %u textures, at most %d", n,
              AUR_MAX_TEXTURES);
    AUR_CHECK(n == 0 || textures, AUR_ERR_INVALID, "aur_scene_set_textures: null texture table");
    const uint32_t count = sc->nmh->input_count;
    AUR_CHECK(count == 0 || texcoords, AUR_ERR_INVALID, "aur_scene_set_textures: null texcoords");
    for (uint32_t i = 0; i < n; ++i)
        AUR_CHECK(textures[i].width >= 1 && textures[i].height >= 1 && textures[i].rgba, AUR_ERR_INVALID,
                  "aur_scene_set_textures: texture %u is empty", i);
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    free_textures(sc);
    cudaStream_t s = ctx->stream;
    const uint32_t N = sc->nmh->count;
    if (N) {
        float* staged = nullptr;
        if (::aur::dev_malloc(&sc->texcoords, (size_t)N * 24) != cudaSuccess ||
            ::aur::dev_malloc_async(&staged, (size_t)count * 24, s) != cudaSuccess) {
            cudaGetLastError();
            free_textures(sc);
            return fail(AUR_ERR_OOM, "aur_scene_set_textures: out of device memory");
        }
        cudaMemcpyAsync(staged, texcoords, (size_t)count * 24, cudaMemcpyHostToDevice, s);
        // applyIndices for the texcoords (rebuilder.cu:217-245)
        k_apply<<<(N + 255) / 256, 256, 0, s>>>(sc->nmh->perm, N, count, (const uint16_t*)staged, 12,
                                               (uint16_t*)sc->texcoords);
        cudaFreeAsync(staged, s);
    }
    // every texture's texels in one buffer; tex_info[t] = (first texel, width, height)
    uint4 info[AUR_MAX_TEXTURES];
    std::memset(info, 0, sizeof(info));
    size_t texels = 0;
    for (uint32_t i = 0; i < n; ++i) {
        info[i] = make_uint4((uint32_t)texels, textures[i].width, textures[i].height, 0u);
        texels += (size_t)textures[i].width * textures[i].height;
        AUR_CHECK(texels < (1ull << 32), AUR_ERR_INVALID, "aur_scene_set_textures: more than 2^32 texels");
    }
    if (::aur::dev_malloc(&sc->tex_info, sizeof(info)) != cudaSuccess ||
        (texels && ::aur::dev_malloc(&sc->texels, texels * sizeof(uchar4)) != cudaSuccess)) {
        cudaGetLastError();
        free_textures(sc);
        return fail(AUR_ERR_OOM, "aur_scene_set_textures: out of device memory");
    }
    cudaMemcpyAsync(sc->tex_info, info, sizeof(info), cudaMemcpyHostToDevice, s);
    for (uint32_t i = 0; i < n; ++i)
        cudaMemcpyAsync(sc->texels + info[i].x, textures[i].rgba,
                        (size_t)textures[i].width * textures[i].height * sizeof(uchar4), cudaMemcpyHostToDevice, s);
    sc->num_textures = n;
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        free_textures(sc);
        return cuda_fail(e, "aur_scene_set_textures", __FILE__, __LINE__);
    }
    return AUR_OK;
}

aur_status aur_scene_texfetch(aur_ctx* ctx, const aur_scene* sc, uint32_t texture, const float* uv, uint32_t n,
                              float* rgb) {
    clear_error();
    AUR_CHECK(ctx && sc, AUR_ERR_INVALID, "aur_scene_texfetch: null argument");
    AUR_CHECK(n == 0 || (uv && rgb), AUR_ERR_INVALID, "aur_scene_texfetch: null buffer");
    AUR_CHECK(texture >= 1 && (texture > AUR_MAX_TEXTURES || texture <= sc->num_textures), AUR_ERR_INVALID,
              "aur_scene_texfetch: texture %u, scene has %u", texture, sc->num_textures);
    if (n == 0) return AUR_OK;
    AUR_CUDA(cudaSetDevice(ctx->device));
    k_texfetch<<<(n + 255) / 256, 256, 0, ctx->stream>>>(scene_view(sc), texture, uv, n, rgb);
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

aur_status aur_scene_set_lights(aur_ctx* ctx, aur_scene* sc, const aur_light* lights, uint32_t n) {
    AUR_CHECK(ctx && sc, AUR_ERR_INVALID, "aur_scene_set_lights: null argument");
    AUR_CHECK(n == sc->num_lights, AUR_ERR_INVALID, "aur_scene_set_lights: %u lights, scene has %u", n, sc->num_lights);
    for (uint32_t i = 0; i < n; ++i)
        AUR_CHECK(lights[i].type != AUR_LIGHT_AREA || lights[i].samples >= 1, AUR_ERR_INVALID,
                  "aur_scene_set_lights: area light %u needs samples >= 1", i);
    AUR_CUDA(cudaSetDevice(ctx->device));
    if (n) AUR_CUDA(cudaMemcpyAsync(sc->lights, lights, sizeof(aur_light) * n, cudaMemcpyHostToDevice, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    return AUR_OK;
}

aur_status aur_camera_make(aur_float3 position, aur_float3 direction, float fov_x, float fov_y, float aspect,
                           aur_camera* out) {
    AUR_CHECK(out, AUR_ERR_INVALID, "aur_camera_make: null output");
    const f3 fwd = normalize(from(direction));
    const f3 right = cross(fwd, mk3(0.0f, 1.0f, 0.0f));
    const f3 up = cross(right, fwd);
    out->position = position;
    out->forward = to(fwd);
    out->right = to(right);
    out->up = to(up);
    out->tanfov_x = tanf(fov_x);
    out->tanfov_y = tanf(fov_y);
    out->aspect = aspect;
    return AUR_OK;
}

}  // extern "C"
