// render.cu — the plain GPU path tracer and the renderer-helper entry points.
//
// The reference renders sample by sample from the host: generateRays, then
// cudaRaytraceMonteCarlo on 65,536-ray tiles with a device sync per tile,
// then drawPixels (render/monteCarloRaytracer.cpp:81-120). aur_render fuses
// ray generation and integration into one kernel over (sample, pixel) pairs
// of a batch of samples, writes each sample's colour, and a second kernel adds
// the samples to the frame in sample order — the same additions in the same
// order as drawPixels, independent of the thread schedule.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "aur_integrate.cuh"
#include "aur_internal.h"

namespace aur {
namespace {

constexpr int kRenderThreads = 128;
// The fused sample kernel is compiled for 10 resident blocks per SM (at most
// 51 registers, a few hundred bytes of spills served by L1): measured 19 %
// faster than its free 128 registers, which allowed 4 blocks. The per-tile
// kernel (k_raytrace_mc) runs grids of one 65,536-ray tile, too small for
// occupancy to matter, and is left unconstrained (a cap made it slower).
constexpr int kRenderBlocksPerSm = 10;
// The MIS instantiations carry more live state (two strategies per light
// sample, the emitter sample): 8 blocks per SM (64 registers) measured 9-17 %
// faster than 10 or 12, and 4-9 % faster than 6.
constexpr int kRenderBlocksPerSmMis = 8;

inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

const char kAccumMagic[8] = {'A', 'U', 'R', 'A', 'C', 'C', '1', '\0'};

__device__ __forceinline__ StackRef stack_ref(uint32_t* smem, int cap) {
    StackRef s;
    s.lo = reinterpret_cast<float*>(smem) + threadIdx.x;
    s.hi = reinterpret_cast<float*>(smem + cap * blockDim.x) + threadIdx.x;
    s.stride = blockDim.x;
    s.cap = cap;
    return s;
}

// colors[b * P + p] = (rgb, hit) of sample s0 + b at pixel p. kGeneric
// selects the integrator with the specular ray stack, kMis the
// AUR_MODE_PATH_MIS estimator.
template <bool kGeneric, bool kMis>
__global__ void __launch_bounds__(kRenderThreads, kMis ? kRenderBlocksPerSmMis : kRenderBlocksPerSm) k_render_samples(SceneView sc, aur_camera cam, aur_render_params p,
                                                                   uint32_t s0, uint32_t nb, float4* __restrict__ colors,
                                                                   uint32_t* __restrict__ err, int cap) {
    extern __shared__ uint32_t smem[];
    const StackRef stk = stack_ref(smem, cap);
    const uint64_t P = (uint64_t)p.width * p.height;
    const uint64_t t = (uint64_t)blockIdx.x * kRenderThreads + threadIdx.x;
    if (t >= P * nb) return;
    const uint32_t pix = (uint32_t)(t % P);
    const uint32_t s = s0 + (uint32_t)(t / P);
    const PathRay r = camera_ray(cam, p.width, p.height, pix % p.width, pix / p.width, s, p.spp);
    uint32_t visits = 0;
    const SampleResult res =
        kGeneric ? integrate<kMis>(sc, p.max_depth, p.mode, p.seed, p.scene_id, pix, s, r, stk, visits, err)
                 : integrate_diffuse<kMis>(sc, p.max_depth, p.mode, p.seed, p.scene_id, pix, s, r, stk, visits, err);
    colors[t] = make_float4(res.color.x, res.color.y, res.color.z, res.any_hit ? 1.0f : 0.0f);
}

// drawPixels (utility.cu:199-219) for nb consecutive samples, in order.
__global__ void k_accumulate(const float4* __restrict__ colors, uint32_t P, uint32_t nb, float weight,
                             float4* __restrict__ accum) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= P) return;
    float4 a = accum[pix];
    for (uint32_t b = 0; b < nb; ++b) {
        const float4 c = colors[(size_t)b * P + pix];
        if (c.w != 0.0f) {
            a.x += c.x * weight;
            a.y += c.y * weight;
            a.z += c.z * weight;
            a.w += weight;
        }
    }
    accum[pix] = a;
}

// cudaGenerateRaysKernel(Multisample) (utility.cu:18-77)
__global__ void k_generate_rays(uint32_t W, uint32_t H, uint32_t sample, uint32_t samples, aur_camera cam,
                                aur_path_ray* __restrict__ rays, aur_hitpoint* __restrict__ hits) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= W * H) return;
    const PathRay r = camera_ray(cam, W, H, pix % W, pix / W, sample, samples);
    aur_path_ray o;
    o.pos = to(r.pos);
    o.dir = to(r.dir);
    o.t = kInfinity;
    o.weight = 1.0f;
    o.eta = 1.0f;
    rays[pix] = o;
    hits[pix].color = to(mk3(0.0f));
    hits[pix].triangle_id = -1;
}

// cudaRaytraceKernel (monteCarloRaytracer.cu:90-113) on caller-provided rays.
template <bool kGeneric, bool kMis>
__global__ void __launch_bounds__(kRenderThreads) k_raytrace_mc(SceneView sc, aur_render_params p, uint32_t sample,
                                                                uint32_t offset, uint32_t num,
                                                                const aur_path_ray* __restrict__ rays,
                                                                aur_hitpoint* __restrict__ hits,
                                                                uint32_t* __restrict__ err, int cap) {
    extern __shared__ uint32_t smem[];
    const StackRef stk = stack_ref(smem, cap);
    const uint32_t t = blockIdx.x * kRenderThreads + threadIdx.x;
    if (t >= num) return;
    const uint32_t id = offset + t;
    const aur_path_ray in = rays[id];
    PathRay r;
    r.pos = from(in.pos);
    r.dir = from(in.dir);
    r.weight = in.weight;
    r.eta = in.eta;
    r.thr = mk3(in.weight);
    r.pdf = 0.0f;
    uint32_t visits = 0;
    const SampleResult res =
        kGeneric ? integrate<kMis>(sc, p.max_depth, p.mode, p.seed, p.scene_id, id, sample, r, stk, visits, err)
                 : integrate_diffuse<kMis>(sc, p.max_depth, p.mode, p.seed, p.scene_id, id, sample, r, stk, visits,
                                           err);
    aur_hitpoint h = hits[id];
    h.color = to(from(h.color) + res.color);
    if (res.any_hit) {
        h.position = to(res.last_pos);
        h.wo = to(res.last_wo);
        h.u = res.last_u;
        h.v = res.last_v;
        h.triangle_id = (int32_t)res.last_tri;
    }
    hits[id] = h;
}

__global__ void k_draw_pixels(uint32_t P, float weight, const aur_hitpoint* __restrict__ hits,
                              float4* __restrict__ accum) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= P) return;
    const aur_hitpoint h = hits[pix];
    if (h.triangle_id != -1) {
        float4 a = accum[pix];
        a.x += h.color.x * weight;
        a.y += h.color.y * weight;
        a.z += h.color.z * weight;
        a.w += weight;
        accum[pix] = a;
    }
}

// cudaFilterPixelsKernel (kernels/utility.cu:231-252): nine taps clamped to
// the region (the row below clamped to region.top), summed in the
// reference's order. Each thread walks kFilterRows rows of one column and
// keeps the two previous rows' taps in registers, so a pixel costs three
// loads instead of nine.
constexpr uint32_t kFilterRows = 16;

struct Taps {
    float4 l, c, r;
};

__device__ __forceinline__ Taps filter_row(const float4* __restrict__ in, size_t row, uint32_t xl, uint32_t x,
                                           uint32_t xr) {
    Taps t;
    t.l = __ldg(in + row + xl);
    t.c = __ldg(in + row + x);
    t.r = __ldg(in + row + xr);
    return t;
}

__global__ void k_filter_pixels(uint32_t width, aur_rect r, const float4* __restrict__ in, float4* __restrict__ out) {
    const uint32_t x = r.left + blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y0 = r.bottom + (blockIdx.y * blockDim.y + threadIdx.y) * kFilterRows;
    if (x > r.right || y0 > r.top) return;
    const uint32_t xl = x > r.left ? x - 1 : r.left, xr = x < r.right ? x + 1 : r.right;
    const uint32_t y1 = min(y0 + kFilterRows - 1, r.top);
    Taps a = filter_row(in, (size_t)width * (y0 > r.bottom ? y0 - 1 : r.bottom), xl, x, xr);
    Taps b = filter_row(in, (size_t)width * y0, xl, x, xr);
    for (uint32_t y = y0; y <= y1; ++y) {
        const Taps c = filter_row(in, (size_t)width * (y < r.top ? y + 1 : r.top), xl, x, xr);
        float4 v;
#define AUR_TAPS(q)                                                                                                  \
        v.q = a.l.q * 0.0625f + a.c.q * 0.125f + a.r.q * 0.0625f + b.l.q * 0.125f + b.c.q * 0.25f + b.r.q * 0.125f + \
              c.l.q * 0.0625f + c.c.q * 0.125f + c.r.q * 0.0625f
        AUR_TAPS(x);
        AUR_TAPS(y);
        AUR_TAPS(z);
        AUR_TAPS(w);
#undef AUR_TAPS
        out[(size_t)width * y + x] = v;
        a = b;
        b = c;
    }
}

}  // namespace

SceneView scene_view(const aur_scene* sc) {
    SceneView v;
    v.recs = sc->nmh->node_recs;
    v.nodes = sc->nmh->nodes;
    v.perm = sc->nmh->perm;
    v.normals = sc->normals;
    v.sids = sc->shader_ids;
    v.shaders = sc->shaders;
    v.lights = sc->lights;
    v.num_lights = sc->num_lights;
    v.texcoords = sc->texcoords;
    v.texels = sc->texels;
    v.tex_info = sc->tex_info;
    v.verts = sc->nmh->verts;
    v.mis_tri = sc->mis_tri;
    v.mis_cdf = sc->mis_cdf;
    v.mis_pa = sc->mis_pa;
    v.mis_count = sc->mis_count;
    return v;
}

aur_status check_scene_textures(const aur_scene* sc) {
    AUR_CHECK(sc->max_texture <= sc->num_textures, AUR_ERR_INVALID,
              "render: a shader uses texture %u but the scene has %u textures (aur_scene_set_textures)",
              sc->max_texture, sc->num_textures);
    return AUR_OK;
}

aur_status check_params(const aur_render_params* p) {
    AUR_CHECK(p, AUR_ERR_INVALID, "render: null parameters");
    AUR_CHECK(p->width > 0 && p->height > 0 && (uint64_t)p->width * p->height < (1ull << 31), AUR_ERR_INVALID,
              "render: bad frame size %ux%u", p->width, p->height);
    AUR_CHECK(p->spp >= 1 && p->spp <= 65535, AUR_ERR_INVALID, "render: spp %u outside [1, 65535]", p->spp);
    AUR_CHECK(p->max_depth <= AUR_MAX_DEPTH, AUR_ERR_INVALID, "render: max_depth %u > %u", p->max_depth,
              AUR_MAX_DEPTH);
    AUR_CHECK(p->mode == AUR_MODE_REFERENCE || p->mode == AUR_MODE_PATH || p->mode == AUR_MODE_PATH_MIS,
              AUR_ERR_INVALID, "render: unknown mode %u", p->mode);
    const uint32_t end = p->sample_end ? p->sample_end : p->spp;
    AUR_CHECK(p->sample_begin <= end && end <= p->spp, AUR_ERR_INVALID, "render: sample range [%u, %u) outside spp %u",
              p->sample_begin, end, p->spp);
    return AUR_OK;
}

int stack_cap(const aur_scene* sc) { return (int)sc->nmh->levels + 1; }

}  // namespace aur

using namespace aur;

extern "C" {

aur_status aur_render(aur_ctx* ctx, const aur_scene* scene, const aur_camera* camera, const aur_render_params* params,
                      float* accum) {
    AUR_RANGE("aur_render");
    clear_error();
    AUR_CHECK(ctx && scene && camera && accum, AUR_ERR_INVALID, "aur_render: null argument");
    aur_status st = check_params(params);
    if (st == AUR_OK) st = check_scene_textures(scene);
    if (st != AUR_OK) return st;
    const bool mis = params->mode == AUR_MODE_PATH_MIS;
    AUR_CHECK(!mis || scene->num_lights < 32767, AUR_ERR_INVALID,
              "aur_render: AUR_MODE_PATH_MIS takes at most 32766 lights (scene has %u)", scene->num_lights);
    AUR_CUDA(cudaSetDevice(ctx->device));
    if (mis) {
        st = build_mis_table(ctx, scene);
        if (st != AUR_OK) return st;
    }
    const aur_render_params p = *params;
    const uint32_t s0 = p.sample_begin, s1 = p.sample_end ? p.sample_end : p.spp;
    if (s1 == s0) return AUR_OK;
    const uint64_t P = (uint64_t)p.width * p.height;
    const uint32_t batch = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(s1 - s0, (1ull << 24) / P));
    float4* colors = nullptr;
    AUR_CHECK(::aur::dev_malloc_async(&colors, P * batch * sizeof(float4), ctx->stream) == cudaSuccess, AUR_ERR_OOM,
              "aur_render: out of device memory");
    const int cap = stack_cap(scene);
    const size_t smem = (size_t)2 * cap * kRenderThreads * sizeof(uint32_t);
    const SceneView sv = scene_view(scene);
    const float weight = 1.0f / (float)p.spp;
    for (uint32_t s = s0; s < s1; s += batch) {
        const uint32_t nb = std::min(batch, s1 - s);
        const dim3 grid(cdiv(P * nb, kRenderThreads));
        if (scene->has_specular) {
            if (mis)
                k_render_samples<true, true><<<grid, kRenderThreads, smem, ctx->stream>>>(sv, *camera, p, s, nb,
                                                                                      colors, ctx->d_flags, cap);
            else
                k_render_samples<true, false><<<grid, kRenderThreads, smem, ctx->stream>>>(sv, *camera, p, s, nb,
                                                                                       colors, ctx->d_flags, cap);
        } else {
            if (mis)
                k_render_samples<false, true><<<grid, kRenderThreads, smem, ctx->stream>>>(sv, *camera, p, s, nb,
                                                                                       colors, ctx->d_flags, cap);
            else
                k_render_samples<false, false><<<grid, kRenderThreads, smem, ctx->stream>>>(sv, *camera, p, s, nb,
                                                                                        colors, ctx->d_flags, cap);
        }
        k_accumulate<<<cdiv(P, 256), 256, 0, ctx->stream>>>(colors, (uint32_t)P, nb, weight, (float4*)accum);
    }
    cudaFreeAsync(colors, ctx->stream);
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

aur_status aur_generate_rays(aur_ctx* ctx, uint32_t width, uint32_t height, uint32_t sample_id, uint32_t samples,
                             const aur_camera* camera, aur_path_ray* rays, aur_hitpoint* hits) {
    AUR_RANGE("aur_generate_rays");
    AUR_CHECK(ctx && camera && rays && hits, AUR_ERR_INVALID, "aur_generate_rays: null argument");
    AUR_CHECK(width && height && samples >= 1 && sample_id < samples, AUR_ERR_INVALID,
              "aur_generate_rays: bad size or sample");
    AUR_CUDA(cudaSetDevice(ctx->device));
    const uint32_t P = width * height;
    k_generate_rays<<<cdiv(P, 256), 256, 0, ctx->stream>>>(width, height, sample_id, samples, *camera, rays, hits);
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

aur_status aur_raytrace_monte_carlo(aur_ctx* ctx, const aur_scene* scene, const aur_render_params* params,
                                    uint32_t sample_id, uint32_t offset, uint32_t num_rays, aur_path_ray* rays,
                                    aur_hitpoint* hits) {
    AUR_RANGE("aur_raytrace_monte_carlo");
    AUR_CHECK(ctx && scene && params && rays && hits, AUR_ERR_INVALID, "aur_raytrace_monte_carlo: null argument");
    AUR_CHECK(params->max_depth <= AUR_MAX_DEPTH && params->mode <= AUR_MODE_PATH_MIS, AUR_ERR_INVALID,
              "aur_raytrace_monte_carlo: bad parameters");
    aur_status st = check_scene_textures(scene);
    if (st != AUR_OK) return st;
    const bool mis = params->mode == AUR_MODE_PATH_MIS;
    AUR_CHECK(!mis || scene->num_lights < 32767, AUR_ERR_INVALID,
              "aur_raytrace_monte_carlo: AUR_MODE_PATH_MIS takes at most 32766 lights (scene has %u)",
              scene->num_lights);
    AUR_CUDA(cudaSetDevice(ctx->device));
    if (num_rays == 0) return AUR_OK;
    if (mis) {
        st = build_mis_table(ctx, scene);
        if (st != AUR_OK) return st;
    }
    const int cap = stack_cap(scene);
    const size_t smem = (size_t)2 * cap * kRenderThreads * sizeof(uint32_t);
    const dim3 grid(cdiv(num_rays, kRenderThreads));
    const SceneView sv = scene_view(scene);
    const aur_render_params& p = *params;
    aur_path_ray* r = rays;
    aur_hitpoint* h = hits;
    if (scene->has_specular) {
        if (mis)
            k_raytrace_mc<true, true><<<grid, kRenderThreads, smem, ctx->stream>>>(sv, p, sample_id, offset, num_rays,
                                                                                  r, h, ctx->d_flags, cap);
        else
            k_raytrace_mc<true, false><<<grid, kRenderThreads, smem, ctx->stream>>>(sv, p, sample_id, offset,
                                                                                   num_rays, r, h, ctx->d_flags, cap);
    } else {
        if (mis)
            k_raytrace_mc<false, true><<<grid, kRenderThreads, smem, ctx->stream>>>(sv, p, sample_id, offset,
                                                                                   num_rays, r, h, ctx->d_flags, cap);
        else
            k_raytrace_mc<false, false><<<grid, kRenderThreads, smem, ctx->stream>>>(sv, p, sample_id, offset,
                                                                                    num_rays, r, h, ctx->d_flags, cap);
    }
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

aur_status aur_draw_pixels(aur_ctx* ctx, uint32_t width, uint32_t height, float weight, const aur_hitpoint* hits,
                           float* accum) {
    AUR_RANGE("aur_draw_pixels");
    AUR_CHECK(ctx && hits && accum, AUR_ERR_INVALID, "aur_draw_pixels: null argument");
    AUR_CUDA(cudaSetDevice(ctx->device));
    const uint32_t P = width * height;
    if (P == 0) return AUR_OK;
    k_draw_pixels<<<cdiv(P, 256), 256, 0, ctx->stream>>>(P, weight, hits, (float4*)accum);
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

aur_status aur_filter_pixels(aur_ctx* ctx, uint32_t width, uint32_t height, const aur_rect* region, const float* in,
                             float* out) {
    AUR_RANGE("aur_filter_pixels");
    clear_error();
    AUR_CHECK(ctx && in && out, AUR_ERR_INVALID, "aur_filter_pixels: null argument");
    AUR_CHECK(in != out, AUR_ERR_INVALID, "aur_filter_pixels: in and out must be distinct buffers");
    AUR_CHECK(width && height && (uint64_t)width * height < (1ull << 31), AUR_ERR_INVALID,
              "aur_filter_pixels: bad frame size %ux%u", width, height);
    const aur_rect r = region ? *region : aur_rect{0u, width - 1, 0u, height - 1};
    AUR_CHECK(r.left <= r.right && r.right < width && r.bottom <= r.top && r.top < height, AUR_ERR_INVALID,
              "aur_filter_pixels: region [%u, %u] x [%u, %u] outside %ux%u", r.left, r.right, r.bottom, r.top, width,
              height);
    AUR_CHECK((r.top - r.bottom) / (4u * kFilterRows) < 65535u, AUR_ERR_INVALID,
              "aur_filter_pixels: region taller than %u rows", 65535u * 4u * kFilterRows);
    AUR_CUDA(cudaSetDevice(ctx->device));
    const dim3 block(32, 4);
    const dim3 grid(cdiv(r.right - r.left + 1, block.x), cdiv(r.top - r.bottom + 1, block.y * kFilterRows));
    k_filter_pixels<<<grid, block, 0, ctx->stream>>>(width, r, reinterpret_cast<const float4*>(in),
                                                    reinterpret_cast<float4*>(out));
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

aur_status aur_accum_save(aur_ctx* ctx, const char* path, uint32_t width, uint32_t height, uint32_t samples_done,
                          uint32_t spp, const float* accum) {
    clear_error();
    AUR_CHECK(ctx && path && accum, AUR_ERR_INVALID, "aur_accum_save: null argument");
    AUR_CHECK(width && height && (uint64_t)width * height < (1ull << 31), AUR_ERR_INVALID,
              "aur_accum_save: bad frame size %ux%u", width, height);
    AUR_CHECK(samples_done <= spp, AUR_ERR_INVALID, "aur_accum_save: %u samples done of %u", samples_done, spp);
    AUR_CUDA(cudaSetDevice(ctx->device));
    const size_t bytes = (size_t)width * height * sizeof(float4);
    std::vector<unsigned char> host(bytes);
    AUR_CUDA(cudaMemcpyAsync(host.data(), accum, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    FILE* f = std::fopen(path, "wb");
    AUR_CHECK(f, AUR_ERR_INVALID, "aur_accum_save: cannot open %s for writing", path);
    const uint32_t head[4] = {width, height, samples_done, spp};
    const bool good = std::fwrite(kAccumMagic, 1, 8, f) == 8 && std::fwrite(head, 4, 4, f) == 4 &&
                      std::fwrite(host.data(), 1, bytes, f) == bytes;
    const bool closed = std::fclose(f) == 0;
    AUR_CHECK(good && closed, AUR_ERR_INVALID, "aur_accum_save: write to %s failed", path);
    return AUR_OK;
}

aur_status aur_accum_load(aur_ctx* ctx, const char* path, uint32_t width, uint32_t height, uint32_t* samples_done,
                          uint32_t* spp, float* accum) {
    clear_error();
    AUR_CHECK(ctx && path && accum && samples_done && spp, AUR_ERR_INVALID, "aur_accum_load: null argument");
    FILE* f = std::fopen(path, "rb");
    AUR_CHECK(f, AUR_ERR_INVALID, "aur_accum_load: cannot open %s", path);
    char magic[8];
    uint32_t head[4];
    const bool good = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kAccumMagic, 8) == 0 &&
                      std::fread(head, 4, 4, f) == 4;
    if (!good || head[0] != width || head[1] != height || head[2] > head[3]) {
        std::fclose(f);
        return fail(AUR_ERR_INVALID, "aur_accum_load: %s is not a %ux%u accumulation checkpoint", path, width, height);
    }
    const size_t bytes = (size_t)width * height * sizeof(float4);
    std::vector<unsigned char> host(bytes);
    const bool body = std::fread(host.data(), 1, bytes, f) == bytes;
    std::fclose(f);
    AUR_CHECK(body, AUR_ERR_INVALID, "aur_accum_load: %s is truncated", path);
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaMemcpyAsync(accum, host.data(), bytes, cudaMemcpyHostToDevice, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    *samples_done = head[2];
    *spp = head[3];
    return AUR_OK;
}

aur_status aur_clear_pixels(aur_ctx* ctx, uint32_t width, uint32_t height, float* accum) {
    AUR_CHECK(ctx && accum, AUR_ERR_INVALID, "aur_clear_pixels: null argument");
    AUR_CUDA(cudaSetDevice(ctx->device));
    AUR_CUDA(cudaMemsetAsync(accum, 0, (size_t)width * height * sizeof(float4), ctx->stream));
    return AUR_OK;
}

}  // extern "C"
