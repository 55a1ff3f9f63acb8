// adjoint.cu — path-replay backpropagation through the integrator.
//
// Gradients of a loss L(image) with respect to every shader's diffuse colour,
// every shader's emission colour and every light's colour, given dL/dimage.
// No counterpart in the
// reference. Method: path replay backpropagation (D. Vicini, S. Speierer,
// W. Jakob, "Path Replay Backpropagation", ACM TOG 40(4), 2021), in one pass
// per camera sample: the integrator's ray stack (monteCarloRaytracer.cu:26-88,
// the same estimator and counter-RNG draws as aur_render) is walked again,
// and at vertex k with throughput T_k and Lambert colour
// c_k = diffuse_color * diffuse the replay adds
//   dL/dc_k  += g * (T_k * D_k / c_k + L_after_k / c_k)
//   dL/dcolor_l += g * T_k * dD_k/dcolor_l
// where D_k is the direct light at k (ambient, delta and area terms,
// radiance.cuh:13-80), g = dL/dpixel / spp, and L_after_k the radiance of
// the rays that descend from k's diffuse bounce (c_k enters the throughput
// f*|cos|/pdf of every later vertex, BSDF::samplef, bsdf.cuh:222-236). The
// rays that descend from a bounce are exactly those traced between its pop
// and the stack's return to its height before the push (depth first), so a
// marker per pending bounce sums that radiance and hands it over when the
// subtree ends; no primal pass is needed. D_k / c_k is evaluated directly
// (f replaced by 1/pi), so the direct part needs no division; the
// later-vertex part divides by c_k and is skipped for colour channels that
// are exactly zero.
// Emission E_s of shader s enters linearly: at every vertex on s as T_k * E_s
// (times the emission's MIS weight in AUR_MODE_PATH_MIS,
// monteCarloRaytracer.cu:42), and in AUR_MODE_PATH_MIS through the emitter
// sample of every vertex, f * E_s * G with G the sample's geometric factor
// over its density. So
//   dL/dE_s += g * T_k * w_k  (vertex on s),  g * T_k * f_k * G  (emitter on s, visible).
// Neither the MIS weights nor the light-selection table depend on E_s: the
// table weighs triangles by the shader's scalar `emission` times area
// (emitter.cu's weight), not by its emission colour.
#include <algorithm>
#include <vector>

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "aur_integrate.cuh"
#include "aur_internal.h"

namespace aur {
namespace {

constexpr int kAdjThreads = 128;
// The replay kernel is compiled for 8 resident blocks per SM (at most 64
// registers): 24 % faster than its free 150-160 registers (3 blocks).
constexpr int kAdjBlocksPerSm = 8;
constexpr uint32_t kSharedLights = 64;

// Per-unit-colour radiance of a light sample (Lr = color * s), light.cuh:228-259.
__device__ __forceinline__ float light_scale(const aur_light& L, const f3& dir, float t) {
    if (L.type == AUR_LIGHT_AMBIENT) return L.intensity * (1.0f - L.ambient);
    if (L.type == AUR_LIGHT_POINT) return L.intensity / (t * t);
    if (L.type == AUR_LIGHT_DIRECTIONAL) return L.intensity;
    return L.intensity * fmaxf(0.0f, dot(from(L.direction), -dir));
}

// Adds g_c1 * d(colour1)/d(diffuse_color) = g_c1 * diffuse to shader si's
// gradient (colour1 = diffuse_color * diffuse; a textured shader's colour is
// not its diffuse_color, so it gets none). Lanes that hit the same shader
// (large triangles are hit by most of a warp) are summed first, so a warp
// issues one atomic per shader instead of one per lane.
__device__ __forceinline__ void add_diffuse_grad(float* __restrict__ d_diffuse, uint32_t si, const aur_shader* sh,
                                                 const f3& g_c1) {
    const f3 gd = sh->texture > 0 ? mk3(0.0f) : g_c1 * sh->diffuse;
    namespace cg = cooperative_groups;
    const cg::coalesced_group active = cg::coalesced_threads();
    const cg::coalesced_group same = cg::labeled_partition(active, si);
    const float sx = cg::reduce(same, gd.x, cg::plus<float>());
    const float sy = cg::reduce(same, gd.y, cg::plus<float>());
    const float sz = cg::reduce(same, gd.z, cg::plus<float>());
    if (same.thread_rank() == 0 && (sx != 0.0f || sy != 0.0f || sz != 0.0f)) {
        atomicAdd(d_diffuse + 3 * si + 0, sx);
        atomicAdd(d_diffuse + 3 * si + 1, sy);
        atomicAdd(d_diffuse + 3 * si + 2, sz);
    }
}

// Adds g to shader si's entry of a per-shader gradient (emission), summed per
// warp over the lanes that hit the same shader first.
__device__ __forceinline__ void add_shader_grad(float* __restrict__ d, uint32_t si, const f3& gs) {
    namespace cg = cooperative_groups;
    const cg::coalesced_group active = cg::coalesced_threads();
    const cg::coalesced_group same = cg::labeled_partition(active, si);
    const float sx = cg::reduce(same, gs.x, cg::plus<float>());
    const float sy = cg::reduce(same, gs.y, cg::plus<float>());
    const float sz = cg::reduce(same, gs.z, cg::plus<float>());
    if (same.thread_rank() == 0 && (sx != 0.0f || sy != 0.0f || sz != 0.0f)) {
        atomicAdd(d + 3 * si + 0, sx);
        atomicAdd(d + 3 * si + 1, sy);
        atomicAdd(d + 3 * si + 2, sz);
    }
}

// Direct light at a hit as the primal computes it (direct_light), with its
// derivatives: Dp receives the direct light per unit Lambert colour, and the
// light-colour gradients g * thr * d(direct)/d(colour_l) are added (light 0
// into gl0, the others to d_light). ew: the emission's MIS weight; bounce:
// whether a diffuse bounce follows the hit (both for AUR_MODE_PATH_MIS).
// With d_emission, the emission gradients of the hit's own shader si and of
// the emitter sample's shader are added too.
template <bool kMis>
__device__ __forceinline__ f3 direct_grad(const SceneView& sc, const aur_shader* sh, const Bsdf& b, const f3& f,
                                          const f3& position, const f3& wo, float ew, bool bounce, uint32_t seed,
                                          uint32_t scene, uint32_t pixel, uint32_t sample, uint32_t rix, const f3& thr,
                                          const f3& g, float* __restrict__ d_light, f3& gl0, f3& Dp,
                                          float* __restrict__ d_emission, uint32_t si, const StackRef& stk,
                                          uint32_t& visits, uint32_t* err) {
    f3 Li = kMis ? from(sh->emission_color) * ew : from(sh->emission_color);
    if (d_emission) add_shader_grad(d_emission, si, kMis ? (g * thr) * ew : g * thr);
    Dp = mk3(0.0f);   // direct light per unit Lambert colour
    for (uint32_t i = 0; i < sc.num_lights; ++i) {
        const aur_light& L = sc.lights[i];
        f3 dl = mk3(0.0f);   // d(direct)/d(light colour), per channel
        if (L.type == AUR_LIGHT_AMBIENT) {
            const f3 X = (from(L.color) * L.intensity) * L.ambient;
            Li = Li + f * X;
            Dp = Dp + X * kInvPi;
            dl = dl + f * (L.intensity * L.ambient);
        }
        if (L.type != AUR_LIGHT_AREA) {
            f3 wdir; float wt, pdf;
            const f3 Ls = sample_light(L, position, seed, scene, pixel, sample, rix, 0u, wdir, wt, pdf);
            if (pdf > 0.0f && !zero(Ls)) {
                float du = 0.0f, dv = 0.0f;
                if (!zero(f) &&
                    traverse<true>(sc.recs, sc.nodes, sc.perm, position, wdir, wt, du, dv, stk, visits, err) == kNoPrim) {
                    const float cs = fmaxf(0.0f, dot(wdir, b.N));
                    Li = Li + f * Ls * cs;
                    Dp = Dp + Ls * (kInvPi * cs);
                    dl = dl + f * (light_scale(L, wdir, wt) * cs);
                }
            }
        } else if (kMis) {
            // both strategies of every sample, as in direct_light_mis
            f3 acc = mk3(0.0f), accp = mk3(0.0f), accl = mk3(0.0f);
            const AreaLightMis q = area_light_setup(L, f);
            if (q.active) {
                for (int32_t j = 0; j < L.samples; ++j) {
                    f3 Ls = mk3(0.0f);
                    for (int h2 = 0; h2 < 2; ++h2) {
                        const ShadowSample ss =
                            h2 == 0 ? area_light_sample(q, i, (uint32_t)j, b, f, position, wo, seed, scene, pixel,
                                                        sample, rix)
                                    : area_bsdf_sample(q, i, (uint32_t)j, b, f, position, wo, seed, scene, pixel,
                                                       sample, rix);
                        float du = 0.0f, dv = 0.0f, tt = ss.tmax;
                        if (ss.cand && traverse<true>(sc.recs, sc.nodes, sc.perm, ss.o, ss.d, tt, du, dv, stk,
                                                      visits, err) == kNoPrim) {
                            Ls = Ls + ss.c;
                            accp = accp + ss.e * (ss.geo * kInvPi);
                            accl = accl + f * (L.intensity * ss.geo);
                        }
                    }
                    acc = acc + Ls;
                }
            }
            const float ns = (float)L.samples;
            Li = Li + mk3(acc.x / ns, acc.y / ns, acc.z / ns);
            Dp = Dp + mk3(accp.x / ns, accp.y / ns, accp.z / ns);
            dl = dl + mk3(accl.x / ns, accl.y / ns, accl.z / ns);
        } else {
            f3 acc = mk3(0.0f), accp = mk3(0.0f), accl = mk3(0.0f);
            for (int32_t j = 0; j < L.samples; ++j) {
                f3 wdir; float wt, lpdf;
                const f3 Lr = sample_light(L, position, seed, scene, pixel, sample, rix, light_slot(i, (uint32_t)j),
                                           wdir, wt, lpdf);
                f3 wpos = position;
                wpos.x += kEpsilon * wdir.x;
                wpos.y += kEpsilon * wdir.y;
                wpos.z += kEpsilon * wdir.z;
                wt += kEpsilon;
                if (lpdf > 0.0f && !zero(Lr)) {
                    float du = 0.0f, dv = 0.0f;
                    if (!zero(f) &&
                        traverse<true>(sc.recs, sc.nodes, sc.perm, wpos, wdir, wt, du, dv, stk, visits, err) == kNoPrim) {
                        const float cs = fmaxf(0.0f, dot(wdir, b.N));
                        acc = acc + f * Lr * cs;
                        accp = accp + Lr * (kInvPi * cs);
                        accl = accl + f * (light_scale(L, wdir, wt - kEpsilon) * cs);
                    }
                }
            }
            const float ns = (float)L.samples;
            Li = Li + mk3(acc.x / ns, acc.y / ns, acc.z / ns);
            Dp = Dp + mk3(accp.x / ns, accp.y / ns, accp.z / ns);
            dl = dl + mk3(accl.x / ns, accl.y / ns, accl.z / ns);
        }
        const f3 gl = g * thr * dl;
        if (i == 0) {
            gl0 = gl0 + gl;
        } else if (gl.x != 0.0f || gl.y != 0.0f || gl.z != 0.0f) {
            atomicAdd(d_light + 3 * i + 0, gl.x);
            atomicAdd(d_light + 3 * i + 1, gl.y);
            atomicAdd(d_light + 3 * i + 2, gl.z);
        }
    }
    if (kMis) {   // the emitter sample (direct_light_mis)
        const ShadowSample ss =
            emitter_shadow_sample(sc, b, f, position, wo, bounce, seed, scene, pixel, sample, rix);
        float du = 0.0f, dv = 0.0f, tt = ss.tmax;
        const bool vis = ss.cand && traverse<true>(sc.recs, sc.nodes, sc.perm, ss.o, ss.d, tt, du, dv, stk,
                                                   visits, err) == kNoPrim;
        Li = Li + (vis ? ss.c : mk3(0.0f));
        if (vis) Dp = Dp + ss.e * (ss.geo * kInvPi);
        if (d_emission && vis) add_shader_grad(d_emission, ss.esi, (g * thr) * (f * ss.geo));
    }
    return Li;
}

// The replay of one camera sample: integrate()'s ray stack
// (monteCarloRaytracer.cu:26-88) walked again with the same draws. A hit's
// colour Li * thr depends on its own vertex's colour through the direct
// light, and on the colour of every vertex whose diffuse bounce lies on its
// way from the camera through thr, as a factor. The rays that descend from a
// diffuse bounce are exactly those traced between its pop and the return of
// the stack to the height it had before the bounce was pushed (depth first),
// so a marker per pending bounce sums its subtree's radiance; when the
// subtree ends, g * subtree / c_k goes to the bouncing vertex's shader.
// Gradients of light 0 are summed in `gl0` (reduced once per block by the
// caller); those of further lights go to d_light with atomics. kMis:
// AUR_MODE_PATH_MIS, whose MIS weights do not depend on the colours (Lambert
// densities are |cos| / pi), so every direct term stays linear in the vertex
// colour and in the light colour. One pass replaces a primal pass (each
// sample's radiance) plus a replay: 29.3 -> 21.1 ms on the differentiable
// workload (256x256, 64 spp, path mode).
template <bool kMis>
__device__ void replay_stack(const SceneView& sc, uint32_t max_depth, uint32_t mode, uint32_t seed, uint32_t scene,
                             uint32_t pixel, uint32_t sample, const PathRay& primary, const StackRef& stk,
                             const f3& g, float* __restrict__ d_diffuse, float* __restrict__ d_light,
                             float* __restrict__ d_emission, f3& gl0, uint32_t& visits, uint32_t* err) {
    struct Marker {
        f3 col0, c1;          // colour before the subtree, the bouncing vertex's Lambert colour
        const aur_shader* sh;
        uint32_t si;
        int base;             // stack height before the bounce was pushed
    };
    PathRay stack[AUR_MAX_DEPTH + 2];
    Marker mk[AUR_MAX_DEPTH + 2];
    int sp = 0, nm = 0;
    stack[sp++] = primary;
    int depth = 0;
    f3 col = mk3(0.0f);
    uint32_t ray_index = 0;
    const int maxd = (int)max_depth;
    const bool path = kMis || mode == AUR_MODE_PATH;
    auto close = [&](const Marker& m) {
        const f3 sub = col - m.col0;
        f3 dc;
        dc.x = m.c1.x != 0.0f ? sub.x / m.c1.x : 0.0f;
        dc.y = m.c1.y != 0.0f ? sub.y / m.c1.y : 0.0f;
        dc.z = m.c1.z != 0.0f ? sub.z / m.c1.z : 0.0f;
        add_diffuse_grad(d_diffuse, m.si, m.sh, g * dc);
    };
    for (;;) {
        while (nm > 0 && sp <= mk[nm - 1].base) close(mk[--nm]);
        if (!(depth <= maxd && sp > 0)) break;
        PathRay ray = stack[--sp];
        const uint32_t rix = ray_index++;
        float t = kInfinity, u = 0.0f, v = 0.0f;
        const uint32_t tri = traverse<false>(sc.recs, sc.nodes, sc.perm, ray.pos, ray.dir, t, u, v, stk, visits, err);
        if (tri == kNoPrim) continue;
        const f3 position = ray.pos + (ray.dir * t);
        const f3 wo = -ray.dir;
        const uint32_t sid = sc.sids[tri];
        const uint32_t si = sid > 0 ? sid - 1 : 0;
        const aur_shader* sh = sc.shaders + si;
        const float refl = sh->reflectivity, trans = sh->translucence;
        const Bsdf b = get_bsdf(sc, sh, tri, u, v);
        const f3 f = bsdf_f(b);
        const bool specular = refl > 0.0f || trans > 0.0f;
        const bool bounce_follows = !specular && depth + 1 <= maxd;   // as direct_light is told in the primal
        const float ew = kMis ? emission_weight(sc, tri, ray.dir, t, ray.pdf) : 1.0f;
        // the continuation changes the ray's throughput before the colour
        // update; the direct light's derivatives scale with that throughput
        PathRay cur = ray;
        const Continuation kc =
            continue_ray<kMis>(sh, b, cur, position, wo, path, depth, maxd, seed, scene, pixel, sample, rix);
        f3 Dp;
        const f3 Li = direct_grad<kMis>(sc, sh, b, f, position, wo, ew, bounce_follows, seed, scene, pixel, sample, rix,
                                        cur.thr, g, d_light, gl0, Dp, d_emission, si, stk, visits, err);
        add_diffuse_grad(d_diffuse, si, sh, g * (cur.thr * Dp));
        col = col + Li * cur.thr;
        for (int q = 0; q < kc.n; ++q) {
            if (kc.bounced && q == kc.n - 1) {   // the diffuse bounce: its subtree scales with this vertex's colour
                Marker m;
                m.col0 = col;
                m.c1 = b.color1;
                m.sh = sh;
                m.si = si;
                m.base = sp;
                mk[nm++] = m;
            }
            if (sp < AUR_MAX_DEPTH + 2) stack[sp++] = kc.ray[q]; else atomicOr(err, 2u);
        }
    }
    while (nm > 0) close(mk[--nm]);
}

__device__ __forceinline__ StackRef adj_stack(uint32_t* smem, int cap) {
    StackRef stk;
    stk.lo = reinterpret_cast<float*>(smem) + threadIdx.x;
    stk.hi = reinterpret_cast<float*>(smem + cap * kAdjThreads) + threadIdx.x;
    stk.stride = kAdjThreads;
    stk.cap = cap;
    return stk;
}

// Replay kernel: one thread per camera sample of samples [s0, s0 + nb).
template <bool kMis>
__global__ void __launch_bounds__(kAdjThreads, kAdjBlocksPerSm) k_adj_replay(SceneView sc, aur_camera cam,
                                                                            aur_render_params p, uint32_t s0,
                                                                            uint32_t nb,
                                                                            const float4* __restrict__ d_image,
                                                                            float* __restrict__ d_diffuse,
                                                                            float* __restrict__ d_light,
                                                                            float* __restrict__ d_emission,
                                                                            uint32_t* __restrict__ err, int cap) {
    extern __shared__ uint32_t smem[];
    const StackRef stk = adj_stack(smem, cap);
    // light gradients are reduced in shared memory first (one light is hit by every sample)
    float* s_light = reinterpret_cast<float*>(smem + 2 * cap * kAdjThreads);
    const bool shared_lights = sc.num_lights <= kSharedLights;
    if (shared_lights)
        for (uint32_t i = threadIdx.x; i < 3 * sc.num_lights; i += kAdjThreads) s_light[i] = 0.0f;
    __syncthreads();
    const uint64_t P = (uint64_t)p.width * p.height;
    const uint64_t t = (uint64_t)blockIdx.x * kAdjThreads + threadIdx.x;
    f3 gl0 = mk3(0.0f);
    if (t < P * nb) {
        const uint32_t pix = (uint32_t)(t % P);
        const uint32_t s = s0 + (uint32_t)(t / P);
        const PathRay r = camera_ray(cam, p.width, p.height, pix % p.width, pix / p.width, s, p.spp);
        const float4 di = d_image[pix];
        const float w = 1.0f / (float)p.spp;
        const f3 g = mk3(di.x * w, di.y * w, di.z * w);
        uint32_t visits = 0;
        replay_stack<kMis>(sc, p.max_depth, p.mode, p.seed, p.scene_id, pix, s, r, stk, g, d_diffuse,
                           shared_lights ? s_light : d_light, d_emission, gl0, visits, err);
    }
    // light 0: warp sum, then one shared atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        gl0.x += __shfl_down_sync(0xffffffffu, gl0.x, o);
        gl0.y += __shfl_down_sync(0xffffffffu, gl0.y, o);
        gl0.z += __shfl_down_sync(0xffffffffu, gl0.z, o);
    }
    if ((threadIdx.x & 31) == 0 && sc.num_lights > 0) {
        float* dst = shared_lights ? s_light : d_light;
        atomicAdd(dst + 0, gl0.x);
        atomicAdd(dst + 1, gl0.y);
        atomicAdd(dst + 2, gl0.z);
    }
    __syncthreads();
    if (shared_lights)
        for (uint32_t i = threadIdx.x; i < 3 * sc.num_lights; i += kAdjThreads)
            if (s_light[i] != 0.0f) atomicAdd(d_light + i, s_light[i]);
}

inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace


}  // namespace aur

using namespace aur;

extern "C" {

aur_status aur_render_adjoint(aur_ctx* ctx, const aur_scene* scene, const aur_camera* camera,
                              const aur_render_params* params, const float* d_image, float* d_diffuse,
                              float* d_light_color, float* d_emission) {
    AUR_RANGE("aur_render_adjoint");
    clear_error();
    AUR_CHECK(ctx && scene && camera && d_image && d_diffuse && (d_light_color || scene->num_lights == 0),
              AUR_ERR_INVALID, "aur_render_adjoint: null argument");
    aur_status st = check_params(params);
    if (st == AUR_OK) st = check_scene_textures(scene);
    if (st != AUR_OK) return st;
    const bool mis = params->mode == AUR_MODE_PATH_MIS;
    AUR_CHECK(!mis || scene->num_lights < 32767, AUR_ERR_INVALID,
              "aur_render_adjoint: AUR_MODE_PATH_MIS takes at most 32766 lights (scene has %u)", scene->num_lights);
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
    const int cap = (int)scene->nmh->levels + 1;
    const size_t smem = (size_t)2 * cap * kAdjThreads * sizeof(uint32_t) + 3 * kSharedLights * sizeof(float);
    AUR_CUDA(cudaFuncSetAttribute(k_adj_replay<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    AUR_CUDA(cudaFuncSetAttribute(k_adj_replay<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const SceneView sv = scene_view(scene);
    const float4* di = (const float4*)d_image;
    for (uint32_t s = s0; s < s1; s += batch) {
        const uint32_t nb = std::min(batch, s1 - s);
        const uint32_t grid = cdiv(P * nb, kAdjThreads);
        if (mis)
            k_adj_replay<true><<<grid, kAdjThreads, smem, ctx->stream>>>(sv, *camera, p, s, nb, di, d_diffuse,
                                                                        d_light_color, d_emission, ctx->d_flags, cap);
        else
            k_adj_replay<false><<<grid, kAdjThreads, smem, ctx->stream>>>(sv, *camera, p, s, nb, di, d_diffuse,
                                                                         d_light_color, d_emission, ctx->d_flags, cap);
    }
    AUR_CUDA(cudaGetLastError());
    return AUR_OK;
}

}  // extern "C"
