// wavefront.cu — batched wavefront path tracer: many scenes, one graph launch.
//
// Estimator: exactly the plain integrator's (aur_integrate.cuh, after
// kernels/monteCarloRaytracer.cu:23-113) — same counter-RNG keys (seed,
// scene id) x (pixel, sample, ray index, slot), same arithmetic in the same
// order — so every path sample has the same value as in aur_render and the
// frames are identical. A path slot carries one camera sample; in batches
// with specular shaders it also keeps the sample's ray stack, so the
// reflection, refraction and bounce rays are traced one after the other in
// the plain integrator's order. In AUR_MODE_PATH_MIS the
// shade stage queues both strategies of every area-light sample and the
// emitter sample (the ShadowSample helpers of aur_integrate.cuh), and the
// combine stage adds them in the plain integrator's order.
//
// Structure (Laine, Karras, Aila, "Megakernels considered harmful", HPG'13):
// a pool of paths in flight (SoA state) and index queues; each iteration runs
//   generate  : refill free pool slots with new (scene, pixel, sample) items
//   extend    : closest hit of every queued path          (persistent kernel)
//   shade     : BSDF, light samples -> shadow-ray queue, bounce direction
//   shadow    : any hit of every shadow ray                (persistent kernel)
//   combine   : Li in the reference's light order, colour += Li * throughput,
//               continue (next queue) or finish (write the sample, free slot)
// Samples are processed in waves of `samples_per_wave` per pixel; a wave's
// samples are added to each frame in sample order afterwards, as drawPixels
// would. The whole render is one CUDA graph: an outer conditional while node
// over waves and an inner one over iterations, both bounded by iteration
// limits that stop the loop and raise an error instead of spinning.
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

#include "aur_integrate.cuh"
#include "aur_internal.h"

namespace aur {
namespace {

constexpr int kMaxLightSlots = 32;
// WfCtl::error bits: 1 = iteration limit reached, 2 = a path needed more
// light samples than the batch was sized for (aur_scene_set_lights after
// aur_batch_create).
constexpr uint32_t kWfErrLightSlots = 2u;
// WfCtl::error bit 4: a path's ray stack would have overflowed (the plain
// integrator's stack check; cannot happen within AUR_MAX_DEPTH).
constexpr uint32_t kWfErrStack = 4u;
// Specular batches keep each sample's pending rays (the ray stack of the
// plain integrator, monteCarloRaytracer.cu:26-88) with its path.
constexpr uint32_t kWfStack = AUR_MAX_DEPTH + 2;
// Largest block of the stage kernels: the traversal and shading stages are
// compiled for it with at most 64 registers (4 blocks of 256 per SM), which
// measured faster than their unconstrained 70-72 registers.
constexpr int kWfMaxBlock = 256;

struct WfScene {
    const float4* recs;
    const uint32_t* perm;
    const float* normals;
    const uint16_t* sids;
    const aur_shader* shaders;
    const aur_light* lights;
    const float* texcoords;
    const uchar4* texels;
    const uint4* tex_info;
    // AUR_MODE_PATH_MIS: NMH-ordered vertices and the light-selection table
    const float* verts;
    const uint32_t* mis_tri;
    const float* mis_cdf;
    const float* mis_pa;
    uint32_t mis_count;
    uint32_t nodes;
    float packet_span;   // largest origin spread of a warp packet (1/64 of the soup's extent)
    uint32_t num_lights;
    uint32_t width, height;
    uint32_t pix_off;
    uint32_t scene_id;
    aur_camera cam;
};

struct WfCtl {
    unsigned long long total_ext, total_shadow;   // work counters (reset per render)
    uint32_t error;
    uint32_t total_iters;
    uint32_t wave, num_waves;
    uint32_t s_begin, s_end, spw;
    uint32_t s0, nb;
    uint32_t items_total, items_issued;
    uint32_t ext_count[2];
    uint32_t shadow_count;
    uint32_t free_count;
    uint32_t iter, iter_limit;
    uint32_t ext_fetch, shadow_fetch;   // dynamic-fetch cursors of the extend / shadow kernels
    uint32_t ext_chunk;                 // chunk cursor of k_wf_extend_packets
    uint32_t ext_defer;                 // chunks it left to k_wf_extend
};

struct WfArgs {
    WfCtl* ctl;
    const WfScene* scenes;
    const uint32_t* pix_off;      // num_scenes + 1
    float4* const* accum;         // per scene frame
    uint32_t num_scenes;
    uint32_t P_tot;
    uint32_t Q;                   // paths in flight
    uint32_t M;                   // light-sample slots per path
    uint32_t spp, max_depth, mode, seed;
    int cap;                      // traversal stack entries
    // path state, indexed by pool slot
    float4* o;      // origin
    float4* d;      // direction
    float4* thr;    // throughput, w = density of the bounce that made the ray (0: camera ray)
    float4* col;    // colour, w = any hit
    float4* hit;    // t, u, v, tri
    uint4* meta;    // item, depth, ray index, scene
    float4* ndir;   // bounce direction, w = 1 if the path continues
    float4* nthr;   // bounce throughput, w = the bounce's density (AUR_MODE_PATH_MIS)
    float4* fsh;    // f = color1 / pi
    float4* emi;    // emission
    float4* cj;     // Q * M light-sample contributions, w = candidate
    uint32_t* vis;  // visibility bits per slot
    // queues
    uint32_t* ext_q[2];
    uint32_t* free_list;
    float4* sh_o;   // shadow ray origin, w = tmax
    float4* sh_d;   // shadow ray direction, w = (slot << 5 | light slot) bits
    uint32_t* defer;   // chunks of 32 extend-queue entries left to k_wf_extend
    float4* out;    // per wave: nb * P_tot sample colours, indexed by item
    // specular batches: per slot a stack of kWfStack pending rays, entry e
    // component k (pos + weight, dir + eta, thr + pdf) at stk[(e * 3 + k) * Q + slot]
    float4* stk;
    uint32_t* sp;   // stack depth per slot
    cudaGraphConditionalHandle h_inner, h_outer;
    uint32_t in_graph;   // 1 when launched by the graph: only then may kernels set its conditionals
};

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

// Warp-aggregated atomic increment.
__device__ __forceinline__ uint32_t agg_inc(uint32_t* ctr) {
    const uint32_t m = __activemask();
    const int leader = __ffs(m) - 1;
    uint32_t lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    uint32_t base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(ctr, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & lt);
}

__device__ __forceinline__ StackRef wf_stack(uint32_t* smem, int cap) {
    StackRef s;
    s.lo = reinterpret_cast<float*>(smem) + threadIdx.x;
    s.hi = reinterpret_cast<float*>(smem + cap * blockDim.x) + threadIdx.x;
    s.stride = blockDim.x;
    s.cap = cap;
    return s;
}

__device__ __forceinline__ uint32_t find_scene(const uint32_t* pix_off, uint32_t n, uint32_t gp) {
    uint32_t lo = 0, hi = n;   // pix_off[lo] <= gp < pix_off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (pix_off[mid] <= gp) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t grid_threads() { return gridDim.x * blockDim.x; }
__device__ __forceinline__ uint32_t global_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }

// Work items of a wave are numbered scene-major: scene s owns items
// [nb * pix_off[s], nb * pix_off[s + 1]), sample b of its local pixel lp is
// item nb * pix_off[s] + b * (width * height) + lp. The paths in flight then
// come from a few scenes at a time, whose node records stay in L2, instead of
// the same sample of every scene.
// Within a sample, consecutive items walk the frame in 8x4-pixel tiles
// (bands of 4 rows, blocks of 8 columns; narrower blocks at the right and top
// edges), so that the 32 primary rays a warp generates share a compact
// footprint. `tile_pixel` maps the item's position in that walk to the
// row-major pixel index; it is a bijection on [0, width * height).
constexpr uint32_t kTileW = 8, kTileH = 4;

__device__ __forceinline__ uint32_t tile_pixel(uint32_t q, uint32_t w, uint32_t h) {
    const uint32_t band = q / (w * kTileH);
    const uint32_t hb = min(kTileH, h - band * kTileH);
    const uint32_t idx = q - band * w * kTileH;
    const uint32_t cb = idx / (kTileW * hb);
    const uint32_t wb = min(kTileW, w - cb * kTileW);
    const uint32_t i = idx - cb * kTileW * hb;
    const uint32_t x = cb * kTileW + i % wb, y = band * kTileH + i / wb;
    return y * w + x;
}

struct ItemRef {
    uint32_t b, q, pix;   // sample within the wave, position in the tile walk, row-major pixel
};
__device__ __forceinline__ ItemRef decode_item(uint32_t item, uint32_t nb, const WfScene& sc) {
    const uint32_t local = item - nb * sc.pix_off;
    const uint32_t npix = sc.width * sc.height;
    ItemRef r;
    r.b = local / npix;
    r.q = local - r.b * npix;
    r.pix = tile_pixel(r.q, sc.width, sc.height);
    return r;
}

__device__ __forceinline__ void finish_path(const WfArgs& a, uint32_t slot, uint32_t item, const float4& c) {
    a.out[item] = c;
    a.free_list[agg_inc(&a.ctl->free_count)] = slot;
}

// Wave set-up: sample range, counters, free list; (re)opens the inner loop.
__global__ void k_wf_setup(WfArgs a) {
    WfCtl* c = a.ctl;
    const uint32_t Q = a.Q;
    for (uint32_t i = global_tid(); i < Q; i += grid_threads()) a.free_list[i] = Q - 1 - i;
    if (global_tid() == 0) {
        const uint32_t s0 = c->s_begin + c->wave * c->spw;
        const uint32_t nb = min(c->spw, c->s_end - s0);
        c->s0 = s0;
        c->nb = nb;
        c->items_total = a.P_tot * nb;
        c->items_issued = 0;
        c->ext_count[0] = c->ext_count[1] = 0;
        c->shadow_count = 0;
        c->free_count = Q;
        c->iter = 0;
        if (a.in_graph) cudaGraphSetConditional(a.h_inner, c->error ? 0u : 1u);
    }
}

// Refill free slots with new camera samples, appended to the current queue.
__global__ void k_wf_generate(WfArgs a) {
    const WfCtl* c = a.ctl;
    const uint32_t cur = c->iter & 1u;
    const uint32_t remaining = c->items_total - c->items_issued;
    const uint32_t n_new = min(c->free_count, remaining);
    const uint32_t base = c->ext_count[cur];
    for (uint32_t i = global_tid(); i < n_new; i += grid_threads()) {
        const uint32_t slot = a.free_list[c->free_count - 1 - i];
        const uint32_t item = c->items_issued + i;
        const uint32_t s = find_scene(a.pix_off, a.num_scenes, item / c->nb);
        const WfScene& sc = a.scenes[s];
        const ItemRef ir = decode_item(item, c->nb, sc);
        const uint32_t lp = ir.pix;
        const PathRay r = camera_ray(sc.cam, sc.width, sc.height, lp % sc.width, lp / sc.width, c->s0 + ir.b, a.spp);
        a.o[slot] = make_float4(r.pos.x, r.pos.y, r.pos.z, r.weight);   // w: the ray's weight (specular batches)
        a.d[slot] = make_float4(r.dir.x, r.dir.y, r.dir.z, r.eta);      // w: the ray's eta
        a.thr[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        a.col[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        a.meta[slot] = make_uint4(item, 0u, 0u, s);
        if (a.sp) a.sp[slot] = 0u;
        a.ext_q[cur][base + i] = slot;
    }
}

__global__ void k_wf_generate_commit(WfArgs a) {
    WfCtl* c = a.ctl;
    const uint32_t cur = c->iter & 1u;
    const uint32_t n_new = min(c->free_count, c->items_total - c->items_issued);
    c->free_count -= n_new;
    c->items_issued += n_new;
    c->ext_count[cur] += n_new;
    c->ext_fetch = 0;
    c->shadow_fetch = 0;
    c->ext_chunk = 0;
    c->ext_defer = 0;
}

// Next queue position for a lane that needs work (one atomic per warp).
__device__ __forceinline__ uint32_t fetch_next(uint32_t* cursor) { return agg_inc(cursor); }

// Takes the next chunk of 32 queue entries for the whole warp (one atomic);
// returns false when the n entries are exhausted.
__device__ __forceinline__ bool next_chunk(uint32_t* cursor, uint32_t n, uint32_t& chunk) {
    uint32_t ch = 0;
    if (lane_id() == 0) ch = atomicAdd(cursor, 1u);
    chunk = __shfl_sync(0xffffffffu, ch, 0);
    return chunk < ((n + 31u) >> 5);
}

// True when every valid lane's ray has lane 0's scene and direction octant
// (lane 0 is valid) and the origins lie within the scene's packet span;
// otherwise lane 0 appends the chunk to the deferred list.
__device__ __forceinline__ bool packet_or_defer(const WfArgs& a, uint32_t* defer_count, uint32_t chunk, bool valid,
                                                uint32_t scene, const f3& pos, const f3& dir, uint32_t& scene0,
                                                uint32_t& oct0) {
    const uint32_t oct = dir_octant(dir);
    scene0 = __shfl_sync(0xffffffffu, scene, 0);
    oct0 = __shfl_sync(0xffffffffu, oct, 0);
    if (__all_sync(0xffffffffu, !valid || (scene == scene0 && oct == oct0)) &&
        warp_origin_span(pos, valid) <= a.scenes[scene0].packet_span)
        return true;
    if (lane_id() == 0) a.defer[atomicAdd(defer_count, 1u)] = chunk;
    return false;
}

// Closest hit, first pass: chunks of 32 queued paths of one scene and one
// direction octant (the camera rays of an 8x4 pixel tile, say) are
// traversed as warp packets (traverse_packet); the other chunks are left to
// k_wf_extend. Same results either way.
__global__ void __launch_bounds__(kWfMaxBlock, 4) k_wf_extend_packets(WfArgs a) {
    extern __shared__ uint32_t smem[];
    const StackRef stk = wf_stack(smem, a.cap);
    WfCtl* c = a.ctl;
    const uint32_t cur = c->iter & 1u;
    const uint32_t n = c->ext_count[cur];
    uint32_t chunk;
    while (next_chunk(&c->ext_chunk, n, chunk)) {
        const uint32_t i = chunk * 32u + lane_id();
        const bool valid = i < n;
        uint32_t slot = 0, scene = 0;
        f3 pos = mk3(0.0f), dir = mk3(0.0f);
        if (valid) {
            slot = a.ext_q[cur][i];
            scene = a.meta[slot].w;
            const float4 o = a.o[slot], d = a.d[slot];
            pos = mk3(o.x, o.y, o.z);
            dir = mk3(d.x, d.y, d.z);
        }
        uint32_t scene0, oct0;
        if (!packet_or_defer(a, &c->ext_defer, chunk, valid, scene, pos, dir, scene0, oct0)) continue;
        const WfScene& sc = a.scenes[scene0];
        float best_t = kInfinity, bu = 0.0f, bv = 0.0f;
        const uint32_t best = traverse_packet<false>(sc.recs, sc.nodes, sc.perm, valid, oct0, pos, dir, best_t, bu, bv,
                                                     stk);
        if (valid) a.hit[slot] = make_float4(best_t, bu, bv, __uint_as_float(best));
    }
}

// Closest hit for the queued paths of the deferred chunks: persistent lanes
// fetch them dynamically, so a lane whose ray finished takes the next one at
// once. Positions past the queue's end in the last chunk trace the last
// entry again (the same hit, written twice).
__global__ void __launch_bounds__(kWfMaxBlock, 4) k_wf_extend(WfArgs a) {
    extern __shared__ uint32_t smem[];
    const StackRef stk = wf_stack(smem, a.cap);
    WfCtl* c = a.ctl;
    const uint32_t cur = c->iter & 1u;
    const uint32_t n = c->ext_count[cur];
    const uint32_t m = c->ext_defer * 32u;
    uint32_t visits = 0;
    uint32_t slot = 0xFFFFFFFFu;
    const float4* recs = nullptr;
    const uint32_t* perm = nullptr;
    uint32_t nodes = 0;
    f3 pos = mk3(0.0f), dir = mk3(0.0f), inv = mk3(0.0f);
    float best_t = 0.0f, bu = 0.0f, bv = 0.0f;
    uint32_t best = kNoPrim;
    TravState s;
    trav_init(s);
    for (;;) {
        if (slot == 0xFFFFFFFFu) {
            const uint32_t j = fetch_next(&c->ext_fetch);
            if (j >= m) break;
            slot = a.ext_q[cur][min(a.defer[j >> 5] * 32u + (j & 31u), n - 1u)];
            const WfScene& sc = a.scenes[a.meta[slot].w];
            recs = sc.recs; perm = sc.perm; nodes = sc.nodes;
            const float4 o = a.o[slot], d = a.d[slot];
            pos = mk3(o.x, o.y, o.z);
            dir = mk3(d.x, d.y, d.z);
            inv = box_inv(dir);
            best_t = kInfinity; bu = bv = 0.0f; best = kNoPrim;
            trav_init(s);
        }
        Sector s0;
        float4 q5;
        float nlo, nhi;
        if (trav_next(s, recs, nodes, pos, dir, inv, best_t, stk, s0, nlo, nhi, visits)) {
            node_triangles<false>(recs, s.k, s0, perm, pos, dir, best_t, bu, bv, best, q5);
            trav_descend(s, recs, q5, pos, dir, inv, best_t, nodes, stk, nlo, nhi);
        } else {
            a.hit[slot] = make_float4(best_t, bu, bv, __uint_as_float(best));
            slot = 0xFFFFFFFFu;
        }
    }
}

// The per-slot ray stack of specular batches.
__device__ __forceinline__ void wf_push(const WfArgs& a, uint32_t slot, uint32_t& sp, const PathRay& r, WfCtl* c) {
    if (sp >= kWfStack) {
        atomicOr(&c->error, kWfErrStack);
        return;
    }
    const size_t b = (size_t)sp * 3 * a.Q + slot;
    a.stk[b] = make_float4(r.pos.x, r.pos.y, r.pos.z, r.weight);
    a.stk[b + a.Q] = make_float4(r.dir.x, r.dir.y, r.dir.z, r.eta);
    a.stk[b + 2 * (size_t)a.Q] = make_float4(r.thr.x, r.thr.y, r.thr.z, r.pdf);
    ++sp;
}

// Pops the slot's next pending ray into its current-ray state (the plain
// integrator's `while (depth <= maxd && sp > 0)` loop); false when the
// sample is done.
__device__ __forceinline__ bool wf_pop_next(const WfArgs& a, uint32_t slot, uint32_t depth, uint32_t sp) {
    if (!(depth <= a.max_depth && sp > 0)) return false;
    --sp;
    const size_t b = (size_t)sp * 3 * a.Q + slot;
    a.o[slot] = a.stk[b];
    a.d[slot] = a.stk[b + a.Q];
    a.thr[slot] = a.stk[b + 2 * (size_t)a.Q];
    a.sp[slot] = sp;
    a.meta[slot].z += 1u;   // the sample's next ray index
    return true;
}

// Shading: misses finish (specular batches: the sample's next pending ray
// goes on); hits get their light samples (shadow rays queued) and, in path
// mode, their bounce; specular batches push reflection, refraction and
// bounce rays on the slot's stack in the plain integrator's order.
// kMis: the mode is AUR_MODE_PATH_MIS; kSpec: the batch has specular shaders.
template <bool kMis, bool kSpec>
__global__ void __launch_bounds__(kWfMaxBlock, 4) k_wf_shade(WfArgs a) {
    WfCtl* c = a.ctl;
    const uint32_t cur = c->iter & 1u;
    const uint32_t n = c->ext_count[cur];
    for (uint32_t i = global_tid(); i < n; i += grid_threads()) {
        const uint32_t slot = a.ext_q[cur][i];
        const uint4 m = a.meta[slot];
        const float4 h = a.hit[slot];
        const uint32_t tri = __float_as_uint(h.w);
        if (tri == kNoPrim) {
            if (kSpec && wf_pop_next(a, slot, m.y, a.sp[slot])) {
                a.ext_q[cur ^ 1u][agg_inc(&c->ext_count[cur ^ 1u])] = slot;
                continue;
            }
            finish_path(a, slot, m.x, a.col[slot]);
            continue;
        }
        const WfScene& sc = a.scenes[m.w];
        const ItemRef ir = decode_item(m.x, c->nb, sc);
        const uint32_t pix = ir.pix, sample = c->s0 + ir.b, rix = m.z;
        const float4 o4 = a.o[slot], d4 = a.d[slot];
        const f3 pos = mk3(o4.x, o4.y, o4.z), dir = mk3(d4.x, d4.y, d4.z);
        const f3 position = pos + (dir * h.x);
        const f3 wo = -dir;
        const uint32_t sid = sc.sids[tri];
        const aur_shader* sh = sc.shaders + (sid > 0 ? sid - 1 : 0);
        constexpr bool mis = kMis;
        SceneView sv;
        sv.normals = sc.normals;
        sv.texcoords = sc.texcoords;
        sv.texels = sc.texels;
        sv.tex_info = sc.tex_info;
        sv.sids = sc.sids;
        sv.shaders = sc.shaders;
        sv.verts = sc.verts;
        sv.mis_tri = sc.mis_tri;
        sv.mis_cdf = sc.mis_cdf;
        sv.mis_pa = sc.mis_pa;
        sv.mis_count = sc.mis_count;
        const Bsdf bs = get_bsdf(sv, sh, tri, h.y, h.z);
        const f3 f = bsdf_f(bs);
        const uint32_t depth = m.y + 1u;
        const bool specular = kSpec && (sh->reflectivity > 0.0f || sh->translucence > 0.0f);
        // does a diffuse bounce follow this hit (the emitter sample's weight)?
        const bool bounce = kSpec ? !specular && m.y + 1u <= a.max_depth : depth <= a.max_depth;
        a.fsh[slot] = make_float4(f.x, f.y, f.z, 0.0f);
        const f3 em = mis ? from(sh->emission_color) * emission_weight(sv, tri, dir, h.x, a.thr[slot].w)
                          : from(sh->emission_color);
        a.emi[slot] = make_float4(em.x, em.y, em.z, 0.0f);
        a.vis[slot] = 0u;
        float4* cj = a.cj + (size_t)slot * a.M;
        uint32_t q = 0;
        // queues one shadow ray of light-sample slot q
        auto queue = [&](const ShadowSample& ss, uint32_t qq) {
            cj[qq] = make_float4(ss.c.x, ss.c.y, ss.c.z, ss.cand ? 1.0f : 0.0f);
            if (ss.cand) {
                const uint32_t e = agg_inc(&c->shadow_count);
                a.sh_o[e] = make_float4(ss.o.x, ss.o.y, ss.o.z, ss.tmax);
                a.sh_d[e] = make_float4(ss.d.x, ss.d.y, ss.d.z, __uint_as_float((slot << 5) | qq));
            }
        };
        for (uint32_t li = 0; li < sc.num_lights; ++li) {
            const aur_light& L = sc.lights[li];
            if (mis && L.type == AUR_LIGHT_AREA) {
                // both strategies of every sample (direct_light_mis), two slots each
                const AreaLightMis al = area_light_setup(L, f);
                for (uint32_t j = 0; j < (uint32_t)L.samples; ++j, q += 2) {
                    if (q + 1 >= a.M) {   // lights given more samples since the batch was created
                        atomicOr(&c->error, kWfErrLightSlots);
                        break;
                    }
                    ShadowSample ss;
                    ss.cand = false;
                    ss.c = mk3(0.0f);
                    if (al.active)
                        ss = area_light_sample(al, li, j, bs, f, position, wo, a.seed, sc.scene_id, pix, sample, rix);
                    queue(ss, q);
                    if (al.active)
                        ss = area_bsdf_sample(al, li, j, bs, f, position, wo, a.seed, sc.scene_id, pix, sample, rix);
                    queue(ss, q + 1);
                }
                continue;
            }
            const uint32_t ns = L.type == AUR_LIGHT_AREA ? (uint32_t)L.samples : 1u;
            for (uint32_t j = 0; j < ns; ++j, ++q) {
                if (q >= a.M) {   // lights given more samples since the batch was created
                    atomicOr(&c->error, kWfErrLightSlots);
                    break;
                }
                f3 wdir;
                float wt, pdf;
                const uint32_t lslot = L.type == AUR_LIGHT_AREA ? light_slot(li, j) : 0u;
                const f3 Lr = sample_light(L, position, a.seed, sc.scene_id, pix, sample, rix, lslot, wdir, wt, pdf);
                f3 wpos = position;
                if (L.type == AUR_LIGHT_AREA) {
                    wpos.x += kEpsilon * wdir.x;
                    wpos.y += kEpsilon * wdir.y;
                    wpos.z += kEpsilon * wdir.z;
                    wt += kEpsilon;
                }
                const bool cand = pdf > 0.0f && !zero(Lr) && !zero(f);
                const f3 cc = f * Lr * fmaxf(0.0f, dot(wdir, bs.N));
                cj[q] = make_float4(cc.x, cc.y, cc.z, cand ? 1.0f : 0.0f);
                if (cand) {
                    const uint32_t e = agg_inc(&c->shadow_count);
                    a.sh_o[e] = make_float4(wpos.x, wpos.y, wpos.z, wt);
                    a.sh_d[e] = make_float4(wdir.x, wdir.y, wdir.z, __uint_as_float((slot << 5) | q));
                }
            }
        }
        if (mis) {   // the emitter sample (direct_light_mis), last slot
            if (q >= a.M) {
                atomicOr(&c->error, kWfErrLightSlots);
            } else {
                queue(emitter_shadow_sample(sv, bs, f, position, wo, bounce, a.seed, sc.scene_id, pix, sample, rix), q);
            }
        }
        if (kSpec) {
            // integrate(): the specular rays and the diffuse bounce onto the stack
            const float4 t4 = a.thr[slot];
            PathRay ray;
            ray.pos = pos;
            ray.dir = dir;
            ray.thr = mk3(t4.x, t4.y, t4.z);
            ray.weight = o4.w;
            ray.eta = d4.w;
            ray.pdf = t4.w;
            int dep = (int)m.y;
            uint32_t sp = a.sp[slot];
            const Continuation k = continue_ray<kMis>(sh, bs, ray, position, wo, kMis || a.mode == AUR_MODE_PATH, dep,
                                                      (int)a.max_depth, a.seed, sc.scene_id, pix, sample, rix);
            for (int q = 0; q < k.n; ++q) wf_push(a, slot, sp, k.ray[q], c);
            const f3 thr = ray.thr;
            a.thr[slot] = make_float4(thr.x, thr.y, thr.z, 0.0f);   // the colour update's throughput
            a.sp[slot] = sp;
            a.meta[slot].y = (uint32_t)dep;
            continue;
        }
        // bounce (BSDF::samplef, bsdf.cuh:222-236)
        float cont = 0.0f, bpdf = 0.0f;
        f3 wi = mk3(0.0f), nt = mk3(0.0f);
        if (mis && depth <= a.max_depth) {
            const float4 t4 = a.thr[slot];
            if (mis_bounce(bs, wo, mk3(t4.x, t4.y, t4.z), a.seed, sc.scene_id, pix, sample, rix, wi, nt, bpdf))
                cont = 1.0f;
        } else if (a.mode == AUR_MODE_PATH && depth <= a.max_depth) {
            float u1, u2;
            draw2(a.seed, sc.scene_id, pix, sample, rix, 0u, u1, u2);
            const f3 lwo = world_to_local(wo, bs.N, bs.S, bs.T);
            f3 lwi = sample_hemisphere_cosine(u1, u2);
            if (lwo.z < 0.0f) lwi.z *= -1.0f;
            bpdf = (lwo.z * lwi.z > 0.0f) ? fabsf(lwi.z) * kInvPi : 0.0f;
            wi = local_to_world(lwi, bs.N, bs.S, bs.T);
            if (bpdf > 0.0f && !zero(f)) {
                const float4 t4 = a.thr[slot];
                nt = mk3(t4.x, t4.y, t4.z) * (f * (fabsf(dot(wi, bs.N)) / bpdf));
                cont = 1.0f;
            }
        }
        a.ndir[slot] = make_float4(wi.x, wi.y, wi.z, cont);
        a.nthr[slot] = make_float4(nt.x, nt.y, nt.z, bpdf);
        a.meta[slot].y = depth;
    }
}

// Any hit for every queued shadow ray; unoccluded rays set their bit.
// Persistent lanes with dynamic fetch, as in k_wf_extend. (Warp packets, as
// in the extend stage, made this stage slower: the rays of a chunk start at
// different surface points and share few nodes.)
__global__ void __launch_bounds__(kWfMaxBlock, 4) k_wf_shadow(WfArgs a) {
    extern __shared__ uint32_t smem[];
    const StackRef stk = wf_stack(smem, a.cap);
    WfCtl* c = a.ctl;
    const uint32_t n = c->shadow_count;
    uint32_t visits = 0;
    uint32_t id = 0xFFFFFFFFu;
    const float4* recs = nullptr;
    const uint32_t* perm = nullptr;
    uint32_t nodes = 0;
    f3 pos = mk3(0.0f), dir = mk3(0.0f), inv = mk3(0.0f);
    float tmax = 0.0f, bu = 0.0f, bv = 0.0f;
    uint32_t best = kNoPrim;
    TravState s;
    trav_init(s);
    for (;;) {
        if (id == 0xFFFFFFFFu) {
            const uint32_t i = fetch_next(&c->shadow_fetch);
            if (i >= n) break;
            const float4 o = a.sh_o[i], d = a.sh_d[i];
            id = __float_as_uint(d.w);
            const WfScene& sc = a.scenes[a.meta[id >> 5].w];
            recs = sc.recs; perm = sc.perm; nodes = sc.nodes;
            pos = mk3(o.x, o.y, o.z);
            dir = mk3(d.x, d.y, d.z);
            inv = box_inv(dir);
            tmax = o.w;
            best = kNoPrim;
            trav_init(s);
        }
        Sector s0;
        float4 q5;
        float nlo, nhi;
        bool done;
        if (trav_next(s, recs, nodes, pos, dir, inv, tmax, stk, s0, nlo, nhi, visits)) {
            done = node_triangles<true>(recs, s.k, s0, perm, pos, dir, tmax, bu, bv, best, q5);
            if (!done) trav_descend(s, recs, q5, pos, dir, inv, tmax, nodes, stk, nlo, nhi);
        } else {
            done = true;
        }
        if (done) {
            if (best == kNoPrim) atomicOr(&a.vis[id >> 5], 1u << (id & 31u));
            id = 0xFFFFFFFFu;
        }
    }
}

// Li in the reference's order (radiance.cuh:13-80, monteCarloRaytracer.cu:42-52),
// colour update, then continue or finish. kMis and kSpec as in k_wf_shade.
template <bool kMis, bool kSpec>
__global__ void k_wf_combine(WfArgs a) {
    WfCtl* c = a.ctl;
    const uint32_t cur = c->iter & 1u, nxt = cur ^ 1u;
    const uint32_t n = c->ext_count[cur];
    for (uint32_t i = global_tid(); i < n; i += grid_threads()) {
        const uint32_t slot = a.ext_q[cur][i];
        const float4 h = a.hit[slot];
        if (__float_as_uint(h.w) == kNoPrim) continue;   // finished in shade
        const uint4 m = a.meta[slot];
        const WfScene& sc = a.scenes[m.w];
        const float4 f4 = a.fsh[slot], e4 = a.emi[slot];
        const f3 f = mk3(f4.x, f4.y, f4.z);
        const uint32_t vis = a.vis[slot];
        const float4* cj = a.cj + (size_t)slot * a.M;
        constexpr bool mis = kMis;
        f3 Li = mk3(e4.x, e4.y, e4.z);
        uint32_t q = 0;
        for (uint32_t li = 0; li < sc.num_lights; ++li) {
            const aur_light& L = sc.lights[li];
            if (L.type == AUR_LIGHT_AMBIENT) Li = Li + f * ((from(L.color) * L.intensity) * L.ambient);
            if (mis && L.type == AUR_LIGHT_AREA) {
                // direct_light_mis: per sample, the light then the BSDF strategy
                f3 acc = mk3(0.0f);
                for (int32_t j = 0; j < L.samples; ++j) {
                    f3 Ls = mk3(0.0f);
                    for (int h2 = 0; h2 < 2; ++h2, ++q) {
                        const float4 v = q < a.M ? cj[q] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        if (v.w != 0.0f && ((vis >> q) & 1u)) Ls = Ls + mk3(v.x, v.y, v.z);
                    }
                    acc = acc + Ls;
                }
                const float ns = (float)L.samples;
                Li = Li + mk3(acc.x / ns, acc.y / ns, acc.z / ns);
            } else if (L.type != AUR_LIGHT_AREA) {
                const float4 v = q < a.M ? cj[q] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (v.w != 0.0f && ((vis >> q) & 1u)) Li = Li + mk3(v.x, v.y, v.z);
                ++q;
            } else {
                f3 acc = mk3(0.0f);
                for (int32_t j = 0; j < L.samples; ++j, ++q) {
                    f3 Ls = mk3(0.0f);
                    const float4 v = q < a.M ? cj[q] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (v.w != 0.0f && ((vis >> q) & 1u)) Ls = Ls + mk3(v.x, v.y, v.z);
                    acc = acc + Ls;
                }
                const float ns = (float)L.samples;
                Li = Li + mk3(acc.x / ns, acc.y / ns, acc.z / ns);
            }
        }
        if (mis) {   // the emitter sample: added whether or not it contributes
            const float4 v = q < a.M ? cj[q] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            Li = Li + ((v.w != 0.0f && ((vis >> q) & 1u)) ? mk3(v.x, v.y, v.z) : mk3(0.0f));
        }
        const float4 t4 = a.thr[slot];
        float4 col = a.col[slot];
        const f3 cc = mk3(col.x, col.y, col.z) + Li * mk3(t4.x, t4.y, t4.z);
        col = make_float4(cc.x, cc.y, cc.z, 1.0f);
        if (kSpec) {
            a.col[slot] = col;
            if (wf_pop_next(a, slot, a.meta[slot].y, a.sp[slot]))
                a.ext_q[nxt][agg_inc(&c->ext_count[nxt])] = slot;
            else
                finish_path(a, slot, m.x, col);
            continue;
        }
        const float4 nd = a.ndir[slot];
        if (nd.w != 0.0f) {
            const float4 o4 = a.o[slot], d4 = a.d[slot];
            const f3 position = mk3(o4.x, o4.y, o4.z) + (mk3(d4.x, d4.y, d4.z) * h.x);
            a.o[slot] = make_float4(position.x, position.y, position.z, 0.0f);
            a.d[slot] = make_float4(nd.x, nd.y, nd.z, 0.0f);
            a.thr[slot] = a.nthr[slot];
            a.col[slot] = col;
            a.meta[slot].z = m.z + 1u;
            a.ext_q[nxt][agg_inc(&c->ext_count[nxt])] = slot;
        } else {
            finish_path(a, slot, m.x, col);
        }
    }
}

// End of an iteration: clear the consumed queue, decide whether to loop.
__global__ void k_wf_end(WfArgs a) {
    WfCtl* c = a.ctl;
    const uint32_t cur = c->iter & 1u, nxt = cur ^ 1u;
    c->total_ext += c->ext_count[cur];
    c->total_shadow += c->shadow_count;
    c->ext_count[cur] = 0;
    c->shadow_count = 0;
    c->iter += 1;
    c->total_iters += 1;
    bool more = c->items_issued < c->items_total || c->ext_count[nxt] > 0;
    if (c->iter > c->iter_limit) { c->error |= 1u; more = false; }
    if (c->error) more = false;
    if (a.in_graph) cudaGraphSetConditional(a.h_inner, more ? 1u : 0u);
}

// drawPixels for the wave's samples, in sample order.
__global__ void k_wf_accumulate(WfArgs a) {
    const WfCtl* c = a.ctl;
    const float weight = 1.0f / (float)a.spp;
    const uint32_t nb = c->nb;
    for (uint32_t gp = global_tid(); gp < a.P_tot; gp += grid_threads()) {
        const uint32_t s = find_scene(a.pix_off, a.num_scenes, gp);
        const uint32_t q = gp - a.pix_off[s];   // position in the tile walk
        const uint32_t npix = a.pix_off[s + 1] - a.pix_off[s];
        const float4* out = a.out + (size_t)nb * a.pix_off[s] + q;
        float4* acc = a.accum[s] + tile_pixel(q, a.scenes[s].width, a.scenes[s].height);
        float4 v = *acc;
        for (uint32_t b = 0; b < nb; ++b) {
            const float4 cv = out[(size_t)b * npix];
            if (cv.w != 0.0f) {
                v.x += cv.x * weight;
                v.y += cv.y * weight;
                v.z += cv.z * weight;
                v.w += weight;
            }
        }
        *acc = v;
    }
}

__global__ void k_wf_next_wave(WfArgs a) {
    WfCtl* c = a.ctl;
    c->wave += 1;
    if (a.in_graph) cudaGraphSetConditional(a.h_outer, (c->wave < c->num_waves && !c->error) ? 1u : 0u);
}

inline uint32_t cdiv(uint64_t x, uint64_t y) { return (uint32_t)((x + y - 1) / y); }

}  // namespace
}  // namespace aur

using namespace aur;

struct aur_batch {
    int device = 0;
    uint32_t num_scenes = 0;
    aur_render_params params{};
    aur_wavefront_tuning tuning{};
    WfArgs args{};
    void* mem = nullptr;             // one allocation for state, queues, tables
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap_stream = nullptr;
    uint32_t grid = 0, block = 0;
    size_t smem = 0;
    std::vector<float4*> accum_host;
    std::vector<const aur_scene*> scene_ptrs;   // AUR_MODE_PATH_MIS: tables to keep current
    std::vector<WfScene> table_host;            // host copy of the device scene table
};

namespace {

// The shade and combine instantiations for the batch's mode and materials.
void launch_shade(const WfArgs& a, uint32_t g, uint32_t bs, cudaStream_t s) {
    const bool mis = a.mode == AUR_MODE_PATH_MIS, spec = a.stk != nullptr;
    if (mis && spec) k_wf_shade<true, true><<<g, bs, 0, s>>>(a);
    else if (mis) k_wf_shade<true, false><<<g, bs, 0, s>>>(a);
    else if (spec) k_wf_shade<false, true><<<g, bs, 0, s>>>(a);
    else k_wf_shade<false, false><<<g, bs, 0, s>>>(a);
}
void launch_combine(const WfArgs& a, uint32_t g, uint32_t bs, cudaStream_t s) {
    const bool mis = a.mode == AUR_MODE_PATH_MIS, spec = a.stk != nullptr;
    if (mis && spec) k_wf_combine<true, true><<<g, bs, 0, s>>>(a);
    else if (mis) k_wf_combine<true, false><<<g, bs, 0, s>>>(a);
    else if (spec) k_wf_combine<false, true><<<g, bs, 0, s>>>(a);
    else k_wf_combine<false, false><<<g, bs, 0, s>>>(a);
}

aur_status make_graph(aur_batch* bt) {
    WfArgs& a = bt->args;
    a.in_graph = 1;
    AUR_CUDA(cudaGraphCreate(&bt->graph, 0));
    AUR_CUDA(cudaGraphConditionalHandleCreate(&a.h_outer, bt->graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams outer = {};
    outer.type = cudaGraphNodeTypeConditional;
    outer.conditional.handle = a.h_outer;
    outer.conditional.type = cudaGraphCondTypeWhile;
    outer.conditional.size = 1;
    cudaGraphNode_t outer_node;
    AUR_CUDA(cudaGraphAddNode(&outer_node, bt->graph, nullptr, nullptr, 0, &outer));
    cudaGraph_t wave_body = outer.conditional.phGraph_out[0];
    // the inner handle belongs to the wave body; create it before capturing
    AUR_CUDA(cudaGraphConditionalHandleCreate(&a.h_inner, wave_body, 1, cudaGraphCondAssignDefault));
    const uint32_t g = bt->grid, bs = bt->block;
    cudaStream_t s = bt->cap_stream;
    // wave body part 1: set-up
    AUR_CUDA(cudaStreamBeginCaptureToGraph(s, wave_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    k_wf_setup<<<g, bs, 0, s>>>(a);
    cudaGraph_t tmp;
    AUR_CUDA(cudaStreamEndCapture(s, &tmp));
    size_t nn = 0;
    AUR_CUDA(cudaGraphGetNodes(wave_body, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    AUR_CUDA(cudaGraphGetNodes(wave_body, nodes.data(), &nn));
    AUR_CHECK(nn == 1, AUR_ERR_CUDA, "wavefront graph: unexpected set-up node count %zu", nn);
    cudaGraphNode_t setup_node = nodes[0];
    // inner loop node
    cudaGraphNodeParams inner = {};
    inner.type = cudaGraphNodeTypeConditional;
    inner.conditional.handle = a.h_inner;
    inner.conditional.type = cudaGraphCondTypeWhile;
    inner.conditional.size = 1;
    cudaGraphNode_t inner_node;
    AUR_CUDA(cudaGraphAddNode(&inner_node, wave_body, &setup_node, nullptr, 1, &inner));
    cudaGraph_t iter_body = inner.conditional.phGraph_out[0];
    AUR_CUDA(cudaStreamBeginCaptureToGraph(s, iter_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    k_wf_generate<<<g, bs, 0, s>>>(a);
    k_wf_generate_commit<<<1, 1, 0, s>>>(a);
    k_wf_extend_packets<<<g, bs, bt->smem, s>>>(a);
    k_wf_extend<<<g, bs, bt->smem, s>>>(a);
    launch_shade(a, g, bs, s);
    k_wf_shadow<<<g, bs, bt->smem, s>>>(a);
    launch_combine(a, g, bs, s);
    k_wf_end<<<1, 1, 0, s>>>(a);
    AUR_CUDA(cudaStreamEndCapture(s, &tmp));
    // wave body part 2: accumulate after the inner loop
    AUR_CUDA(cudaStreamBeginCaptureToGraph(s, wave_body, &inner_node, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    k_wf_accumulate<<<g, bs, 0, s>>>(a);
    k_wf_next_wave<<<1, 1, 0, s>>>(a);
    AUR_CUDA(cudaStreamEndCapture(s, &tmp));
    AUR_CUDA(cudaGraphInstantiate(&bt->exec, bt->graph, 0));
    a.in_graph = 0;   // the host-launched (profiling) form must not touch the conditionals
    return AUR_OK;
}

// AUR_MODE_PATH_MIS: a scene whose shaders changed since the last render
// dropped its light-selection table; rebuild it and point the device scene
// table at the new one, so that the frames keep equalling aur_render's.
aur_status refresh_mis_tables(aur_ctx* ctx, aur_batch* bt) {
    if (bt->params.mode != AUR_MODE_PATH_MIS) return AUR_OK;
    for (uint32_t i = 0; i < bt->num_scenes; ++i) {
        const aur_scene* sc = bt->scene_ptrs[i];
        const aur_status st = build_mis_table(ctx, sc);
        if (st != AUR_OK) return st;
        WfScene& w = bt->table_host[i];
        if (w.mis_tri == sc->mis_tri && w.mis_cdf == sc->mis_cdf && w.mis_pa == sc->mis_pa &&
            w.mis_count == sc->mis_count)
            continue;
        w.mis_tri = sc->mis_tri;
        w.mis_cdf = sc->mis_cdf;
        w.mis_pa = sc->mis_pa;
        w.mis_count = sc->mis_count;
        AUR_CUDA(cudaMemcpyAsync((void*)(bt->args.scenes + i), &w, sizeof(WfScene), cudaMemcpyHostToDevice,
                                 ctx->stream));
        AUR_CUDA(cudaStreamSynchronize(ctx->stream));   // w is pageable host memory
    }
    return AUR_OK;
}

void batch_free(aur_batch* bt) {
    if (!bt) return;
    cudaSetDevice(bt->device);
    if (bt->exec) cudaGraphExecDestroy(bt->exec);
    if (bt->graph) cudaGraphDestroy(bt->graph);
    if (bt->cap_stream) cudaStreamDestroy(bt->cap_stream);
    cudaFree(bt->mem);
    delete bt;
}

}  // namespace

extern "C" {

aur_status aur_batch_create(aur_ctx* ctx, const aur_scene* const* scenes, const aur_camera* cameras,
                            const aur_render_params* params, uint32_t num_scenes, const aur_wavefront_tuning* tuning,
                            aur_batch** out) {
    AUR_RANGE("aur_batch_create");
    clear_error();
    AUR_CHECK(ctx && scenes && cameras && params && out && num_scenes > 0, AUR_ERR_INVALID,
              "aur_batch_create: null argument or no scenes");
    const aur_render_params& p0 = params[0];
    aur_status st = check_params(&p0);
    if (st != AUR_OK) return st;
    const bool mis = p0.mode == AUR_MODE_PATH_MIS;
    uint64_t P_tot = 0;
    uint32_t M = 1, cap = 2;
    bool spec = false;
    std::vector<WfScene> table(num_scenes);
    std::vector<uint32_t> pix_off(num_scenes + 1);
    for (uint32_t i = 0; i < num_scenes; ++i) {
        const aur_scene* sc = scenes[i];
        const aur_render_params& p = params[i];
        AUR_CHECK(sc, AUR_ERR_INVALID, "aur_batch_create: scene %u is null", i);
        st = check_params(&p);
        if (st == AUR_OK) st = check_scene_textures(sc);
        if (st != AUR_OK) return st;
        AUR_CHECK(p.spp == p0.spp && p.max_depth == p0.max_depth && p.mode == p0.mode && p.seed == p0.seed &&
                      p.sample_begin == p0.sample_begin && p.sample_end == p0.sample_end,
                  AUR_ERR_INVALID, "aur_batch_create: scene %u differs in spp/depth/mode/seed/sample range", i);
        AUR_CHECK(sc->nmh->device == ctx->device, AUR_ERR_INVALID, "aur_batch_create: scene %u on another device", i);
        // specular materials need the per-sample ray stack of the plain path
        spec = spec || sc->has_specular;
        std::vector<aur_light> lt(sc->num_lights);
        if (sc->num_lights)
            AUR_CUDA(cudaMemcpy(lt.data(), sc->lights, sizeof(aur_light) * sc->num_lights, cudaMemcpyDeviceToHost));
        // light-sample slots per hit: one per sample (MIS: two per area-light
        // sample, plus the emitter sample)
        uint32_t m = mis ? 1u : 0u;
        for (const aur_light& l : lt) m += l.type == AUR_LIGHT_AREA ? (mis ? 2u : 1u) * (uint32_t)l.samples : 1u;
        if (mis) {
            AUR_CHECK(sc->num_lights < 32767, AUR_ERR_INVALID,
                      "aur_batch_create: AUR_MODE_PATH_MIS takes at most 32766 lights (scene %u has %u)", i,
                      sc->num_lights);
            AUR_CUDA(cudaSetDevice(ctx->device));
            st = build_mis_table(ctx, sc);
            if (st != AUR_OK) return st;
        }
        AUR_CHECK(m <= (uint32_t)kMaxLightSlots, AUR_ERR_UNSUPPORTED,
                  "aur_batch_create: scene %u needs %u light samples per hit (limit %d)", i, m, kMaxLightSlots);
        M = std::max(M, m);
        cap = std::max(cap, sc->nmh->levels + 1);
        WfScene& w = table[i];
        w.recs = sc->nmh->node_recs;
        w.perm = sc->nmh->perm;
        w.normals = sc->normals;
        w.sids = sc->shader_ids;
        w.shaders = sc->shaders;
        w.lights = sc->lights;
        w.texcoords = sc->texcoords;
        w.texels = sc->texels;
        w.tex_info = sc->tex_info;
        w.verts = sc->nmh->verts;
        w.mis_tri = sc->mis_tri;
        w.mis_cdf = sc->mis_cdf;
        w.mis_pa = sc->mis_pa;
        w.mis_count = sc->mis_count;
        w.nodes = sc->nmh->nodes;
        w.packet_span = sc->nmh->extent * (1.0f / 64.0f);
        w.num_lights = sc->num_lights;
        w.width = p.width;
        w.height = p.height;
        w.pix_off = (uint32_t)P_tot;
        w.scene_id = p.scene_id;
        w.cam = cameras[i];
        pix_off[i] = (uint32_t)P_tot;
        P_tot += (uint64_t)p.width * p.height;
        AUR_CHECK(P_tot < (1ull << 31), AUR_ERR_INVALID, "aur_batch_create: too many pixels in the batch");
    }
    pix_off[num_scenes] = (uint32_t)P_tot;
    const uint32_t s_end = p0.sample_end ? p0.sample_end : p0.spp;
    const uint32_t nsamp = s_end - p0.sample_begin;
    AUR_CHECK(nsamp > 0, AUR_ERR_INVALID, "aur_batch_create: empty sample range");

    aur_wavefront_tuning tn{};
    if (tuning) tn = *tuning;
    if (tn.paths_in_flight == 0) tn.paths_in_flight = 1u << 21;
    if (tn.block_size == 0) tn.block_size = 128;
    if (tn.blocks_per_sm == 0) tn.blocks_per_sm = 6;
    if (tn.samples_per_wave == 0) {
        // cap the wave's sample buffer at about 4 GiB (16 B per sample)
        tn.samples_per_wave = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(nsamp, (1ull << 28) / P_tot));
    }
    tn.samples_per_wave = std::min(tn.samples_per_wave, nsamp);
    AUR_CHECK(tn.block_size % 32 == 0 && tn.block_size >= 32 && tn.block_size <= (uint32_t)kWfMaxBlock, AUR_ERR_INVALID,
              "aur_batch_create: block_size must be a multiple of 32 in [32, %d]", kWfMaxBlock);
    AUR_CHECK(tn.paths_in_flight >= 1024 && tn.paths_in_flight <= (1u << 26), AUR_ERR_INVALID,
              "aur_batch_create: paths_in_flight must be in [1024, 2^26]");
    AUR_CHECK(tn.blocks_per_sm >= 1 && tn.blocks_per_sm <= 32, AUR_ERR_INVALID,
              "aur_batch_create: blocks_per_sm must be in [1, 32]");
    AUR_CUDA(cudaSetDevice(ctx->device));

    aur_batch* bt = new aur_batch();
    bt->device = ctx->device;
    bt->num_scenes = num_scenes;
    bt->params = p0;
    bt->tuning = tn;
    bt->block = tn.block_size;
    bt->grid = (uint32_t)ctx->sm_count * tn.blocks_per_sm;
    bt->smem = (size_t)2 * cap * tn.block_size * sizeof(uint32_t);
    bt->accum_host.assign(num_scenes, nullptr);
    bt->scene_ptrs.assign(scenes, scenes + num_scenes);
    bt->table_host = table;
    const uint64_t Q = tn.paths_in_flight;
    const uint64_t out_items = P_tot * tn.samples_per_wave;
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
    const size_t o_ctl = take(sizeof(WfCtl)), o_tab = take(sizeof(WfScene) * num_scenes);
    const size_t o_pix = take(4 * (num_scenes + 1)), o_acc = take(sizeof(float4*) * num_scenes);
    const size_t o_o = take(16 * Q), o_d = take(16 * Q), o_thr = take(16 * Q), o_col = take(16 * Q);
    const size_t o_hit = take(16 * Q), o_meta = take(16 * Q), o_ndir = take(16 * Q), o_nthr = take(16 * Q);
    const size_t o_fsh = take(16 * Q), o_emi = take(16 * Q), o_cj = take(16 * Q * M), o_vis = take(4 * Q);
    const size_t o_q0 = take(4 * Q), o_q1 = take(4 * Q), o_free = take(4 * Q);
    const size_t o_sho = take(16 * Q * M), o_shd = take(16 * Q * M), o_out = take(16 * out_items);
    const size_t o_def = take(4 * ((Q + 31) / 32));
    const size_t o_stk = spec ? take(16 * 3 * (size_t)kWfStack * Q) : 0, o_sp = spec ? take(4 * Q) : 0;
    if (::aur::dev_malloc(&bt->mem, off) != cudaSuccess) {
        cudaGetLastError();
        batch_free(bt);
        return fail(AUR_ERR_OOM, "aur_batch_create: out of device memory (%zu bytes)", off);
    }
    char* base = (char*)bt->mem;
    WfArgs& a = bt->args;
    a.ctl = (WfCtl*)(base + o_ctl);
    a.scenes = (const WfScene*)(base + o_tab);
    a.pix_off = (const uint32_t*)(base + o_pix);
    a.accum = (float4* const*)(base + o_acc);
    a.num_scenes = num_scenes;
    a.P_tot = (uint32_t)P_tot;
    a.Q = (uint32_t)Q;
    a.M = M;
    a.spp = p0.spp;
    a.max_depth = p0.max_depth;
    a.mode = p0.mode;
    a.seed = p0.seed;
    a.cap = (int)cap;
    a.o = (float4*)(base + o_o); a.d = (float4*)(base + o_d); a.thr = (float4*)(base + o_thr);
    a.col = (float4*)(base + o_col); a.hit = (float4*)(base + o_hit); a.meta = (uint4*)(base + o_meta);
    a.ndir = (float4*)(base + o_ndir); a.nthr = (float4*)(base + o_nthr); a.fsh = (float4*)(base + o_fsh);
    a.emi = (float4*)(base + o_emi); a.cj = (float4*)(base + o_cj); a.vis = (uint32_t*)(base + o_vis);
    a.ext_q[0] = (uint32_t*)(base + o_q0); a.ext_q[1] = (uint32_t*)(base + o_q1);
    a.free_list = (uint32_t*)(base + o_free);
    a.sh_o = (float4*)(base + o_sho); a.sh_d = (float4*)(base + o_shd); a.out = (float4*)(base + o_out);
    a.defer = (uint32_t*)(base + o_def);
    a.stk = spec ? (float4*)(base + o_stk) : nullptr;
    a.sp = spec ? (uint32_t*)(base + o_sp) : nullptr;
    cudaMemcpy(base + o_tab, table.data(), sizeof(WfScene) * num_scenes, cudaMemcpyHostToDevice);
    cudaMemcpy(base + o_pix, pix_off.data(), 4 * (num_scenes + 1), cudaMemcpyHostToDevice);
    WfCtl ctl{};
    ctl.s_begin = p0.sample_begin;
    ctl.s_end = s_end;
    ctl.spw = tn.samples_per_wave;
    ctl.num_waves = cdiv(nsamp, tn.samples_per_wave);
    // every iteration either starts new paths or advances live ones by a bounce
    const uint64_t waves_of_pool = cdiv(P_tot * tn.samples_per_wave, Q) + 1;
    ctl.iter_limit = (uint32_t)std::min<uint64_t>(0x7FFFFFFFull, 4 * waves_of_pool * (p0.max_depth + 2) + 64);
    if (tn.max_iterations) ctl.iter_limit = tn.max_iterations;
    cudaMemcpy(a.ctl, &ctl, sizeof(ctl), cudaMemcpyHostToDevice);
    cudaError_t e = cudaSuccess;
    for (const void* k : {(const void*)k_wf_extend_packets, (const void*)k_wf_extend, (const void*)k_wf_shadow})
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bt->smem);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&bt->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGetLastError();
        batch_free(bt);
        return cuda_fail(e, "aur_batch_create set-up", __FILE__, __LINE__);
    }
    st = make_graph(bt);
    if (st != AUR_OK) {
        cudaGetLastError();
        batch_free(bt);
        return st;
    }
    *out = bt;
    return AUR_OK;
}

aur_status aur_batch_render(aur_ctx* ctx, aur_batch* bt, float* const* accum) {
    AUR_RANGE("aur_batch_render");
    clear_error();
    AUR_CHECK(ctx && bt && accum, AUR_ERR_INVALID, "aur_batch_render: null argument");
    AUR_CHECK(ctx->device == bt->device, AUR_ERR_INVALID, "aur_batch_render: batch lives on another device");
    AUR_CUDA(cudaSetDevice(ctx->device));
    for (uint32_t i = 0; i < bt->num_scenes; ++i) {
        AUR_CHECK(accum[i], AUR_ERR_INVALID, "aur_batch_render: frame %u is null", i);
        AUR_CHECK(!bt->scene_ptrs[i]->has_specular || bt->args.stk, AUR_ERR_INVALID,
                  "aur_batch_render: scene %u has specular shaders now; the batch was created without: create it "
                  "again", i);
        bt->accum_host[i] = (float4*)accum[i];
    }
    const aur_status st = refresh_mis_tables(ctx, bt);
    if (st != AUR_OK) return st;
    const WfArgs& a = bt->args;
    AUR_CUDA(cudaMemcpyAsync((void*)a.accum, bt->accum_host.data(), sizeof(float4*) * bt->num_scenes,
                             cudaMemcpyHostToDevice, ctx->stream));
    // reset the per-launch part of the control block: wave, error, iteration count
    // counters, error and iteration total sit at the front of the control block
    AUR_CUDA(cudaMemsetAsync(a.ctl, 0, offsetof(WfCtl, num_waves), ctx->stream));
    AUR_CUDA(cudaGraphLaunch(bt->exec, ctx->stream));
    return AUR_OK;
}

aur_status aur_batch_status(aur_ctx* ctx, aur_batch* bt, uint32_t* iterations) {
    AUR_CHECK(ctx && bt, AUR_ERR_INVALID, "aur_batch_status: null argument");
    AUR_CUDA(cudaSetDevice(ctx->device));
    WfCtl c;
    AUR_CUDA(cudaMemcpyAsync(&c, bt->args.ctl, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    if (iterations) *iterations = c.total_iters;
    AUR_CHECK(!(c.error & kWfErrLightSlots), AUR_ERR_INVALID,
              "wavefront render stopped: a scene's lights now take more samples per hit than when the batch "
              "was created; create the batch again");
    AUR_CHECK(c.error == 0, AUR_ERR_TIMEOUT,
              "wavefront render stopped: iteration limit %u reached (flags 0x%x)",
              c.iter_limit, c.error);
    AUR_CHECK(c.wave == c.num_waves, AUR_ERR_TIMEOUT, "wavefront render ended after %u of %u waves", c.wave,
              c.num_waves);
    return AUR_OK;
}

aur_status aur_batch_counters(aur_ctx* ctx, aur_batch* bt, unsigned long long counters[3]) {
    AUR_CHECK(ctx && bt && counters, AUR_ERR_INVALID, "aur_batch_counters: null argument");
    AUR_CUDA(cudaSetDevice(ctx->device));
    WfCtl c;
    AUR_CUDA(cudaMemcpyAsync(&c, bt->args.ctl, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream));
    AUR_CUDA(cudaStreamSynchronize(ctx->stream));
    counters[0] = c.total_ext;
    counters[1] = c.total_shadow;
    counters[2] = c.total_iters;
    return AUR_OK;
}

aur_status aur_batch_tuning(const aur_batch* bt, aur_wavefront_tuning* out) {
    AUR_CHECK(bt && out, AUR_ERR_INVALID, "aur_batch_tuning: null argument");
    *out = bt->tuning;
    return AUR_OK;
}

aur_status aur_batch_destroy(aur_batch* bt) {
    batch_free(bt);
    return AUR_OK;
}

// Runs the batch's stage kernels one by one from the host, without the
// graph, and accumulates the time of each stage with CUDA events:
// stage_ms[0..6] = set-up, generate (+commit), extend, shade, shadow,
// combine (+end), accumulate (+next wave). Same kernels, same results; for
// profiling only (one host round trip per iteration).
aur_status aur_batch_profile(aur_ctx* ctx, aur_batch* bt, float* const* accum, float stage_ms[7]) {
    clear_error();
    AUR_CHECK(ctx && bt && accum && stage_ms, AUR_ERR_INVALID, "aur_batch_profile: null argument");
    AUR_CUDA(cudaSetDevice(ctx->device));
    for (uint32_t i = 0; i < bt->num_scenes; ++i) bt->accum_host[i] = (float4*)accum[i];
    const aur_status rs = refresh_mis_tables(ctx, bt);
    if (rs != AUR_OK) return rs;
    const WfArgs& a = bt->args;
    cudaStream_t st = ctx->stream;
    AUR_CUDA(cudaMemcpyAsync((void*)a.accum, bt->accum_host.data(), sizeof(float4*) * bt->num_scenes,
                             cudaMemcpyHostToDevice, st));
    AUR_CUDA(cudaMemsetAsync(a.ctl, 0, offsetof(WfCtl, num_waves), st));
    cudaEvent_t ev[8];
    for (auto& e : ev) cudaEventCreate(&e);
    for (int i = 0; i < 7; ++i) stage_ms[i] = 0.0f;
    auto lap = [&](int stage, int e0, int e1) {
        float ms = 0.0f;
        cudaEventSynchronize(ev[e1]);
        cudaEventElapsedTime(&ms, ev[e0], ev[e1]);
        stage_ms[stage] += ms;
    };
    const uint32_t g = bt->grid, bs = bt->block;
    WfCtl c;
    AUR_CUDA(cudaMemcpyAsync(&c, a.ctl, sizeof(c), cudaMemcpyDeviceToHost, st));
    AUR_CUDA(cudaStreamSynchronize(st));
    for (uint32_t w = 0; w < c.num_waves; ++w) {
        cudaEventRecord(ev[0], st);
        k_wf_setup<<<g, bs, 0, st>>>(a);
        cudaEventRecord(ev[1], st);
        lap(0, 0, 1);
        for (uint32_t it = 0;; ++it) {
            cudaEventRecord(ev[0], st);
            k_wf_generate<<<g, bs, 0, st>>>(a);
            k_wf_generate_commit<<<1, 1, 0, st>>>(a);
            cudaEventRecord(ev[1], st);
            k_wf_extend_packets<<<g, bs, bt->smem, st>>>(a);
            k_wf_extend<<<g, bs, bt->smem, st>>>(a);
            cudaEventRecord(ev[2], st);
            launch_shade(a, g, bs, st);
            cudaEventRecord(ev[3], st);
            k_wf_shadow<<<g, bs, bt->smem, st>>>(a);
            cudaEventRecord(ev[4], st);
            launch_combine(a, g, bs, st);
            k_wf_end<<<1, 1, 0, st>>>(a);
            cudaEventRecord(ev[5], st);
            AUR_CUDA(cudaMemcpyAsync(&c, a.ctl, sizeof(c), cudaMemcpyDeviceToHost, st));
            AUR_CUDA(cudaStreamSynchronize(st));
            lap(1, 0, 1); lap(2, 1, 2); lap(3, 2, 3); lap(4, 3, 4); lap(5, 4, 5);
            const uint32_t nxt = c.iter & 1u;
            const bool more = (c.items_issued < c.items_total || c.ext_count[nxt] > 0) && !c.error;
            if (!more || it > c.iter_limit) break;
        }
        cudaEventRecord(ev[0], st);
        k_wf_accumulate<<<g, bs, 0, st>>>(a);
        k_wf_next_wave<<<1, 1, 0, st>>>(a);
        cudaEventRecord(ev[1], st);
        lap(6, 0, 1);
    }
    for (auto& e : ev) cudaEventDestroy(e);
    AUR_CUDA(cudaGetLastError());
    return aur_batch_status(ctx, bt, nullptr);
}

aur_status aur_batch_autotune(aur_ctx* ctx, const aur_scene* const* scenes, const aur_camera* cameras,
                              const aur_render_params* params, uint32_t num_scenes, aur_wavefront_tuning* best,
                              float* best_ms) {
    AUR_RANGE("aur_batch_autotune");
    clear_error();
    AUR_CHECK(ctx && scenes && cameras && params && best && num_scenes > 0, AUR_ERR_INVALID,
              "aur_batch_autotune: null argument");
    AUR_CUDA(cudaSetDevice(ctx->device));
    // up to two samples per pixel of the real batch (fewer if it asks for
    // fewer), into scratch frames. Pools up to 4x the probe's paths are timed
    // (they run it in one wave and tie within noise; larger ones would only
    // hold memory).
    std::vector<aur_render_params> p1(params, params + num_scenes);
    uint32_t probe = 2;
    for (const auto& p : p1) {
        const uint32_t s1 = p.sample_end ? p.sample_end : p.spp;
        probe = std::min(probe, s1 > p.sample_begin ? s1 - p.sample_begin : 1u);
    }
    for (auto& p : p1) { p.sample_end = p.sample_begin + probe; }
    size_t pixels = 0;
    for (uint32_t i = 0; i < num_scenes; ++i) pixels += (size_t)p1[i].width * p1[i].height;
    const uint64_t probe_items = (uint64_t)pixels * probe;
    float4* frames = nullptr;
    AUR_CHECK(::aur::dev_malloc(&frames, pixels * sizeof(float4)) == cudaSuccess, AUR_ERR_OOM, "aur_batch_autotune: out of memory");
    std::vector<float*> acc(num_scenes);
    for (uint32_t i = 0, o = 0; i < num_scenes; o += p1[i].width * p1[i].height, ++i) acc[i] = (float*)(frames + o);
    // Larger pools mean fewer, fuller iterations: on the 64-scene sphere batch
    // 32M paths in flight ran 16 % faster than 8M. A candidate that does not
    // fit in memory fails in aur_batch_create and is skipped.
    const uint32_t pools[] = {1u << 20, 1u << 21, 1u << 22, 1u << 23, 1u << 24, 1u << 25, 1u << 26};
    // specular batches carry 864 bytes of ray stack per path: pools up to 8M (7 GB)
    bool spec = false;
    for (uint32_t i = 0; i < num_scenes; ++i) spec = spec || (scenes[i] && scenes[i]->has_specular);
    const uint32_t max_pool = spec ? (1u << 23) : (1u << 26);
    const uint32_t blocks[] = {128, 256};
    const uint32_t per_sm[] = {4, 8, 16};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_t = 1e30f;
    aur_status st = AUR_OK;
    struct Timed {
        aur_wavefront_tuning t;
        float ms;
    };
    std::vector<Timed> timed;
    for (uint32_t pool : pools)
        for (uint32_t bs : blocks)
            for (uint32_t bps : per_sm) {
                if ((uint64_t)bs * bps > 2048 || pool > max_pool) continue;
                if (pool > 4 * probe_items && pool != pools[0]) continue;
                aur_wavefront_tuning t{pool, 1, bs, bps, 0};
                aur_batch* bt = nullptr;
                if (aur_batch_create(ctx, scenes, cameras, p1.data(), num_scenes, &t, &bt) != AUR_OK) {
                    clear_error();
                    continue;
                }
                float ms = 0.0f;
                aur_status s2 = AUR_OK;
                for (int rep = 0; rep < 2 && s2 == AUR_OK; ++rep) {   // the first launch warms up
                    cudaEventRecord(e0, ctx->stream);
                    s2 = aur_batch_render(ctx, bt, acc.data());
                    cudaEventRecord(e1, ctx->stream);
                    cudaEventSynchronize(e1);
                    cudaEventElapsedTime(&ms, e0, e1);
                }
                if (s2 == AUR_OK) s2 = aur_batch_status(ctx, bt, nullptr);
                aur_batch_destroy(bt);
                if (s2 != AUR_OK) { st = s2; continue; }
                timed.push_back({t, ms});
                best_t = std::min(best_t, ms);
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(frames);
    if (timed.empty()) return st != AUR_OK ? st : fail(AUR_ERR_CUDA, "aur_batch_autotune: no candidate ran");
    // Of the candidates within 3 % of the fastest probe, the largest pool (then
    // the fastest): the probe is short, and a render of many samples runs
    // fewer, fuller iterations with a larger pool (over all 64 samples of the
    // 64-scene sphere batch: 16M 3.56 s, 32M 3.31 s, 64M 3.04 s, equal on
    // the probe; the terrain's 16 samples: 2M 1.70 s, 16M 1.67 s).
    const Timed* pick = nullptr;
    for (const Timed& c : timed) {
        if (c.ms > best_t * 1.03f) continue;
        if (!pick || c.t.paths_in_flight > pick->t.paths_in_flight ||
            (c.t.paths_in_flight == pick->t.paths_in_flight && c.ms < pick->ms))
            pick = &c;
    }
    *best = pick->t;
    best_t = pick->ms;
    best->samples_per_wave = 0;   // chosen per batch from the frame size
    if (best_ms) *best_ms = best_t;
    return AUR_OK;
}

}  // extern "C"
