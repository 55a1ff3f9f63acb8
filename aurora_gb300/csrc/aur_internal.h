// aur_internal.h — library-internal objects and error plumbing.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/aurora_gb300.h"

namespace aur {

// Thread-local error message; returns `st` for tail calls.
aur_status fail(aur_status st, const char* fmt, ...);
aur_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);
void clear_error();

#define AUR_CUDA(call)                                                                    \
    do {                                                                                  \
        cudaError_t aur_e_ = (call);                                                      \
        if (aur_e_ != cudaSuccess) return ::aur::cuda_fail(aur_e_, #call, __FILE__, __LINE__); \
    } while (0)

#define AUR_CHECK(cond, st, ...)                                  \
    do {                                                          \
        if (!(cond)) return ::aur::fail((st), __VA_ARGS__);       \
    } while (0)

// Every device and pinned allocation of the library goes through these, so
// that tests can make the k-th one fail (aur_debug_fail_allocation) and check
// each caller's out-of-memory path.
cudaError_t alloc_device(void** p, size_t bytes);
cudaError_t alloc_device_async(void** p, size_t bytes, cudaStream_t s);
cudaError_t alloc_pinned(void** p, size_t bytes);
template <typename T>
inline cudaError_t dev_malloc(T** p, size_t bytes) { return alloc_device((void**)p, bytes); }
template <typename T>
inline cudaError_t dev_malloc_async(T** p, size_t bytes, cudaStream_t s) {
    return alloc_device_async((void**)p, bytes, s);
}

// NVTX range over an entry point (a no-op unless a profiler is attached).
struct Range {
    explicit Range(const char* name);
    ~Range();
};
#define AUR_RANGE(name) ::aur::Range aur_range_(name)

// Grow-only device scratch owned by a context (stream-ordered allocation).
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};

// Largest triangle count: node indices carry the axis in their top 2 bits.
constexpr uint32_t kMaxTriangles = 1u << 30;
// Traversal stack entries per thread (one per heap level; 2^30 triangles
// give 30 levels).
constexpr int kStackDepth = 32;

// A context's cached NMH build (scratch and recorded launch graph), owned
// by nmh_build.cu; freed with the context.
struct BuildCache;

}  // namespace aur

struct aur_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;       // launch stream (own or caller's)
    cudaStream_t copy_in = nullptr;      // host-buffer pipelines
    cudaStream_t copy_out = nullptr;
    cudaStream_t compute2 = nullptr;     // second launch stream of the host-buffer pipelines
    uint32_t* d_flags = nullptr;         // small device scratch: counters, error flags
    aur::Scratch pipe[2];                // double-buffered device chunks for *_host calls
    aur::Scratch out[2];
    aur::Scratch defer[2];               // per trace slot: ray chunks left to the per-lane kernel
    cudaEvent_t ev[8] = {};
    aur::BuildCache* build = nullptr;    // created by the first aur_nmh_build
    uint32_t lookback_test = 0;          // test hook for the next build (aur_debug_lookback_timeout)
};

struct aur_nmh {
    int device = 0;
    uint32_t count = 0;       // triangles after even padding
    uint32_t input_count = 0; // triangles as given
    uint32_t levels = 0;
    uint32_t nodes = 0;       // count / 2
    void* mem = nullptr;          // one allocation holding the three arrays below
    float4* node_recs = nullptr;  // nodes * 8 float4 (slab, 2 x (v1, e1, e2), children's boxes)
    uint32_t* perm = nullptr;     // NMH position -> original prim id
    float* verts = nullptr;       // count * 9, NMH order, reference layout
    // node_recs as a linear texture of float4 texels: k_trace reads one of a
    // node's four sectors through the texture path (0: none, plain loads)
    cudaTextureObject_t rec_tex = 0;
    // Largest side of the bounding box of all triangles (from the root node's
    // record): the scale for deciding when a warp's rays are close enough
    // together to traverse as a packet.
    float extent = 0.0f;
};

struct aur_scene {
    aur_nmh* nmh = nullptr;
    float* normals = nullptr;         // count * 9, NMH order
    uint16_t* shader_ids = nullptr;   // count, NMH order
    aur_shader* shaders = nullptr;
    uint32_t num_shaders = 0;
    aur_light* lights = nullptr;
    uint32_t num_lights = 0;
    bool has_specular = false;        // any shader with reflectivity or translucence > 0
    uint32_t max_texture = 0;         // largest texture id (<= 32) any shader names
    float* texcoords = nullptr;       // count * 6, NMH order
    uint32_t num_textures = 0;
    uchar4* texels = nullptr;         // all textures' RGBA8 texels, row-major, one after another
    uint4* tex_info = nullptr;        // per texture: first texel, width, height
    // Light-selection table of AUR_MODE_PATH_MIS, built by the first render
    // that needs it and dropped when the shaders change.
    mutable bool mis_ready = false;
    mutable uint32_t mis_count = 0;
    mutable uint32_t* mis_tri = nullptr;   // mis_count NMH positions
    mutable float* mis_cdf = nullptr;      // mis_count
    mutable float* mis_pa = nullptr;       // count: selection probability / area per NMH triangle
};

namespace aur {

aur_status nmh_build_impl(aur_ctx* ctx, const float* vertices, uint32_t count, aur_nmh** out);
// Releases the context's cached build scratch and graph (after its last launch).
void free_build_cache(aur_ctx* ctx);
aur_status check_params(const aur_render_params* p);
// Builds the scene's light-selection table for AUR_MODE_PATH_MIS if it is
// not built (stream-synchronous); free_mis_table drops it.
aur_status build_mis_table(aur_ctx* ctx, const aur_scene* sc);
void free_mis_table(const aur_scene* sc);
// Every texture the scene's shaders name exists (and texcoords were given).
aur_status check_scene_textures(const aur_scene* sc);
// slot: the work counters (d_flags[16 + 4 * slot ...]) and deferred-chunk
// list (defer[slot]) of the launch; launches that may run concurrently need
// distinct slots (0 or 1).
aur_status launch_trace(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, aur_hit* hits,
                        uint32_t* occluder, unsigned long long* counters, cudaStream_t stream, bool pruned,
                        int slot = 0);

}  // namespace aur
