/*
 * aurora_gb300 — C ABI of the GB300-native (sm_103a) rendering hot path.
 *
 * The entry points replace the free functions the Aurora renderer binds in
 * src/kernels/kernels.h:27-64 (Nadrin/aurora). Each declaration below names the
 * reference function it stands in for. Everything crossing this boundary is a
 * plain C type: POD structs, raw pointers and sizes. No C++ or torch types.
 *
 * Conventions
 *  - Every function returns aur_status. AUR_OK is 0. On failure a message for
 *    the calling thread is available from aur_last_error().
 *  - An aur_ctx owns one CUDA device and one stream. Calls on one context must
 *    not race each other; distinct contexts are independent.
 *  - Pointers documented as "device" must be device-accessible memory of the
 *    context's device; "host" pointers are ordinary (preferably pinned) host
 *    memory. Library-owned objects (aur_nmh, aur_scene) are freed by their
 *    destroy function and never free caller memory (unlike cudaRebuildNMH,
 *    which frees and replaces the caller's Geometry, rebuilder.cu:444-445).
 *  - Triangle soups use the reference layout (data/geometry.h:13-55,
 *    kernels/lib/primitive.cuh:288-293): vertices are 9 floats per triangle
 *    ordered [x1 x2 x3 y1 y2 y3 z1 z2 z3]; normals are 9 floats per triangle
 *    ordered [n1.xyz n2.xyz n3.xyz]; shader ids are 1-based uint16 (0 selects
 *    shader 0, util/array.h:12-18).
 */
#ifndef AURORA_GB300_H
#define AURORA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */

typedef enum aur_status {
    AUR_OK = 0,
    AUR_ERR_INVALID = 1,     /* bad argument, size or pointer */
    AUR_ERR_OOM = 2,         /* device allocation failed (reference: MS::kInsufficientMemory) */
    AUR_ERR_CUDA = 3,        /* CUDA runtime error; the message holds cudaGetErrorString */
    AUR_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    AUR_ERR_OVERFLOW = 5,    /* a fixed-capacity device stack or queue would overflow */
    AUR_ERR_UNSUPPORTED = 6, /* feature outside this library's scope (textures) */
    AUR_ERR_NO_DEVICE = 7    /* no CUDA device, or the device is not sm_103 */
} aur_status;

/* Message describing the last failure on the calling thread ("" if none). */
const char* aur_last_error(void);
/* Library version string. */
const char* aur_version(void);

/* Fault injection for tests of the out-of-memory paths: the k-th device or
 * pinned allocation the library makes from now on (any thread, any context)
 * fails as out of memory, after which injection is off again; k = 0 turns it
 * off. No counterpart in the reference, which checks few of its allocations. */
aur_status aur_debug_fail_allocation(uint32_t k);

/* ------------------------------------------------------------ shared types */

typedef struct aur_float3 { float x, y, z; } aur_float3;

/* Ray for the traversal entry points: origin + tmax, direction + padding.
 * Reference: util/ray.h:13-49 (pos, dir, t). 32 bytes, 16-byte aligned. */
typedef struct aur_ray {
    float ox, oy, oz, tmax;
    float dx, dy, dz, pad;
} aur_ray;

/* Closest-hit result (util/hitpoint.h: u, v, triangleID; ray.t).
 * prim is the ORIGINAL triangle index (before NMH reordering), AUR_NO_HIT on a
 * miss, in which case t = tmax and u = v = 0. */
typedef struct aur_hit { float t, u, v; uint32_t prim; } aur_hit;
#define AUR_NO_HIT 0xFFFFFFFFu

/* util/shader.h:10-33. type: 0 Lambert, 1 Phong (shaded as Lambert,
 * kernels/lib/bsdf.cuh:202-210). texture must be 0 (textures are out of scope). */
typedef struct aur_shader {
    int32_t type;
    aur_float3 diffuse_color;
    aur_float3 emission_color;
    aur_float3 specular_color;
    aur_float3 reflection_color;
    float diffuse;
    float emission;
    float exponent;
    float reflectivity;
    float translucence;
    float refractive_index;
    uint32_t texture;
} aur_shader;

enum { AUR_SHADER_LAMBERT = 0, AUR_SHADER_PHONG = 1 };

/* util/light.h:12-42. For an area light, position is the quad corner v1 and
 * e1, e2 its edges (core/scene.cpp:435-448); direction is the emitting normal.
 * samples >= 1 shadow samples per shading point (numShadowSamples). */
typedef struct aur_light {
    int32_t type;
    float intensity;
    float ambient;
    float area;
    int32_t samples;
    aur_float3 position;
    aur_float3 color;
    aur_float3 direction;
    aur_float3 e1, e2;
} aur_light;

enum { AUR_LIGHT_AMBIENT = 0, AUR_LIGHT_POINT = 1, AUR_LIGHT_DIRECTIONAL = 2, AUR_LIGHT_AREA = 3 };

/* util/camera.h:12-36 (pinhole; tanfov = tanf(port field of view)). */
typedef struct aur_camera {
    aur_float3 position;
    aur_float3 forward;
    aur_float3 right;
    aur_float3 up;
    float tanfov_x, tanfov_y;
    float aspect;
} aur_camera;

/* Integrator selection.
 *  AUR_MODE_REFERENCE: exactly the reference integrator
 *    (kernels/monteCarloRaytracer.cu:23-113): emission + direct lighting at
 *    each hit, specular reflection/refraction rays, no diffuse bounce.
 *  AUR_MODE_PATH: the same, plus a cosine-sampled diffuse bounce
 *    (BSDF::samplef, kernels/lib/bsdf.cuh:222-236) at every non-specular hit
 *    while depth <= max_depth, with RGB path throughput.
 *  AUR_MODE_PATH_MIS: path mode with physically based direct lighting and
 *    multiple importance sampling (power heuristic): area lights by both
 *    halves of estimateDirectRadiance (kernels/lib/radiance.cuh:41-71, the
 *    BSDF half compiled out in the reference) with solid-angle densities and
 *    the reference's emission model Light::L (light.cuh:18-22); emissive
 *    triangles sampled from a table proportional to emission * area, their
 *    emission found by diffuse bounces weighted against it. Images differ
 *    from the other modes by design (the reference's light sample has no
 *    area / distance^2 factor). Every render entry point and the adjoint
 *    take it; at most 32766 lights. */
enum { AUR_MODE_REFERENCE = 0, AUR_MODE_PATH = 1, AUR_MODE_PATH_MIS = 2 };

/* Per-render parameters (Dim(width,height,samples), MAX_DEPTH, RNG seed). */
typedef struct aur_render_params {
    uint32_t width, height;
    uint32_t spp;            /* samples per pixel; sub-pixel grid of (short)sqrtf(spp) */
    uint32_t max_depth;      /* MAX_DEPTH (monteCarloRaytracer.cu:20); <= AUR_MAX_DEPTH */
    uint32_t seed;           /* counter-based RNG key (replaces curand_init seed) */
    uint32_t mode;           /* AUR_MODE_* */
    uint32_t sample_begin;   /* render samples [sample_begin, sample_end) of spp; */
    uint32_t sample_end;     /*   sample_end == 0 means spp */
    uint32_t scene_id;       /* second RNG key word: independent streams per scene */
} aur_render_params;

#define AUR_MAX_DEPTH 16u

/* The reference Ray / HitPoint structs for the renderer-helper entry points
 * (util/ray.h:13-49, util/hitpoint.h:10-23). Layout is part of the ABI. */
typedef struct aur_path_ray {
    aur_float3 pos;
    aur_float3 dir;
    float t;
    float weight;
    float eta;
} aur_path_ray;

typedef struct aur_hitpoint {
    aur_float3 color;
    aur_float3 position;
    aur_float3 wo;
    float u, v;
    int32_t triangle_id;      /* NMH position of the last hit, -1 if none */
} aur_hitpoint;

/* ----------------------------------------------------------------- context */

typedef struct aur_ctx aur_ctx;

/* Creates a context on CUDA device `device` with its own non-blocking stream.
 * Replaces Engine::initialize's cudaSetDevice (core/engine.cpp:33-47). */
aur_status aur_ctx_create(int device, aur_ctx** out);
aur_status aur_ctx_destroy(aur_ctx* ctx);
/* Uses `cuda_stream` (a cudaStream_t) for all later work; NULL restores the
 * context's own stream. To launch on the legacy default stream pass
 * cudaStreamLegacy ((cudaStream_t)0x1). */
aur_status aur_ctx_set_stream(aur_ctx* ctx, void* cuda_stream);
/* Returns the cudaStream_t the context launches on. */
aur_status aur_ctx_get_stream(aur_ctx* ctx, void** cuda_stream);
aur_status aur_ctx_synchronize(aur_ctx* ctx);
/* Number of SMs of the context's device. */
aur_status aur_ctx_sm_count(aur_ctx* ctx, int* sm_count);

/* ------------------------------------------------------------------ memory */

/* Memory policies of core/memory.h (HostMemory, DeviceMemory) plus pinned
 * host memory (the mapped staging buffers of Geometry::resizeStaging,
 * data/geometry.cpp:50-73). */
enum { AUR_HOST_MEMORY = 0, AUR_DEVICE_MEMORY = 1, AUR_PINNED_MEMORY = 2 };

/* Aurora::malloc / memzero / memupload / free (core/memory.cpp). memupload
 * copies `bytes` from host memory to `dst` of the given policy; memdownload
 * copies device memory to host memory. Device operations run on the context's
 * stream and are complete when the call returns. */
aur_status aur_malloc(aur_ctx* ctx, size_t bytes, int policy, void** out);
aur_status aur_free(aur_ctx* ctx, void* ptr, int policy);
aur_status aur_memzero(aur_ctx* ctx, void* ptr, size_t bytes, int policy);
aur_status aur_memupload(aur_ctx* ctx, void* dst, const void* src, size_t bytes, int policy);
aur_status aur_memdownload(aur_ctx* ctx, void* dst, const void* src, size_t bytes);

/* --------------------------------------------------------------------- NMH */

typedef struct aur_nmh aur_nmh;

/* Builds the NMH (implicit pair-heap) over `count` triangles.
 * Replaces cudaRebuildNMH(Geometry&) (kernels/rebuilder.cu:311-450).
 * vertices: device, count*9 floats, reference layout. An odd count is padded
 * by duplicating the last triangle (Geometry::padToEven, data/geometry.cpp:164-176);
 * the duplicate gets prim id `count`. Ties in every ordering are broken by the
 * lower original prim id, which makes the result deterministic where the
 * reference's atomicCAS swap (rebuilder.cu:93-125) is not. A NaN or infinite
 * coordinate returns AUR_ERR_INVALID (the reference's float sorts have no
 * order for NaN).
 * Soups of at most 2^24 triangles (after padding) run from a per-context
 * cache: the build's scratch (about 92 bytes per triangle, kept until the
 * context is destroyed and grown when a larger soup comes) and, for up to
 * four sizes, the launch sequence recorded as one CUDA graph. The first
 * build of a size launches directly; the second records the graph; later
 * ones launch it with the new vertex and output pointers written into it
 * (cudaRebuildNMH runs every frame on the same geometry). Larger soups launch
 * directly with stream-ordered scratch that is released after the build.
 * Builds on one context are serialized on the GPU (each call also waits for
 * its own build before returning). */
aur_status aur_nmh_build(aur_ctx* ctx, const float* vertices, uint32_t count, aur_nmh** out);
/* Test hook for the bounded waits of the build (no counterpart in the
 * reference, whose build waits on nothing on the device). The build's split
 * and partition passes are single-pass scans whose tiles wait for their
 * predecessors' prefixes (decoupled look-back); each wait gives up after a
 * bounded number of spins and the build then returns AUR_ERR_TIMEOUT, with
 * the context still usable. With spins != 0, the next aur_nmh_build on ctx
 * (and only that one) makes every tile after the first wait for `spins`
 * spins on a prefix that nothing publishes, so the give-up path runs on
 * purpose: that build returns AUR_ERR_TIMEOUT and creates no NMH. Soups of
 * at most 4,096 triangles have no such wait and build normally. */
aur_status aur_debug_lookback_timeout(aur_ctx* ctx, uint32_t spins);
/* Test hook (no counterpart in the reference): the NMH's node records are
 * bound as a texture at build, and the traversal entry points read part of
 * each node through it; an NMH too large for a texture (over about 33M
 * triangles) is traversed with plain loads only. This drops the texture of
 * `nmh` (after synchronizing its device), so that tests can compare both
 * paths on small soups. */
aur_status aur_debug_nmh_drop_texture(aur_nmh* nmh);
/* Frees the NMH (its records, permutation and vertices, and the records'
 * texture). Synchronizes the NMH's device first: no launch may still be
 * reading it. */
aur_status aur_nmh_destroy(aur_nmh* nmh);
/* Triangle count after padding and number of heap levels (log2i(count/2)+1). */
aur_status aur_nmh_info(const aur_nmh* nmh, uint32_t* count, uint32_t* levels);
/* Copies the topology to host memory: perm[i] = original prim id at NMH
 * position i (count entries); vertices (nullable) = count*9 floats of the
 * permuted soup in the reference layout (applyIndices, rebuilder.cu:217-245). */
aur_status aur_nmh_export(aur_ctx* ctx, const aur_nmh* nmh, uint32_t* perm, float* vertices);
/* applyIndices (kernels/rebuilder.cu:217-245) for any per-triangle
 * attribute: dst[i] = src[perm[i]] for the `count` NMH positions, each
 * `bytes_per_triangle` bytes (a multiple of 2); the padding triangle of an odd
 * soup reads the last input triangle. src, dst: device. */
aur_status aur_nmh_apply(aur_ctx* ctx, const aur_nmh* nmh, const void* src, uint32_t bytes_per_triangle, void* dst);
/* Device pointer to the perm array (count uint32) owned by the NMH. */
aur_status aur_nmh_perm_device(const aur_nmh* nmh, const uint32_t** perm);

/* NMH build that allocates no device memory. This entry point has no
 * counterpart in the reference. It is for callers that cannot call
 * cudaMalloc: a plug-in whose host application owns the GPU's memory budget
 * and only hands out fixed buffers, or a render loop that must not pay for
 * cudaMalloc / cudaFree, which can synchronize the whole device.
 * Same result as aur_nmh_build, written into caller-owned device buffers:
 *   node_records: ((count+1)/2) * 32 floats, 32-byte aligned (traversal records,
 *                 read with 256-bit loads)
 *   perm:         count + (count & 1) uint32 (NMH position -> original prim id)
 *   nmh_vertices: (count + (count & 1)) * 9 floats (NMH-ordered soup)
 *   levels:       host, nullable; receives 0 for count == 0, else
 *                 log2i((count+1)/2)+1 (the heap's level count)
 * Runs on `cuda_stream` (NULL = the legacy default stream) of the current
 * device and returns after the build has finished on that stream.
 * Limit: at most 65,536 triangles; larger counts return AUR_ERR_INVALID. The
 * scratch is one fixed device array inside the library (about 6 MB), which
 * every GPU that loads the library holds until the process exits. The first
 * call on a device looks up that array's device address
 * (cudaGetSymbolAddress) with the device current; make that first call before
 * any stream capture. The address is kept per device ordinal for the life of
 * the process: a cudaDeviceReset of that device invalidates it, so do not
 * call this entry point again on a device after resetting it. All calls share
 * the array: calls whose work overlaps on the GPU (other streams, other host
 * threads) race and must be serialized by the caller. */
aur_status aur_nmh_build_noalloc(const float* vertices, uint32_t count, void* cuda_stream, float* node_records,
                                 uint32_t* perm, float* nmh_vertices, uint32_t* levels);

/* ------------------------------------------------------------- scene prep */

/* Object-to-world transform of one object (util/transform.h:12-26):
 * triangles [offset, offset + size) use row-vector matrices,
 * p' = p * world_matrix, n' = n * normal_matrix (the inverse transpose). */
typedef struct aur_object_transform {
    uint32_t offset;
    uint32_t size;
    float world_matrix[4][4];
    float normal_matrix[4][4];
} aur_object_transform;

/* cudaTransform (kernels/utility.cu:96-134): writes world-space vertices and
 * normals of `count` triangles. Triangle i uses the last object whose offset
 * is <= i (offsets must be non-decreasing); triangles before the first
 * object are left untouched. src_*, dst_*: device, count*9 floats;
 * transforms: host array of num_objects. */
aur_status aur_transform(aur_ctx* ctx, const float* src_vertices, const float* src_normals, uint32_t count,
                         const aur_object_transform* transforms, uint32_t num_objects, float* dst_vertices,
                         float* dst_normals);
/* cudaGenerateTB (kernels/utility.cu:136-180): per-vertex tangents
 * n x (0,1,0) (n x (0,0,1) when shorter than Epsilon) and bitangents
 * n x tangent. normals, tangents, bitangents: device, count*9 floats. The
 * renderers compute the same frames at shading time and need no stored ones. */
aur_status aur_generate_tb(aur_ctx* ctx, const float* normals, uint32_t count, float* tangents, float* bitangents);

/* --------------------------------------------------------------- traversal */

/* Closest hit for n rays (intersect(), kernels/lib/intersect.cuh:95-152).
 * rays, hits: device. Ties in t go to the lower original prim id. Rays are
 * taken in chunks of 32 consecutive rays: a chunk whose directions share
 * their octant (signs of x, y, z) is traversed by one warp together, which
 * is fastest for coherent rays (a camera's, rays toward one light); the
 * other chunks are traversed one ray per thread. Results are the same. The
 * first call with more rays than before allocates 4 bytes per 32 rays. */
aur_status aur_trace_closest(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, aur_hit* hits);
/* Any hit (shadow ray, intersectAny(), intersect.cuh:36-86): occluder[i] is
 * the original prim id of the first hit found in traversal order with
 * Epsilon < t < tmax, or AUR_NO_HIT. rays, occluder: device. Chunks of
 * one octant go to warp packets as in aur_trace_closest. */
aur_status aur_trace_any(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, uint32_t* occluder);
/* Same as above with HOST buffers: rays go in chunks of up to 8M (a 2M
 * chunk first and, where the count allows, last), traced on the context's
 * stream and one internal launch stream in turn, with two internal copy
 * streams overlapping the copies; returns when all hits are back. The
 * context keeps two 8M-ray slots of device memory (384 MiB each) after the
 * first call. */
aur_status aur_trace_closest_host(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, aur_hit* hits);
aur_status aur_trace_any_host(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, uint32_t* occluder);
/* Counts the reference algorithm's traversal work for n device rays:
 * node_visits[0] = nodes fetched by closest hit, node_visits[1] = by any hit
 * (a node is fetched when popped with index < count, intersect.cuh:103-111),
 * counted by running the traversal without subtree-box pruning. */
aur_status aur_trace_count_visits(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n,
                                  unsigned long long node_visits[2]);

/* Test hook: the number of 32-ray chunks that the last aur_trace_closest /
 * aur_trace_any on this context left to the one-ray-per-thread kernel
 * (directions of more than one octant). Synchronizes the context's stream. */
aur_status aur_debug_trace_deferred(aur_ctx* ctx, uint32_t* chunks);

/* Work of this library's traversal (with subtree-box pruning) over n rays:
 * node records fetched (16-byte slab load), slabs crossed (two triangles,
 * 64 bytes, tested) and children's boxes loaded (48 bytes). No reference
 * counterpart; used for roofline accounting. */
typedef struct aur_trace_work {
    unsigned long long node_fetches;
    unsigned long long slab_crossings;
    unsigned long long box_loads;
} aur_trace_work;
aur_status aur_trace_stats(aur_ctx* ctx, const aur_nmh* nmh, const aur_ray* rays, uint32_t n, aur_trace_work* closest,
                           aur_trace_work* any);

/* ------------------------------------------------------------------- scene */

typedef struct aur_scene aur_scene;

/* Uploads a triangle soup with its materials and lights and builds its NMH
 * (Scene::update / updateMeshes, core/scene.cpp:144-299). Host pointers.
 * normals: nullable (face normals are used); shader_ids: nullable (all 0). */
aur_status aur_scene_create(aur_ctx* ctx, const float* vertices, const float* normals,
                            const uint16_t* shader_ids, uint32_t count,
                            const aur_shader* shaders, uint32_t num_shaders,
                            const aur_light* lights, uint32_t num_lights, aur_scene** out);
aur_status aur_scene_destroy(aur_scene* scene);
aur_status aur_scene_nmh(const aur_scene* scene, const aur_nmh** nmh);
/* Replaces the shader / light tables (same counts as at creation). Host pointers. */
aur_status aur_scene_set_shaders(aur_ctx* ctx, aur_scene* scene, const aur_shader* shaders, uint32_t num_shaders);
aur_status aur_scene_set_lights(aur_ctx* ctx, aur_scene* scene, const aur_light* lights, uint32_t num_lights);

/* An RGBA8 image in host memory: width * height texels of 4 bytes, row-major,
 * row 0 first (Texture::load, data/texture.cpp:15-26). */
typedef struct aur_texture {
    uint32_t width, height;
    const uint8_t* rgba;
} aur_texture;
#define AUR_MAX_TEXTURES 32
/* Textures of a scene (Scene::updateTextures, core/scene.cpp:298-327) and the
 * per-triangle texture coordinates of Geometry::texcoords: `texcoords` holds
 * 6 floats per triangle (u1 v1 u2 v2 u3 v3, Primitive2::readValues,
 * kernels/lib/primitive.cuh:14-19) in the scene's original triangle order,
 * host memory. A shader with texture = t (1-based, shader.h:37) then shades
 * with texel(t - 1, uv) * diffuse instead of diffuse_color * diffuse, where
 * uv interpolates the texcoords barycentrically and texel() is a bilinear,
 * wrapping fetch of normalised RGBA8 (monteCarloRaytracer.cu:37-40,
 * texunit.cuh:11-18, 54-94), computed by the formula the CUDA Programming
 * Guide documents for the texture unit (weights with 8 fractional bits); the
 * texture unit itself blends at a precision the guide leaves open (within
 * 1.3e-3 of this formula on GB300). t > 32 fetches white, as the reference's
 * texfetch does. At most AUR_MAX_TEXTURES textures. Replaces earlier ones.
 * Every render entry point checks that each texture a shader names exists.
 * Frees the scene's previous textures: not while a batch built from the scene
 * (aur_batch_create) or a render on another stream may still read them. */
aur_status aur_scene_set_textures(aur_ctx* ctx, aur_scene* scene, const float* texcoords, const aur_texture* textures,
                                  uint32_t num_textures);
/* An emissive triangle (Emitter, util/emitter.h:10-21): triangle_id is its
 * NMH position, as the reference's ids after the rebuild are. */
typedef struct aur_emitter {
    float area, pdf, cdf;
    aur_float3 power;
    uint32_t triangle_id;
} aur_emitter;
/* cudaCreateEmitters (kernels/emitter.cu:39-119): the triangles (NMH order,
 * the even-padding copy included, as in the reference) whose shader has
 * emission > 0, with area (Primitive3::area), pdf = 1 / area, power = the
 * shader's emission colour and the inclusive CDF of the emission weights
 * normalised to 1 (summed in double; the reference sums in float in Thrust's
 * scan order). `emitters`: device, room for one record per triangle;
 * *num_emitters (host) receives the count. */
aur_status aur_scene_emitters(aur_ctx* ctx, const aur_scene* scene, aur_emitter* emitters, uint32_t* num_emitters);
/* The light-selection table AUR_MODE_PATH_MIS samples emissive triangles
 * from (no reference counterpart; built on first use, rebuilt after
 * aur_scene_set_shaders): the triangles with emission > 0 and positive area,
 * the even-padding copy left out, in NMH order; `cdf` the inclusive CDF of
 * emission * area (summed in double, normalised, rounded to float); `pa` per
 * NMH triangle (aur_nmh_info count) the selection probability / area, 0 for
 * triangles not in the table. Outputs may be NULL, host or device memory;
 * `triangles` and `cdf` need room for one entry per triangle. */
aur_status aur_scene_mis_table(aur_ctx* ctx, const aur_scene* scene, uint32_t* triangles, float* cdf, float* pa,
                               uint32_t* count);
/* texel(texture - 1, uv) for n device (u, v) pairs into n device RGB triples
 * (the fetch the integrators use; no reference counterpart). */
aur_status aur_scene_texfetch(aur_ctx* ctx, const aur_scene* scene, uint32_t texture, const float* uv, uint32_t n,
                              float* rgb);

/* --------------------------------------------------------------- rendering */

/* Camera::Camera (util/camera.h:15-28): forward = normalize(direction),
 * right = cross(forward, (0,1,0)), up = cross(right, forward),
 * tanfov = tanf(fov). Host-only helper. */
aur_status aur_camera_make(aur_float3 position, aur_float3 direction, float fov_x, float fov_y,
                           float aspect, aur_camera* out);

/* Renders params->width x params->height pixels, samples
 * [sample_begin, sample_end) of params->spp, and ADDS them into accum
 * (device float4 per pixel, RGBA, alpha = coverage) with weight 1/spp.
 * Fused form of the reference per-sample loop (monteCarloRaytracer.cpp:81-120):
 * generateRays + cudaRaytraceMonteCarlo + drawPixels. */
aur_status aur_render(aur_ctx* ctx, const aur_scene* scene, const aur_camera* camera,
                      const aur_render_params* params, float* accum);

/* Renderer helpers, one per reference kernel wrapper. */
/* cudaGenerateRays (kernels/utility.cu:79-94). rays, hits: device, width*height. */
aur_status aur_generate_rays(aur_ctx* ctx, uint32_t width, uint32_t height, uint32_t sample_id,
                             uint32_t samples, const aur_camera* camera,
                             aur_path_ray* rays, aur_hitpoint* hits);
/* cudaRaytraceMonteCarlo (monteCarloRaytracer.cu:115-124) on rays
 * [offset, offset+num_rays). The RNG is keyed by (params->seed,
 * params->scene_id, ray index as pixel, sample_id). */
aur_status aur_raytrace_monte_carlo(aur_ctx* ctx, const aur_scene* scene, const aur_render_params* params,
                                    uint32_t sample_id, uint32_t offset, uint32_t num_rays,
                                    aur_path_ray* rays, aur_hitpoint* hits);
/* cudaDrawPixels (kernels/utility.cu:199-229): accum[p] += (color*weight, weight)
 * where hits[p].triangle_id != -1. */
aur_status aur_draw_pixels(aur_ctx* ctx, uint32_t width, uint32_t height, float weight,
                           const aur_hitpoint* hits, float* accum);
/* Renderer::clearPixels (core/renderer.cpp:33-36). */
aur_status aur_clear_pixels(aur_ctx* ctx, uint32_t width, uint32_t height, float* accum);

/* Checkpoints of an accumulation buffer (no counterpart in the reference,
 * whose accumulation lives only in device memory). aur_accum_save writes the
 * width*height float4 pixels of `accum` (device) with the frame's spp and the
 * number of samples already added (samples_done) to `path`: 8-byte magic
 * "AURACC1\0", uint32 width, height, samples_done, spp, then the pixels,
 * little-endian. aur_accum_load reads such a file into `accum` (device) after
 * checking its size, and returns samples_done and spp. The counter-based RNG
 * makes a resumed render (sample_begin = samples_done) equal the
 * uninterrupted one bit for bit. */
aur_status aur_accum_save(aur_ctx* ctx, const char* path, uint32_t width, uint32_t height, uint32_t samples_done,
                          uint32_t spp, const float* accum);
aur_status aur_accum_load(aur_ctx* ctx, const char* path, uint32_t width, uint32_t height, uint32_t* samples_done,
                          uint32_t* spp, float* accum);

/* A pixel rectangle, bounds inclusive (Rect, util/math.h:283-313). */
typedef struct aur_rect {
    uint32_t left, right, bottom, top;
} aur_rect;
/* cudaFilterPixels (kernels/utility.cu:231-268): 3x3 binomial filter
 * (1 2 1 / 2 4 2 / 1 2 1) / 16 of the float4 pixels of `region` (NULL = the
 * whole frame) from `in` into `out`, taps clamped to the region; pixels of
 * `out` outside the region are left as they are. The reference clamps the
 * row below to region.bottom instead of region.top (utility.cu:241-243); here
 * it is clamped to region.top. in and out: device, width*height float4 each,
 * distinct. */
aur_status aur_filter_pixels(aur_ctx* ctx, uint32_t width, uint32_t height, const aur_rect* region, const float* in,
                             float* out);

/* ----------------------------------------------------------------- adjoint */

/* Gradients of a loss with respect to every shader's diffuse_color, every
 * shader's emission_color and every light's color, by path replay
 * backpropagation. No counterpart in the reference. d_image: device,
 * width*height float4 = dLoss/d(accum) of aur_render with the same
 * parameters (alpha ignored). d_diffuse (num_shaders*3), d_light_color
 * (num_lights*3) and d_emission (num_shaders*3, nullable: no emission
 * gradients), device: gradients are ADDED. Same estimator and RNG streams
 * as aur_render, in every mode and for every material (each sample's path is
 * replayed once through the integrator's ray stack; nothing is allocated). In
 * AUR_MODE_PATH_MIS neither the MIS weights nor the light-selection table
 * depend on the differentiated colours (the table weighs emitters by the
 * scalar `emission` times area). A textured shader's colour is not its
 * diffuse_color: its diffuse entries stay zero. Emission colour is found at
 * every hit (monteCarloRaytracer.cu:42) and, in AUR_MODE_PATH_MIS, by the
 * emitter sample of every hit. */
aur_status aur_render_adjoint(aur_ctx* ctx, const aur_scene* scene, const aur_camera* camera,
                              const aur_render_params* params, const float* d_image, float* d_diffuse,
                              float* d_light_color, float* d_emission);

/* ------------------------------------------------------ batched wavefront */

/* Launch configuration of the wavefront integrator (0 = default). */
typedef struct aur_wavefront_tuning {
    uint32_t paths_in_flight;   /* path pool size (queue capacity) */
    uint32_t samples_per_wave;  /* samples per pixel processed per wave */
    uint32_t block_size;        /* threads per block of the stage kernels: multiple of 32, at most 256 */
    uint32_t blocks_per_sm;     /* persistent grid = SMs x blocks_per_sm */
    uint32_t max_iterations;    /* device-side loop limit per wave (0 = derived from the work) */
} aur_wavefront_tuning;

typedef struct aur_batch aur_batch;

/* Prepares a wavefront render of `num_scenes` scenes of uneven size as ONE
 * CUDA graph (conditional while nodes over sample waves and integrator
 * iterations). No counterpart in the reference, which renders one scene per
 * frame with a host loop (render/monteCarloRaytracer.cpp:81-120); each scene's
 * frame equals aur_render's with the same parameters (same estimator, same
 * RNG streams keyed by params[i].scene_id). params[i] may differ in width,
 * height and scene_id only. With specular shaders (reflectivity or
 * translucence > 0) each path keeps its sample's pending rays, the plain
 * integrator's ray stack, in device memory (864 bytes per path in flight);
 * a scene given specular shaders after the batch was created needs a new
 * batch (aur_batch_render returns AUR_ERR_INVALID). The batch reads
 * the scenes' device data in place: each scene must outlive the batch, and
 * its textures must not be replaced (aur_scene_set_textures) while the batch
 * exists. Shaders and lights may be updated between renders (in
 * AUR_MODE_PATH_MIS the next render rebuilds the light-selection tables of
 * scenes whose shaders changed), but the batch is sized for the light
 * samples per hit at creation (AUR_MODE_PATH_MIS: two per area-light sample
 * plus one, at most 32 in all): a render after lights gained samples stops,
 * and aur_batch_status reports AUR_ERR_INVALID. */
aur_status aur_batch_create(aur_ctx* ctx, const aur_scene* const* scenes, const aur_camera* cameras,
                            const aur_render_params* params, uint32_t num_scenes,
                            const aur_wavefront_tuning* tuning, aur_batch** out);
/* Adds every scene's samples into accum[i] (device float4 frames) with one
 * graph launch on the context's stream. */
aur_status aur_batch_render(aur_ctx* ctx, aur_batch* batch, float* const* accum);
/* Waits for the batch and reports device-side failures (iteration limit or
 * stack overflow: AUR_ERR_TIMEOUT). iterations: total integrator iterations. */
aur_status aur_batch_status(aur_ctx* ctx, aur_batch* batch, uint32_t* iterations);
aur_status aur_batch_tuning(const aur_batch* batch, aur_wavefront_tuning* out);
/* Work counters of the last render: counters[0] = closest-hit rays (path
 * segments), counters[1] = shadow rays, counters[2] = integrator iterations. */
aur_status aur_batch_counters(aur_ctx* ctx, aur_batch* batch, unsigned long long counters[3]);
/* Profiling form of aur_batch_render: the same kernels launched one by one
 * without the graph, with per-stage CUDA-event times (ms) in stage_ms:
 * set-up, generate, extend, shade, shadow, combine, accumulate. */
aur_status aur_batch_profile(aur_ctx* ctx, aur_batch* batch, float* const* accum, float stage_ms[7]);
aur_status aur_batch_destroy(aur_batch* batch);
/* Autotuner: times renders of the batch's first two samples (one if it
 * renders one) for a set of candidate tunings (pool size, block size, blocks
 * per SM) and returns the fastest, preferring the largest pool among the
 * candidates within 3 % of the fastest (longer renders run fewer, fuller
 * iterations with it); pools above 4x the probe's paths are not timed.
 * best_ms: the pick's probe time. */
aur_status aur_batch_autotune(aur_ctx* ctx, const aur_scene* const* scenes, const aur_camera* cameras,
                              const aur_render_params* params, uint32_t num_scenes,
                              aur_wavefront_tuning* best, float* best_ms);

#ifdef __cplusplus
}
#endif

#endif /* AURORA_GB300_H */
