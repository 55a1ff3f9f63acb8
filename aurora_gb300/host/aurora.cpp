// aurora.cpp — the Maya-free host layer (see aurora.h).
#include "aurora.h"

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace Aurora {

namespace {
aur_ctx* g_ctx = nullptr;
thread_local std::string g_message;

Status status_of(aur_status s) {
    if (s == AUR_OK) return Status::Success;
    g_message = aur_last_error();
    if (s == AUR_ERR_OOM) return Status::InsufficientMemory;
    if (s == AUR_ERR_INVALID) return Status::InvalidParameter;
    return Status::Failure;
}

bool ok(aur_status s) { return status_of(s) == Status::Success; }
}  // namespace

Status initialize(int device) {
    if (g_ctx) return Status::Success;
    return status_of(aur_ctx_create(device, &g_ctx));
}

aur_ctx* context() {
    if (!g_ctx) initialize(0);
    return g_ctx;
}

void shutdown() {
    aur_ctx_destroy(g_ctx);
    g_ctx = nullptr;
}

std::string lastError() { return g_message; }

// ------------------------------------------------------------- Geometry
// data/geometry.cpp:12-186

void Geometry::initialize() {
    count = 0;
    mode = AllocEmpty;
    vertices = normals = texcoords = tangents = bitangents = nullptr;
    shaders = nullptr;
    nmh = nullptr;
}

bool Geometry::resize(const unsigned int n, GeometryAllocMode allocMode) {
    const unsigned int n2 = n + (n % 2);   // even count (data/geometry.cpp:90)
    if (n2 == count && allocMode == mode) return true;
    free();
    if (allocMode == AllocEmpty) return true;
    const int policy = allocMode == AllocDefault ? AUR_DEVICE_MEMORY : AUR_PINNED_MEMORY;
    aur_ctx* c = context();
    if (!c) return false;
    bool good = ok(aur_malloc(c, n2 * TriangleSize, policy, (void**)&vertices)) &&
                ok(aur_malloc(c, n2 * TriangleSize, policy, (void**)&normals)) &&
                ok(aur_malloc(c, n2 * TriangleUVSize, policy, (void**)&texcoords)) &&
                ok(aur_malloc(c, n2 * sizeof(unsigned short), policy, (void**)&shaders));
    if (good && allocMode == AllocDefault)   // tangent frames only on the device, as the reference
        good = ok(aur_malloc(c, n2 * TriangleSize, policy, (void**)&tangents)) &&
               ok(aur_malloc(c, n2 * TriangleSize, policy, (void**)&bitangents));
    mode = allocMode;
    if (!good) {
        free();
        return false;
    }
    count = n2;
    return true;
}

void Geometry::free() {
    aur_ctx* c = g_ctx;
    if (c && mode != AllocEmpty) {
        const int policy = mode == AllocDefault ? AUR_DEVICE_MEMORY : AUR_PINNED_MEMORY;
        aur_free(c, vertices, policy);
        aur_free(c, normals, policy);
        aur_free(c, texcoords, policy);
        aur_free(c, shaders, policy);
        aur_free(c, tangents, policy);
        aur_free(c, bitangents, policy);
    }
    aur_nmh_destroy(nmh);
    initialize();
}

bool Geometry::copyToDevice(Geometry& dest) const {
    if (mode != AllocStaging || dest.mode != AllocDefault || dest.count != count) return false;
    aur_ctx* c = context();
    return ok(aur_memupload(c, dest.vertices, vertices, count * TriangleSize, AUR_DEVICE_MEMORY)) &&
           ok(aur_memupload(c, dest.normals, normals, count * TriangleSize, AUR_DEVICE_MEMORY)) &&
           ok(aur_memupload(c, dest.texcoords, texcoords, count * TriangleUVSize, AUR_DEVICE_MEMORY)) &&
           ok(aur_memupload(c, dest.shaders, shaders, count * sizeof(unsigned short), AUR_DEVICE_MEMORY));
}

bool Geometry::copyToDeviceTransform(Geometry& dest, const aur_object_transform* transforms,
                                     const unsigned int objects) const {
    if (mode != AllocStaging || dest.mode != AllocDefault || dest.count != count) return false;
    // stage the object-space soup on the device, then bake it (cudaTransform)
    Geometry tmp;
    tmp.initialize();
    if (!tmp.resize(count, AllocDefault) || !copyToDevice(tmp)) {
        tmp.free();
        return false;
    }
    aur_ctx* c = context();
    const bool good =
        ok(aur_transform(c, tmp.vertices, tmp.normals, count, transforms, objects, dest.vertices, dest.normals)) &&
        ok(aur_memupload(c, dest.texcoords, texcoords, count * TriangleUVSize, AUR_DEVICE_MEMORY)) &&
        ok(aur_memupload(c, dest.shaders, shaders, count * sizeof(unsigned short), AUR_DEVICE_MEMORY));
    tmp.free();
    return good;
}

bool Geometry::padToEven(const unsigned int n) {
    // The soup holds count = n + (n % 2) triangles; an odd n gets a copy of its
    // last triangle (data/geometry.cpp:164-176).
    if (count < 2 || mode != AllocStaging) return false;
    if (n % 2 == 0) return true;
    std::memcpy(vertices + (size_t)(count - 1) * TriangleParams, vertices + (size_t)(count - 2) * TriangleParams,
                TriangleSize);
    std::memcpy(normals + (size_t)(count - 1) * TriangleParams, normals + (size_t)(count - 2) * TriangleParams,
                TriangleSize);
    std::memcpy(texcoords + (size_t)(count - 1) * TriangleUVs, texcoords + (size_t)(count - 2) * TriangleUVs,
                TriangleUVSize);
    shaders[count - 1] = shaders[count - 2];
    return true;
}

bool Geometry::rebuild() {
    // cudaRebuildNMH (kernels/rebuilder.cu:311-450): build, then replace the
    // soup by its NMH-ordered copy (applyIndices for every attribute).
    if (mode != AllocDefault) return false;
    aur_ctx* c = context();
    aur_nmh* built = nullptr;
    if (!ok(aur_nmh_build(c, vertices, count, &built))) return false;
    Geometry result;
    result.initialize();
    if (!result.resize(count, AllocDefault)) {
        aur_nmh_destroy(built);
        return false;
    }
    const bool good = ok(aur_nmh_apply(c, built, vertices, (uint32_t)TriangleSize, result.vertices)) &&
                      ok(aur_nmh_apply(c, built, normals, (uint32_t)TriangleSize, result.normals)) &&
                      ok(aur_nmh_apply(c, built, texcoords, (uint32_t)TriangleUVSize, result.texcoords)) &&
                      ok(aur_nmh_apply(c, built, shaders, (uint32_t)sizeof(unsigned short), result.shaders)) &&
                      ok(aur_ctx_synchronize(c));
    if (!good) {
        result.free();
        aur_nmh_destroy(built);
        return false;
    }
    free();
    *this = result;
    nmh = built;
    return true;
}

void Geometry::generateTB() {
    if (mode == AllocDefault) ok(aur_generate_tb(context(), normals, count, tangents, bitangents));
}

// ---------------------------------------------------------------- scene

Status loadSceneFile(const std::string& path, SceneData& out) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        g_message = "cannot open scene file " + path;
        return Status::InvalidParameter;
    }
    char magic[8];
    uint32_t counts[4];
    bool good = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "AURSCN1", 8) == 0 &&
                std::fread(counts, 4, 4, f) == 4 && std::fread(&out.camera, sizeof(aur_camera), 1, f) == 1;
    uint32_t pad = 0;
    good = good && std::fread(&pad, 4, 1, f) == 1;
    if (good) {
        const size_t tri = counts[0];
        out.vertices.resize(tri * 9);
        out.normals.resize(tri * 9);
        out.shaderIds.resize(tri + (tri & 1));
        out.shaders.resize(counts[1]);
        out.lights.resize(counts[2]);
        good = std::fread(out.vertices.data(), 36, tri, f) == tri && std::fread(out.normals.data(), 36, tri, f) == tri &&
               std::fread(out.shaderIds.data(), 2, out.shaderIds.size(), f) == out.shaderIds.size() &&
               std::fread(out.shaders.data(), sizeof(aur_shader), counts[1], f) == counts[1] &&
               std::fread(out.lights.data(), sizeof(aur_light), counts[2], f) == counts[2];
        out.shaderIds.resize(tri);
        // optional: counts[3] textures, after the per-triangle texcoords
        if (good && counts[3]) {
            out.texcoords.resize(tri * 6);
            good = std::fread(out.texcoords.data(), 24, tri, f) == tri;
            out.textures.resize(counts[3]);
            for (uint32_t i = 0; good && i < counts[3]; ++i) {
                uint32_t wh[2];
                good = std::fread(wh, 4, 2, f) == 2 && wh[0] && wh[1] && (uint64_t)wh[0] * wh[1] < (1ull << 30);
                if (!good) break;
                TextureData& t = out.textures[i];
                t.width = wh[0];
                t.height = wh[1];
                t.rgba.resize((size_t)wh[0] * wh[1] * 4);
                good = std::fread(t.rgba.data(), 1, t.rgba.size(), f) == t.rgba.size();
            }
        }
    }
    std::fclose(f);
    if (!good) {
        g_message = "malformed scene file " + path;
        return Status::InvalidParameter;
    }
    return Status::Success;
}

Scene::~Scene() { free(); }

Status Scene::update(const SceneData& d) {
    free();
    const unsigned int n = d.count();
    if (d.normals.size() != d.vertices.size() || d.shaderIds.size() != n) {
        g_message = "Scene::update: vertex, normal and shader-id arrays disagree";
        return Status::InvalidParameter;
    }
    aur_ctx* c = context();
    if (!c) return Status::Failure;
    const Status s = status_of(aur_scene_create(c, d.vertices.data(), d.normals.data(), d.shaderIds.data(), n,
                                                d.shaders.data(), (uint32_t)d.shaders.size(), d.lights.data(),
                                                (uint32_t)d.lights.size(), &m_scene));
    if (s != Status::Success) return s;
    // Scene::updateTextures (core/scene.cpp:298-327)
    if (!d.textures.empty()) {
        if (d.texcoords.size() != (size_t)n * 6) {
            g_message = "Scene::update: textures need 6 texcoords per triangle";
            free();
            return Status::InvalidParameter;
        }
        std::vector<aur_texture> table(d.textures.size());
        for (size_t i = 0; i < table.size(); ++i) {
            table[i].width = d.textures[i].width;
            table[i].height = d.textures[i].height;
            table[i].rgba = d.textures[i].rgba.data();
        }
        const Status ts = status_of(aur_scene_set_textures(c, m_scene, d.texcoords.data(), table.data(),
                                                           (uint32_t)table.size()));
        if (ts != Status::Success) {
            free();
            return ts;
        }
    }
    m_shaders = d.shaders;
    m_lights = d.lights;
    m_count = n;
    return Status::Success;
}

void Scene::free() {
    aur_scene_destroy(m_scene);
    m_scene = nullptr;
    m_shaders.clear();
    m_lights.clear();
    m_count = 0;
}

// ------------------------------------------------------------- renderer
// core/renderer.cpp:14-55

Status Renderer::generateRays(const aur_camera& camera, const Dim& size, const unsigned short sampleID,
                              aur_path_ray* rays, aur_hitpoint* hit) {
    return status_of(aur_generate_rays(context(), size.width, size.height, sampleID, size.depth, &camera, rays, hit));
}

Status Renderer::clearPixels(const Dim& size, void* pixels) {
    return status_of(aur_clear_pixels(context(), size.width, size.height, (float*)pixels));
}

Status Renderer::drawPixels(const Dim& size, const aur_hitpoint* hit, const float weight, void* pixels) {
    return status_of(aur_draw_pixels(context(), size.width, size.height, weight, hit, (float*)pixels));
}

// render/monteCarloRaytracer.cpp
MonteCarloRaytracer::MonteCarloRaytracer()
    : m_pixels(nullptr), m_scene(nullptr), m_camera{}, m_rays(nullptr), m_hit(nullptr), m_maxDepth(8), m_seed(0),
      m_mode(AUR_MODE_REFERENCE) {}

MonteCarloRaytracer::~MonteCarloRaytracer() { destroyFrame(); }

void MonteCarloRaytracer::setIntegrator(unsigned int maxDepth, unsigned int seed, unsigned int mode) {
    m_maxDepth = maxDepth;
    m_seed = seed;
    m_mode = mode;
}

Status MonteCarloRaytracer::createFrame(const unsigned int width, const unsigned int height,
                                        const unsigned short samples, Scene* scene, const aur_camera& camera) {
    destroyFrame();
    if (!scene || !scene->handle() || width == 0 || height == 0 || samples == 0) {
        g_message = "createFrame: no scene, or an empty frame";
        return Status::InvalidParameter;
    }
    aur_ctx* c = context();
    const size_t numRays = (size_t)width * height;
    if (!ok(aur_malloc(c, sizeof(aur_path_ray) * numRays, AUR_DEVICE_MEMORY, (void**)&m_rays)) ||
        !ok(aur_malloc(c, sizeof(aur_hitpoint) * numRays, AUR_DEVICE_MEMORY, (void**)&m_hit)) ||
        !ok(aur_malloc(c, 4 * sizeof(float) * numRays, AUR_DEVICE_MEMORY, (void**)&m_pixels))) {
        destroyFrame();
        return Status::InsufficientMemory;   // monteCarloRaytracer.cpp:28-46
    }
    m_framebuffer.assign(numRays * 4, 0.0f);
    m_scene = scene;
    m_camera = camera;
    m_region = Rect(0, width - 1, 0, height - 1);
    m_size = Dim(width, height, samples);
    return Status::Success;
}

Status MonteCarloRaytracer::destroyFrame() {
    aur_ctx* c = g_ctx;
    if (c) {
        aur_free(c, m_rays, AUR_DEVICE_MEMORY);
        aur_free(c, m_hit, AUR_DEVICE_MEMORY);
        aur_free(c, m_pixels, AUR_DEVICE_MEMORY);
    }
    m_rays = nullptr;
    m_hit = nullptr;
    m_pixels = nullptr;
    m_framebuffer.clear();
    return Status::Success;
}

Status MonteCarloRaytracer::setRegion(const Rect& region) {
    // The ray and pixel kernels cover the whole frame.
    if (region.left != 0 || region.bottom != 0 || region.right + 1 != m_size.width ||
        region.top + 1 != m_size.height) {
        g_message = "setRegion: only the full frame is supported";
        return Status::InvalidParameter;
    }
    m_region = region;
    return Status::Success;
}

Status MonteCarloRaytracer::render(bool ipr) {
    if (!m_pixels || !m_scene) return Status::Failure;
    const float weight = 1.0f / m_size.depth;
    const unsigned int numRays = m_size.width * m_size.height;
    const unsigned int numTiles = (numRays / TileSize) + ((numRays % TileSize) > 0);
    aur_render_params p{};
    p.width = m_size.width;
    p.height = m_size.height;
    p.spp = m_size.depth;
    p.max_depth = m_maxDepth;
    p.seed = m_seed;
    p.mode = m_mode;
    Status s;
    if (!ipr || m_done == 0 || m_done >= m_size.depth) {
        if ((s = clearPixels(m_size, m_pixels)) != Status::Success) return s;
        m_done = 0;
    }
    const unsigned int first = ipr ? m_done : 0u, last = ipr ? m_done + 1 : (unsigned int)m_size.depth;
    for (unsigned int i = first; i < last; i++) {
        if ((s = generateRays(m_camera, m_size, (unsigned short)i, m_rays, m_hit)) != Status::Success) return s;
        for (unsigned int j = 0; j < numTiles; j++) {
            const unsigned int offset = j * TileSize;
            const unsigned int numTileRays = std::min(numRays - offset, TileSize);
            s = status_of(aur_raytrace_monte_carlo(context(), m_scene->handle(), &p, i, offset, numTileRays, m_rays,
                                                   m_hit));
            if (s != Status::Success) return s;
        }
        if ((s = drawPixels(m_size, m_hit, weight, m_pixels)) != Status::Success) return s;
    }
    m_done = last;
    if (m_filter && m_done == m_size.depth)
        if ((s = filterPixels(m_size, m_region, &m_pixels)) != Status::Success) return s;
    return status_of(aur_ctx_synchronize(context()));
}

const float* MonteCarloRaytracer::framebuffer() {
    if (!m_pixels) return nullptr;
    if (!ok(aur_memdownload(context(), m_framebuffer.data(), m_pixels, m_framebuffer.size() * sizeof(float))))
        return nullptr;
    if (m_done > 0 && m_done < m_size.depth) {   // progressive: normalise by the samples done
        const float scale = (float)m_size.depth / (float)m_done;
        for (float& v : m_framebuffer) v *= scale;
    }
    return m_framebuffer.data();
}

Status Renderer::filterPixels(const Dim& size, const Rect& region, float** pixels) {
    aur_ctx* c = context();
    const size_t bytes = (size_t)size.width * size.height * 4 * sizeof(float);
    float* out = nullptr;
    if (!ok(aur_malloc(c, bytes, AUR_DEVICE_MEMORY, (void**)&out))) return Status::InsufficientMemory;
    const aur_rect r{region.left, region.right, region.bottom, region.top};
    if (!ok(aur_memzero(c, out, bytes, AUR_DEVICE_MEMORY)) ||
        !ok(aur_filter_pixels(c, size.width, size.height, &r, *pixels, out))) {
        aur_free(c, out, AUR_DEVICE_MEMORY);
        return Status::Failure;
    }
    if (!ok(aur_ctx_synchronize(c))) {
        aur_free(c, out, AUR_DEVICE_MEMORY);
        return Status::Failure;
    }
    aur_free(c, *pixels, AUR_DEVICE_MEMORY);
    *pixels = out;
    return Status::Success;
}

}  // namespace Aurora
