// aurora.h — Maya-free C++ host layer over the aurora_gb300 C ABI.
//
// Mirrors the reference's host classes on this path with the same names,
// argument meaning and error behaviour, minus Maya: Geometry
// (data/geometry.h), Scene (core/scene.h), Renderer and MonteCarloRaytracer
// (core/renderer.h, render/monteCarloRaytracer.h). Maya's MStatus becomes
// Aurora::Status, MDagPath cameras become aur_camera, RV_PIXEL framebuffers
// become RGBA float4. The scene comes from host arrays (or a scene file)
// instead of Maya's dependency graph. All device work goes through the C ABI;
// this layer has no CUDA code of its own.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "aurora_gb300.h"

namespace Aurora {

enum class Status { Success, Failure, InsufficientMemory, InvalidParameter };

// The process-wide library context (Engine::initialize, core/engine.cpp:33-47).
Status initialize(int device = 0);
aur_ctx* context();
void shutdown();
// Message of the last failing call on this thread.
std::string lastError();

// util/math.h:283-313
struct Rect {
    unsigned int left = 0, right = 0, bottom = 0, top = 0;
    Rect() = default;
    Rect(unsigned int l, unsigned int r, unsigned int b, unsigned int t) : left(l), right(r), bottom(b), top(t) {}
};

struct Dim {
    unsigned int width = 0, height = 0, depth = 1;
    Dim() = default;
    Dim(unsigned int w, unsigned int h = 1, unsigned int d = 1) : width(w), height(h), depth(d) {}
};

// data/geometry.h:13-55. Device (AllocDefault) or pinned host (AllocStaging)
// triangle soup in the reference layout; rebuild() replaces it by its NMH
// order and keeps the NMH for traversal.
class Geometry {
public:
    enum GeometryAllocMode { AllocEmpty = 0, AllocDefault, AllocStaging };

    float* vertices;
    float* normals;
    float* texcoords;
    unsigned short* shaders;
    float* tangents;
    float* bitangents;
    unsigned int count;
    GeometryAllocMode mode;
    aur_nmh* nmh;

    void initialize();
    bool resize(const unsigned int n, GeometryAllocMode allocMode);
    void free();

    bool copyToDevice(Geometry& other) const;
    bool copyToDeviceTransform(Geometry& other, const aur_object_transform* transforms,
                               const unsigned int objects) const;
    bool padToEven(const unsigned int n);

    bool rebuild();
    void generateTB();

    static const size_t TriangleSize = 9 * sizeof(float);
    static const size_t TriangleParams = 9;
    static const size_t TriangleUVSize = 6 * sizeof(float);
    static const size_t TriangleUVs = 6;
};

// An RGBA8 image (Texture, data/texture.h): width * height * 4 bytes, row 0 first.
struct TextureData {
    unsigned int width = 0, height = 0;
    std::vector<uint8_t> rgba;
};

// A scene in host memory: what Scene::update reads instead of Maya nodes.
struct SceneData {
    std::vector<float> vertices;        // count * 9, reference layout
    std::vector<float> normals;         // count * 9
    std::vector<uint16_t> shaderIds;    // count, 1-based
    std::vector<aur_shader> shaders;
    std::vector<aur_light> lights;
    std::vector<float> texcoords;       // count * 6 (u1 v1 u2 v2 u3 v3), with textures
    std::vector<TextureData> textures;  // shader.texture t selects textures[t - 1]
    aur_camera camera{};
    unsigned int count() const { return (unsigned int)(vertices.size() / 9); }
};

// Reads the binary scene file written by aurora_gb300.scenes.write_scene_file.
Status loadSceneFile(const std::string& path, SceneData& out);

// core/scene.h:25-58 without Maya: update() uploads the meshes, shaders and
// lights and builds the NMH (Scene::update(UpdateFull), core/scene.cpp:457-508).
class Scene {
public:
    Scene() = default;
    ~Scene();
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;

    Status update(const SceneData& data);
    void free();

    const aur_scene* handle() const { return m_scene; }
    const std::vector<aur_shader>& shaders() const { return m_shaders; }
    const std::vector<aur_light>& lights() const { return m_lights; }
    unsigned int triangles() const { return m_count; }

protected:
    aur_scene* m_scene = nullptr;
    std::vector<aur_shader> m_shaders;
    std::vector<aur_light> m_lights;
    unsigned int m_count = 0;
};

// core/renderer.h:21-42
class Renderer {
public:
    virtual ~Renderer() {}
    virtual Status createFrame(const unsigned int width, const unsigned int height, const unsigned short samples,
                               Scene* scene, const aur_camera& camera) = 0;
    virtual Status destroyFrame() = 0;
    virtual Status setRegion(const Rect& region) = 0;
    virtual Status update() { return Status::Success; }
    virtual Status render(bool ipr) = 0;
    virtual const float* framebuffer() = 0;

protected:
    static Status generateRays(const aur_camera& camera, const Dim& size, const unsigned short sampleID,
                               aur_path_ray* rays, aur_hitpoint* hit);
    static Status clearPixels(const Dim& size, void* pixels);
    static Status drawPixels(const Dim& size, const aur_hitpoint* hit, const float weight, void* pixels);
    // Renderer::filterPixels (core/renderer.cpp): filters `region` of *pixels
    // into a new buffer (other pixels zero), frees the old one and swaps.
    static Status filterPixels(const Dim& size, const Rect& region, float** pixels);
};

// render/monteCarloRaytracer.h:14-39 with the render loop of
// render/monteCarloRaytracer.cpp:81-120 (65,536-ray tiles per sample).
// render(false) clears and renders every sample of the frame. render(true),
// the interactive (IPR) call, adds the next single sample pass to the frame
// without clearing (starting over once all samples are in), and framebuffer()
// then returns the frame normalised by the samples done: a progressive image
// that after `samples` calls equals render(false)'s bit for bit.
class MonteCarloRaytracer : public Renderer {
public:
    MonteCarloRaytracer();
    ~MonteCarloRaytracer() override;

    Status createFrame(const unsigned int width, const unsigned int height, const unsigned short samples, Scene* scene,
                       const aur_camera& camera) override;
    Status destroyFrame() override;
    Status setRegion(const Rect& region) override;
    Status render(bool ipr) override;
    const float* framebuffer() override;

    // Integrator settings the reference fixes at compile time (MAX_DEPTH) or
    // seeds from GetTickCount(); AUR_MODE_REFERENCE reproduces it.
    void setIntegrator(unsigned int maxDepth, unsigned int seed, unsigned int mode);
    // Applies filterPixels after each complete render (the reference's call
    // is commented out, monteCarloRaytracer.cpp:117).
    void setFilter(bool on) { m_filter = on; }
    // Samples accumulated so far in the frame (progressive rendering).
    unsigned int samplesDone() const { return m_done; }

    static const unsigned int TileSize = 256 * 256;

protected:
    float* m_pixels;
    Scene* m_scene;
    aur_camera m_camera;
    aur_path_ray* m_rays;
    aur_hitpoint* m_hit;
    std::vector<float> m_framebuffer;
    Rect m_region;
    Dim m_size;
    unsigned int m_maxDepth, m_seed, m_mode;
    unsigned int m_done = 0;
    bool m_filter = false;
};

}  // namespace Aurora
