// aurora_render — standalone renderer driver in place of the Maya plug-in
// (src/maya/renderCommand.cpp, core/engine.cpp:171-251).
//
//   aurora_render SCENE.bin OUT.pfm [--width W] [--height H] [--spp S]
//                 [--depth D] [--seed N] [--mode reference|path|mis] [--device K]
//                 [--filter] [--progressive]
//   aurora_render SCENE.bin --dry-run          parse the scene file only
//   aurora_render SCENE.bin --geometry-check   Geometry upload + rebuild + TB
//
// Renders with MonteCarloRaytracer (the reference's per-sample, per-tile
// loop) and writes an RGB PFM (bottom row first, as y = 0 is the bottom row of
// the frame). Prints one JSON line.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "aurora.h"

using namespace Aurora;

static uint64_t fnv1a(const void* data, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) { h ^= p[i]; h *= 1099511628211ull; }
    return h;
}

static int fail(const char* what) {
    std::fprintf(stderr, "aurora_render: %s: %s\n", what, lastError().c_str());
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: aurora_render SCENE.bin OUT.pfm [--width W] [--height H] [--spp S] [--depth D] "
                             "[--seed N] [--mode reference|path|mis] [--device K] | --dry-run | --geometry-check\n");
        return 2;
    }
    std::string scenePath = argv[1], outPath;
    unsigned width = 256, height = 256, spp = 16, depth = 4, seed = 0, mode = AUR_MODE_PATH;
    int device = 0;
    bool dry = false, geomCheck = false, filter = false, progressive = false;
    for (int i = 2; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() { return (i + 1 < argc) ? std::strtoul(argv[++i], nullptr, 10) : 0ul; };
        if (a == "--width") width = (unsigned)next();
        else if (a == "--height") height = (unsigned)next();
        else if (a == "--spp") spp = (unsigned)next();
        else if (a == "--depth") depth = (unsigned)next();
        else if (a == "--seed") seed = (unsigned)next();
        else if (a == "--device") device = (int)next();
        else if (a == "--mode") {
            const std::string m = i + 1 < argc ? argv[++i] : "";
            mode = m == "reference" ? AUR_MODE_REFERENCE : (m == "mis" ? AUR_MODE_PATH_MIS : AUR_MODE_PATH);
        }
        else if (a == "--dry-run") dry = true;
        else if (a == "--geometry-check") geomCheck = true;
        else if (a == "--filter") filter = true;
        else if (a == "--progressive") progressive = true;
        else if (outPath.empty()) outPath = a;
        else { std::fprintf(stderr, "aurora_render: unknown argument %s\n", a.c_str()); return 2; }
    }
    SceneData data;
    if (loadSceneFile(scenePath, data) != Status::Success) return fail("loading the scene");
    if (dry) {
        std::printf("{\"triangles\": %u, \"shaders\": %zu, \"lights\": %zu, \"textures\": %zu, "
                    "\"vertex_checksum\": %llu}\n",
                    data.count(), data.shaders.size(), data.lights.size(), data.textures.size(),
                    (unsigned long long)fnv1a(data.vertices.data(), data.vertices.size() * sizeof(float)));
        return 0;
    }
    if (initialize(device) != Status::Success) return fail("initializing the device");
    if (geomCheck) {
        // Scene::updateMeshes without Maya: staging soup -> device -> rebuild -> TB
        const unsigned n = data.count();
        Geometry staging, geom;
        staging.initialize();
        geom.initialize();
        if (!staging.resize(n, Geometry::AllocStaging) || !geom.resize(n, Geometry::AllocDefault))
            return fail("allocating geometry");
        std::memcpy(staging.vertices, data.vertices.data(), (size_t)n * Geometry::TriangleSize);
        std::memcpy(staging.normals, data.normals.data(), (size_t)n * Geometry::TriangleSize);
        std::memset(staging.texcoords, 0, (size_t)staging.count * Geometry::TriangleUVSize);
        std::memcpy(staging.shaders, data.shaderIds.data(), (size_t)n * sizeof(unsigned short));
        if (!staging.padToEven(n) || !staging.copyToDevice(geom) || !geom.rebuild()) return fail("rebuilding");
        geom.generateTB();
        std::vector<float> v((size_t)geom.count * 9), tb((size_t)geom.count * 9);
        std::vector<uint32_t> perm(geom.count);
        uint32_t levels = 0, cnt = 0;
        aur_nmh_info(geom.nmh, &cnt, &levels);
        if (aur_memdownload(context(), v.data(), geom.vertices, v.size() * 4) != AUR_OK ||
            aur_memdownload(context(), tb.data(), geom.tangents, tb.size() * 4) != AUR_OK ||
            aur_nmh_export(context(), geom.nmh, perm.data(), nullptr) != AUR_OK)
            return fail("downloading");
        std::printf("{\"count\": %u, \"levels\": %u, \"perm_checksum\": %llu, \"vertex_checksum\": %llu, "
                    "\"tangent_checksum\": %llu}\n",
                    geom.count, levels, (unsigned long long)fnv1a(perm.data(), perm.size() * 4),
                    (unsigned long long)fnv1a(v.data(), v.size() * 4), (unsigned long long)fnv1a(tb.data(), tb.size() * 4));
        staging.free();
        geom.free();
        shutdown();
        return 0;
    }
    if (outPath.empty()) { std::fprintf(stderr, "aurora_render: no output path\n"); return 2; }
    Scene scene;
    if (scene.update(data) != Status::Success) return fail("updating the scene");
    MonteCarloRaytracer renderer;
    renderer.setIntegrator(depth, seed, mode);
    renderer.setFilter(filter);
    if (renderer.createFrame(width, height, (unsigned short)spp, &scene, data.camera) != Status::Success)
        return fail("creating the frame");
    const auto t0 = std::chrono::steady_clock::now();
    if (progressive) {   // the interactive loop: one sample pass per call
        for (unsigned int k = 0; k < spp; ++k)
            if (renderer.render(true) != Status::Success) return fail("rendering");
    } else if (renderer.render(false) != Status::Success) {
        return fail("rendering");
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    const float* fb = renderer.framebuffer();
    if (!fb) return fail("reading the framebuffer");
    FILE* f = std::fopen(outPath.c_str(), "wb");
    if (!f) { std::fprintf(stderr, "aurora_render: cannot write %s\n", outPath.c_str()); return 1; }
    std::fprintf(f, "PF\n%u %u\n-1.0\n", width, height);
    for (size_t p = 0; p < (size_t)width * height; ++p) std::fwrite(fb + 4 * p, sizeof(float), 3, f);
    std::fclose(f);
    std::printf("{\"width\": %u, \"height\": %u, \"spp\": %u, \"render_ms\": %.3f, \"samples_per_s\": %.1f, "
                "\"image_checksum\": %llu}\n",
                width, height, spp, ms, (double)width * height * spp / (ms * 1e-3),
                (unsigned long long)fnv1a(fb, (size_t)width * height * 16));
    renderer.destroyFrame();
    scene.free();
    shutdown();
    return 0;
}
