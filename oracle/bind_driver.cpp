// Driver for the reference renderer built with the GPU integrator that INTEGRATION.md shows
// registered in its factory (oracle/build_binding.py compiles it into oracle/_ref/bind/libc2bind.so).
//
// TEST INFRASTRUCTURE ONLY.  It runs the reference's own front end the way RayTracer's constructor
// and TraceAsync do (src/Core/RayTracer.cpp:11-43): JsonLoader + ConfigLoader, Scene::CreateScene,
// Camera::CreateCamera, Integrator::LoadIntegrator (with the "GPUPathTracer" branch added), then
// Integrator::Render into a reference FrameBuffer and FrameBuffer::GetImageDataRGB32F.
#include <cstdio>
#include <exception>
#include <memory>
#include <string>

#define STB_IMAGE_IMPLEMENTATION
#include <stbi/stb_image.h>

#include <Crystal2.h>
#include <Cameras/Camera.h>
#include <Core/FrameBuffer.h>
#include <Core/Scene.h>
#include <Integrators/GPUPathTracingIntegrator.h>
#include <Integrators/Integrator.h>
#include <Loaders/ConfigLoader.h>
#include <Loaders/JsonLoader.h>
#include <SJson/SJson.h>

extern "C" {

// Renders the scene through the reference's Integrator::Render with the integrator its config
// names; rgb receives GetImageDataRGB32F (rows flipped, width x height x 3).  Returns 0 on success,
// 1 with the exception text in err otherwise.
int bind_render(const char* cfg_path, const char* scene_path, float* rgb, int cap, int* width, int* height, char* err,
                int errlen) {
    try {
        auto cfgNode = loader::JsonLoader::LoadJsonFile(cfg_path);
        auto sceneNode = loader::JsonLoader::LoadJsonFile(scene_path);
        auto info = config::ConfigLoader::LoadConfigInfo(cfgNode);
        auto scene = Scene::CreateScene(sceneNode->GetMember("Scene"), info);
        auto camera = Camera::CreateCamera(sceneNode->GetMember("Camera"), info);
        // what main() does before building the engine (the integrator parses the same two files)
        crystal::GPUPathTracingIntegrator::ConfigPath = cfg_path;
        crystal::GPUPathTracingIntegrator::ScenePath = scene_path;
        auto integrator = crystal::Integrator::LoadIntegrator(cfgNode.get(), info);
        FrameBuffer fb(info.Width, info.Height);
        fb.Clear();
        integrator->Render(scene.get(), camera.get(), &fb);
        *width = fb.Width();
        *height = fb.Height();
        const int n = 3 * fb.Width() * fb.Height();
        if (n > cap) throw std::runtime_error("output buffer too small");
        auto img = fb.GetImageDataRGB32F();
        for (int i = 0; i < n; i++) rgb[i] = img[i];
        return 0;
    } catch (const std::exception& e) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", e.what());
    } catch (...) {
        if (err && errlen > 0) std::snprintf(err, errlen, "unknown exception");
    }
    return 1;
}

}  // extern "C"
