// C++ host interface mirroring the reference's renderer API on top of the C ABI.
//
// The reference selects a Renderer from RenderSettings (src/main.cpp:104-125)
// and calls `render(Scene&, std::string filename)` (src/renderer/renderer.h:30-33),
// which writes <filename>.png and <filename>.hdr (src/image/rgb_image.h:300-318).
// GpuPathtracerMIS is that renderer for `renderer pathtracer_mis`
// (src/renderer/pathtracerMIS.h:17-168), executed on the GPU.  Errors surface
// as std::runtime_error, as the reference's loader and renderers report them
// (caught in main, src/main.cpp:143-145).
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/cpppt_gb300.h"

namespace cpppt_gb300 {

// RenderSettings (src/renderer/renderer.h:11-28): `spp` keeps the reference's
// meaning (spp x spp samples per pixel).
struct RenderSettings {
    int spp = 1;
    int resX = 256;
    int resY = 256;
    std::string scene_name;
    std::string output_name;
    int max_depth = 32;  // pathtracerMIS.h:36
    int rr_start = 3;    // pathtracerMIS.h:118 (i > 2)
    unsigned seed = 0;
    int mode = PT_MODE_MIS;
};

inline void check(pt_status s) {
    if (s != PT_OK) throw std::runtime_error(pt_last_error());
}

// Owns a pt_scene: the scene and its GPU copy.
class Scene {
public:
    Scene() = default;
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;
    ~Scene() { pt_scene_destroy(handle_); }

    // Loader::load_render_settings + Loader::load_scene (src/loader/loader.h:256-374)
    void load(RenderSettings* rs, const std::string& settings_file) {
        pt_render_desc d{};
        char out[4096] = {0};
        pt_scene* h = nullptr;
        check(pt_scene_load(settings_file.c_str(), &h, &d, out, sizeof(out)));
        pt_scene_destroy(handle_);
        handle_ = h;
        int axis = 1;
        while ((axis + 1) * (axis + 1) <= d.spp) axis++;
        rs->spp = axis;
        rs->output_name = out;
        check(pt_scene_info(handle_, &rs->resX, &rs->resY, nullptr, nullptr));
    }

    void create(const pt_scene_desc& desc) {
        pt_scene* h = nullptr;
        check(pt_scene_create(&desc, &h));
        pt_scene_destroy(handle_);
        handle_ = h;
    }

    pt_scene* handle() const { return handle_; }

private:
    pt_scene* handle_ = nullptr;
};

class Renderer {
public:
    virtual ~Renderer() = default;
    virtual void render(Scene& sc, std::string filename) = 0;
};

class GpuPathtracerMIS : public Renderer {
public:
    explicit GpuPathtracerMIS(const RenderSettings& rs) : rs_(rs) {}

    // Renders spp x spp samples per pixel; writes <filename>.png / .hdr
    // unless filename is empty.  The float image stays available in image().
    void render(Scene& sc, std::string filename) override {
        int32_t w = 0, h = 0;
        check(pt_scene_info(sc.handle(), &w, &h, nullptr, nullptr));
        pt_render_desc d{};
        d.spp = rs_.spp * rs_.spp;
        d.max_depth = rs_.max_depth;
        d.rr_start = rs_.rr_start;
        d.seed = rs_.seed;
        d.mode = rs_.mode;
        image_.assign(3 * (size_t)w * h, 0.0f);
        check(pt_render(sc.handle(), &d, image_.data()));
        width_ = w;
        height_ = h;
        if (!filename.empty()) check(pt_image_save(filename.c_str(), image_.data(), w, h));
    }

    const std::vector<float>& image() const { return image_; }
    int width() const { return width_; }
    int height() const { return height_; }

private:
    RenderSettings rs_;
    std::vector<float> image_;
    int width_ = 0, height_ = 0;
};

}  // namespace cpppt_gb300
