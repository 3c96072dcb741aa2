/*
 * pathtracer_gb300.h -- the GB300 path tracer as a renderer of drcd1/cpp-pt.
 *
 * Reference-side adapter: a maintainer of the reference copies this header
 * into the reference tree (next to src/renderer/pathtracerMIS.h) and adds one
 * branch to main()'s renderer chain (src/main.cpp:104-125).  It derives from
 * the reference's `class Renderer { virtual void render(Scene&, std::string)
 * = 0; }` (src/renderer/renderer.h:30-33) and therefore needs the reference's
 * headers before it; it calls the library only through the C ABI of
 * cpppt_gb300.h and links libcpppt_gb300.so.
 *
 * The reference's BVH triangle list and StandardMaterial textures are
 * private (bvh.h:51-54, standard_material.h:13-21), so the adapter reads the
 * same settings and scene files with the library's loader (pt_scene_load,
 * which follows Loader::load_render_settings / Loader::load_scene,
 * loader.h:256-374) instead of walking the Scene it is handed.  It renders
 * spp x spp samples per pixel, 32 bounces, Russian roulette from bounce 3
 * (pathtracerMIS.h:36, 118, 133) and writes <filename>.png and
 * <filename>.hdr like Image::save (rgb_image.h:300-318).  Failures throw
 * std::runtime_error, which main() catches (main.cpp:143-145).
 */
#ifndef CPPPT_PATHTRACER_GB300_H
#define CPPPT_PATHTRACER_GB300_H

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cpppt_gb300.h"

namespace cpppt {

class PathtracerGB300 : public Renderer {
    std::string settings_file;

public:
    explicit PathtracerGB300(std::string settings) : settings_file(std::move(settings)) {}

    void render(Scene&, std::string filename) override {
        pt_scene* s = nullptr;
        pt_render_desc d;
        if (pt_scene_load(settings_file.c_str(), &s, &d, nullptr, 0) != PT_OK)
            throw std::runtime_error(pt_last_error());
        int32_t w = 0, h = 0;
        pt_status st = pt_scene_info(s, &w, &h, nullptr, nullptr);
        std::vector<float> rgb(3 * (size_t)w * (size_t)h);
        if (st == PT_OK) st = pt_render(s, &d, rgb.data());
        if (st == PT_OK) st = pt_image_save(filename.c_str(), rgb.data(), w, h);
        pt_scene_destroy(s);
        if (st != PT_OK) throw std::runtime_error(pt_last_error());
    }
};

}  // namespace cpppt

#endif
