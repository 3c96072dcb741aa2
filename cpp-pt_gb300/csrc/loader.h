// Scene files in the reference's formats (Loader, src/loader/loader.h:20-374):
// render settings, .ptscene, .ptobj meshes (with the .gbbin cache) and
// .ptmat materials with their image textures.
#pragma once
#include <string>
#include <unordered_map>
#include <vector>

#include "host_internal.h"

namespace cpppt_gb300 {
namespace hostimpl {

struct LoadedScene {
    std::vector<float> v, n, t;
    std::vector<int32_t> tri, tri_mat;
    std::vector<pt_material> mats;
    pt_camera cam{};
    bool has_camera = false;
    SceneTextures tx;                                // uv, image textures, material slots
    std::unordered_map<std::string, int> tex_cache;  // path | rgb | srgb -> texture id
};

// Reads a render-settings file and the scene files it names into L;
// rs receives the render parameters (spp = N * N for `spp N`), output the
// output name.  Throws Fail(PT_ERR_IO, ...) on unreadable or malformed files.
void load_files(const std::string& settings_file, LoadedScene& L, pt_render_desc* rs, std::string& output);

// Turns reading and writing of the .gbbin mesh cache on or off.
void set_mesh_cache(bool enabled);

}  // namespace hostimpl
}  // namespace cpppt_gb300
