// Test harness: the reference's main() flow (src/main.cpp:88-142) with the
// GB300 renderer of include/pathtracer_gb300.h selected, compiled against the
// reference's own headers (the copy oracle/build_ref.sh makes) and linked
// with libcpppt_gb300.so.  tests/test_adapter.py builds and runs it.
#include <chrono>
#include <cmath>
#include <fstream>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>

// settings read by the harness patches of the reference copy (bounce limit,
// replica seed offset, progress output)
int cpppt_harness_max_depth = 32;
int cpppt_harness_seed_offset = 0;
int cpppt_harness_verbose = 0;

// the headers the reference's main.cpp includes before its loader (main.cpp:1-31)
#include <camera/camera_perspective.h>
#include <renderer/pathtracerMIS.h>
#include <primitive/bvh.h>
#include <shape/mesh.h>
#include <shape/triangle.h>
#include <primitive/primitive_leaf.h>
#include <bxdf/diffuse_bxdf.h>
#include <bxdf/emissive_bxdf.h>
#include <texture/constant_texture.h>
#include <light/light.h>
#include <light/point_light.h>
#include <light/shape_light.h>
#include <light/light_group.h>
#include <loader/loader.h>
#include <scene.h>

#include "pathtracer_gb300.h"

using namespace cpppt;

int main(int argc, char** argv) {
    try {
        if (argc < 2) {
            std::cout << "Insuficient Arguments" << std::endl;
            return 2;
        }
        RenderSettings rs;
        Scene s;
        SceneData sd;
        Loader::load_render_settings(&rs, argv[1]);
        Loader::load_scene(&s, &sd, &rs, rs.scene_name);
        std::unique_ptr<Renderer> renderer = std::make_unique<PathtracerGB300>(argv[1]);
        auto t1 = std::chrono::high_resolution_clock::now();
        renderer->render(s, rs.output_name);
        auto t2 = std::chrono::high_resolution_clock::now();
        std::chrono::duration<double, std::milli> ms = t2 - t1;
        std::cout << ms.count() * 0.001 << "s\n";
        return 0;
    } catch (std::runtime_error& e) {
        std::cout << e.what() << std::endl;
        return 1;
    }
}
