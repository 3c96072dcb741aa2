// Command-line renderer with the reference's interface (src/main.cpp:89-146):
//   cpppt_render <settings file>
// reads the settings and scene files, renders with GpuPathtracerMIS and
// writes <output>.png / <output>.hdr.  Prints the render time in seconds,
// measured around render() as main.cpp:130-142 does.
#include <chrono>
#include <iostream>

#include "gpu_pathtracer.h"

int main(int argc, char** argv) {
    using namespace cpppt_gb300;
    try {
        if (argc < 2) {
            std::cout << "Insuficient Arguments" << std::endl;
            return 0;
        }
        RenderSettings rs;
        Scene s;
        s.load(&rs, argv[1]);
        if (argc >= 3) rs.max_depth = std::atoi(argv[2]);
        GpuPathtracerMIS renderer(rs);
        auto t1 = std::chrono::high_resolution_clock::now();
        renderer.render(s, rs.output_name);
        auto t2 = std::chrono::high_resolution_clock::now();
        std::chrono::duration<double, std::milli> ms = t2 - t1;
        std::cout << ms.count() * 0.001 << "s\n";
    } catch (const std::runtime_error& e) {
        std::cout << e.what() << std::endl;
        return 1;
    }
    return 0;
}
