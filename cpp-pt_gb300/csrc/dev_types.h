// Types shared by the host code and the CUDA kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cpppt_gb300 {

// Device material; for emitters rgb holds rgb * intensity (EmissiveMaterial::get_bxdf,
// src/bxdf/emissive_material.h:28-30), and alpha the intensity alone when the
// colour is an image texture.
struct DevMaterial {
    int32_t kind;     // PT_MAT_*
    float r, g, b;
    float alpha;      // GGX: max(roughness^2, 0.01) (glossy_bxdf.h:77-79)
    int32_t delta;    // GGX: roughness < 0.01 (glossy_bxdf.h:23)
    float ior;
    uint32_t tex;     // image textures, one byte each (kNoTex: constant): albedo / emission colour
                      // (bits 0-7), roughness (8-15), metal (16-23), normal map (24-31)
};

constexpr uint32_t kNoTex = 0xffu;
constexpr uint32_t kNoTextures = 0xffffffffu;

// CameraPerspective (src/camera/camera_perspective.h:19-39): origin and the
// column basis (x, y, z) of `coords`, stored row-major like Mat3.
struct DevCamera {
    float o[3];
    float m[9];
    float tan_fovy, aspect;
    int32_t width, height;
};

// Default bounds of a ray's traversal (kernel-side bounded loops): steps of
// the persistent loop and entries of the per-lane stack.  A scene may carry
// lower bounds (pt_debug_traversal_limits), never higher ones.
constexpr uint32_t kTraversalStepLimit = 1u << 22;
constexpr int32_t kTraversalStackSize = 64;

struct DevScene {
    // traversal bounds (see kTraversalStepLimit)
    uint32_t step_limit = kTraversalStepLimit;
    int32_t stack_limit = kTraversalStackSize;
    // traversal
    const uint4* nodes;      // 4 per wide node
    int32_t n_nodes;
    int32_t n_tris;
    const float4* tris;      // 3 per triangle in leaf order: {a, rank}, {b-a, parent box}, {c-a, prim}
    const float4* ref_box;   // 2 per reference internal node: lo, hi
    // shading, in insertion order
    const int4* tri_vidx;    // v0, v1, v2, material
    const float4* v_pos;
    const float4* v_nrm;
    const float4* v_btan;    // cross(normal, tangent) (loader.h:237)
    const DevMaterial* mats;
    const int32_t* light_prim;  // emissive triangles in insertion order
    const float* light_area;    // Triangle::area (triangle.h:197-207)
    int32_t n_lights;
    DevCamera cam;
    // image textures (file scenes): per-vertex uv, pixels of every texture,
    // {first float, width, height, channels} per texture
    const float2* v_uv;
    const float* tex_px;
    const int4* tex_info;
    int32_t n_tex;
};

// One render job of a multi-scene batch (the scenes' geometry is merged into
// one device arena; each job renders one scene of it at its own resolution,
// spp and seed into its own range of the merged film).
struct DevBatchJob {
    DevCamera cam;
    unsigned long long work_begin;  // first global work index (pixel x sample) of the job
    unsigned long long film_off;    // first pixel of the job in the merged film
    uint32_t root;                  // wide-node index of the scene's root in the arena
    int32_t light_off, n_lights;    // the scene's emissive triangles in the arena's light list
    int32_t spp, spp_axis, max_depth, rr_start;
    uint32_t seed;
    int32_t tile_w, tile_h;  // pixel order of a pass: tiles of tile_w x tile_h (both divide the resolution)
    int32_t integrator;      // kIntegratorMIS / kIntegratorNEE / kIntegratorPT
};

// The reference's three unidirectional estimators on one wavefront:
// PathtracerMIS (NEE + MIS), Pathtracer (NEE at full weight, emitters only
// after the camera or a delta bounce), PurePt (no NEE, every emitter hit).
constexpr int32_t kIntegratorMIS = 0;
constexpr int32_t kIntegratorNEE = 1;
constexpr int32_t kIntegratorPT = 2;

// Ray-batch status word bits (kernel-side bounded loops report here).
constexpr uint32_t kStatusIterLimit = 1u;
constexpr uint32_t kStatusStackOverflow = 2u;
constexpr uint32_t kStatusQueueOverflow = 4u;
constexpr uint32_t kStatusTensorTimeout = 8u;  // a tensor-core completion wait ran out (bounded spin)
constexpr uint32_t kStatusRoundLimit = 16u;    // a device-driven render loop reached its round bound

// Wavefront counters, one block of device memory per scene.
struct WaveCounters {
    int32_t n_cur, n_next, n_shadow, n_fin;  // n_fin: finished paths of the learned-guide integrator
    int32_t fetch_ext, fetch_sh, free_top, n_rec;  // free_top: vertex-slot free list; n_rec: training records
    uint32_t status;
    float film_safe;  // |contribution| below this cannot carry a film sum out of the 32.32 range
    uint32_t rounds;      // loop bodies run by a device-driven render (k_round_control)
    uint32_t max_rounds;  // its bound
    unsigned long long work_next, work_total;
    unsigned long long stat_closest, stat_shadow, stat_paths, stat_iters;
    unsigned long long stat_nodes, stat_tris;  // counting build of the extend kernel only
    unsigned long long stat_nonfinite;         // contributions dropped because they were inf/NaN
    unsigned long long stat_film_overflow;     // contributions the 32.32 film could not hold
};

// film_safe for a render of at most `per_pixel` film contributions per pixel
// and channel: a sum of contributions below 2^31 / per_pixel stays below
// 2^31, the largest value the signed 32.32 fixed-point film holds.
inline float film_safe_bound(double per_pixel) {
    return (float)(2147483648.0 / (per_pixel > 1.0 ? per_pixel : 1.0));
}

}  // namespace cpppt_gb300
