// Oracle harness around the reference renderer (drcd1/cpp-pt).  TEST
// INFRASTRUCTURE ONLY: tests, the golden-fixture generator and bench.py's
// CPU-baseline leg call it through ctypes; no product code links it.
//
// It compiles against a copy of the reference's own headers (made by
// oracle/build_ref.sh) and exposes, as extern "C":
//   - scene construction from flat arrays, mirroring Loader::load_scene
//     (src/loader/loader.h:314-374): one Mesh per mesh range, one
//     PrimitiveLeaf per triangle in insertion order, one ShapeLight per
//     emissive triangle, then BVH::build;
//   - closest-hit / any-hit queries through BVH::intersect / intersect_any
//     (src/primitive/bvh.h:219-224), reporting the hit's insertion index;
//   - a dump of the BVH that BVH::build made (DFS order of leaves, boxes);
//   - PathtracerMIS::render (src/renderer/pathtracerMIS.h:135-167), returning
//     the float film read from the camera's image;
//   - PPG::render (src/renderer/ppg.h:149-215) the same way.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>
#include <unistd.h>
#include <fcntl.h>
#include <algorithm>
#include <array>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <random>
#include <sstream>
#include <stdexcept>
#include <unordered_map>
#include <utility>
#include <omp.h>

int cpppt_harness_max_depth = 32;
int cpppt_harness_seed_offset = 0;
int cpppt_harness_verbose = 0;

// The BVH's tree and the leaf groups are private members; the harness reads
// them to dump the topology.  Standard headers are already included above.
#define private public
#include <camera/camera_perspective.h>
#include <light/point_light.h>
#include <renderer/pathtracerMIS.h>
#include <renderer/pathtracer.h>
#include <renderer/pure_pt.h>
// SDTree's tree sits in the default-private part of a `class`; read it as a
// struct (its dependencies are already included above).
#define class struct
#include <algorithms/sdtree.h>
#undef class
#include <renderer/ppg.h>
#include <primitive/bvh.h>
#include <shape/triangle.h>
#include <bxdf/glossy_bxdf.h>
#include <bxdf/refraction_bxdf.h>
#include <bxdf/emissive_material.h>
#include <light/shape_light.h>
#include <light/light_group.h>
#include <loader/loader.h>
#undef private

using namespace cpppt;

namespace {

// Material that hands out the reference's RefractionBxDF.  The reference
// loader cannot create one (StandardMaterial::get_bxdf never returns it), so
// scenes with dielectrics need this harness-side material.
class HarnessDielectric : public Material {
    float ior_;
public:
    explicit HarnessDielectric(float ior) : ior_(ior) {}
    std::shared_ptr<BxDF> get_bxdf(const Vec3&) const override {
        return std::make_shared<RefractionBxDF>(ior_);
    }
    Vec3 get_normal_mapped(const Vec3&, const Vec3&, const Vec3&, const Vec3& normal) const override {
        return normal;
    }
};

struct RefScene {
    Scene scene;
    SceneData data;
    RenderSettings rs;
    std::map<const Primitive*, int> leaf_index;
    std::string error;
};

// Redirects fd 1 to /dev/null while the reference prints progress.
struct Quiet {
    int saved = -1;
    Quiet() {
        fflush(stdout);
        std::cout.flush();
        saved = dup(1);
        int devnull = open("/dev/null", O_WRONLY);
        if (devnull >= 0) { dup2(devnull, 1); close(devnull); }
    }
    ~Quiet() {
        fflush(stdout);
        std::cout.flush();
        if (saved >= 0) { dup2(saved, 1); close(saved); }
    }
};

std::shared_ptr<Texture> ctex3(float r, float g, float b) {
    return std::make_shared<ConstantTexture<Vec3>>(Vec3(r, g, b));
}
std::shared_ptr<Texture> ctex1(float v) {
    return std::make_shared<ConstantTexture<float>>(v);
}

}  // namespace

template <class R>
static double render_with(RefScene* rs, int spp_axis, const char* out_prefix, float* rgb_out) {
    RenderSettings settings = rs->rs;
    settings.spp = spp_axis;
    R renderer(settings);
    double seconds;
    {
        Quiet q;
        auto t1 = std::chrono::high_resolution_clock::now();
        renderer.render(rs->scene, out_prefix);
        auto t2 = std::chrono::high_resolution_clock::now();
        seconds = std::chrono::duration<double>(t2 - t1).count();
    }
    RgbImage& img = rs->scene.camera->get_image();
    for (int j = 0; j < img.res.y; j++)
        for (int i = 0; i < img.res.x; i++) {
            Vec3 p = *img.get_pixel(i, j);
            float* o = rgb_out + 3 * (i + j * img.res.x);
            o[0] = p.x; o[1] = p.y; o[2] = p.z;
        }
    return seconds;
}

extern "C" {

// Material kinds: 0 diffuse, 1 GGX conductor, 2 dielectric, 3 emissive.
// mat_params: 8 floats per material {r, g, b, roughness, ior, intensity, 0, 0}.
//
// A diffuse/GGX material is what Loader::parse_mat builds from a DISNEY
// .ptmat (loader.h:154-180) with constant textures: metal 0 or 1, the
// normal map rgb(0.5,0.5,1).  An emissive one is EMISSION rgb(..) float(I)
// (loader.h:181-201).
void* ref_scene_create(int n_meshes, const int* mesh_vert_offset, const int* mesh_tri_offset,
                       const int* mesh_material,
                       const float* vertices, const float* normals, const float* tangents,
                       const int* triangles,
                       int n_materials, const int* mat_kind, const float* mat_params,
                       const float* camera /* origin3 at3 up3 tan_fovy */, int width, int height) {
    auto* rs = new RefScene();
    try {
        Quiet q;
        rs->rs.resX = width;
        rs->rs.resY = height;
        std::vector<std::shared_ptr<Material>> mats;
        for (int m = 0; m < n_materials; m++) {
            const float* p = mat_params + 8 * m;
            switch (mat_kind[m]) {
            case 0:
            case 1:
                mats.push_back(std::make_shared<StandardMaterial>(
                    ctex3(p[0], p[1], p[2]), ctex3(0.5f, 0.5f, 1.0f), ctex1(0.5f), ctex1(p[3]),
                    ctex1(mat_kind[m] == 1 ? 1.0f : 0.0f), ctex1(p[4]), ctex1(0.0f), ctex1(0.0f)));
                break;
            case 2:
                mats.push_back(std::make_shared<HarnessDielectric>(p[4]));
                break;
            case 3:
                mats.push_back(std::make_shared<EmissiveMaterial>(ctex3(p[0], p[1], p[2]), p[5]));
                break;
            default:
                throw std::runtime_error("unknown material kind");
            }
        }
        Vec3 origin(camera[0], camera[1], camera[2]);
        Vec3 at(camera[3], camera[4], camera[5]);
        Vec3 up(camera[6], camera[7], camera[8]);
        rs->scene.camera = std::make_shared<CameraPerspective>(
            Vec2i(width, height), camera[9], origin, normalized(at - origin), up);
        rs->scene.primitive = std::make_shared<BVH>();
        rs->scene.light = std::make_shared<LightGroup>();
        for (int mi = 0; mi < n_meshes; mi++) {
            int v0 = mesh_vert_offset[mi], v1 = mesh_vert_offset[mi + 1];
            int f0 = mesh_tri_offset[mi], f1 = mesh_tri_offset[mi + 1];
            auto mesh = std::make_shared<Mesh>(v1 - v0, f1 - f0);
            for (int v = v0; v < v1; v++) {
                Vec3 pos(vertices[3 * v], vertices[3 * v + 1], vertices[3 * v + 2]);
                Vec3 n(normals[3 * v], normals[3 * v + 1], normals[3 * v + 2]);
                Vec3 t(tangents[3 * v], tangents[3 * v + 1], tangents[3 * v + 2]);
                // loader.h:237: the file stores a tangent, the mesh a bitangent
                mesh->set_vertex_data(v - v0, pos, n, Vec2(0.0f, 0.0f), cross(n, t));
            }
            for (int f = f0; f < f1; f++)
                mesh->set_face_data(f - f0, triangles[3 * f] - v0, triangles[3 * f + 1] - v0,
                                    triangles[3 * f + 2] - v0);
            rs->data.meshes.push_back(mesh);
            rs->data.materials.push_back(mats.at(mesh_material[mi]));
        }
        // loader.h:353-367
        int index = 0;
        for (size_t i = 0; i < rs->data.meshes.size(); i++) {
            for (int j = 0; j < rs->data.meshes[i]->n_triangles(); j++) {
                auto leaf = std::make_shared<PrimitiveLeaf>(
                    std::make_shared<Triangle>(rs->data.meshes[i].get(), j), rs->data.materials[i]);
                rs->scene.primitive->add(leaf);
                rs->leaf_index[leaf.get()] = index++;
                if (rs->data.materials[i]->is_emissive())
                    rs->scene.light->add(std::make_shared<ShapeLight>(leaf));
            }
        }
        rs->scene.primitive->build();
    } catch (std::exception& e) {
        rs->error = e.what();
    }
    return rs;
}

const char* ref_scene_error(void* h) {
    return static_cast<RefScene*>(h)->error.c_str();
}

void ref_scene_destroy(void* h) { delete static_cast<RefScene*>(h); }

// Loads a scene through the reference's own Loader (loader.h:256-374) from a
// render-settings file.  Returns width/height through out params.
void* ref_scene_load(const char* settings_file, int* width, int* height, int* spp) {
    auto* rs = new RefScene();
    try {
        Quiet q;
        Loader::load_render_settings(&rs->rs, settings_file);
        Loader::load_scene(&rs->scene, &rs->data, &rs->rs, rs->rs.scene_name);
        int index = 0;
        for (auto& p : rs->scene.primitive->primitives) rs->leaf_index[p.get()] = index++;
        *width = rs->rs.resX;
        *height = rs->rs.resY;
        *spp = rs->rs.spp;
    } catch (std::exception& e) {
        rs->error = e.what();
    }
    return rs;
}

int ref_num_primitives(void* h) {
    return (int)static_cast<RefScene*>(h)->scene.primitive->primitives.size();
}

// rays: 7 floats each {ox, oy, oz, dx, dy, dz, max_t}.  out_index = insertion
// index of the hit primitive or -1; out_t = the ray's max_t after the query.
void ref_trace_closest(void* h, const float* rays, int n, int* out_index, float* out_t) {
    auto* rs = static_cast<RefScene*>(h);
    const BVH& bvh = *rs->scene.primitive;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        const float* r = rays + 7 * i;
        Ray ray(Vec3(r[0], r[1], r[2]), Vec3(r[3], r[4], r[5]), r[6]);
        Intersection is;
        is.primitive = nullptr;
        bool hit = bvh.intersect(ray, &is);
        out_t[i] = ray.max_t;
        if (hit && is.primitive) {
            auto it = rs->leaf_index.find(is.primitive);
            out_index[i] = it == rs->leaf_index.end() ? -2 : it->second;
        } else {
            out_index[i] = -1;
        }
    }
}

void ref_trace_any(void* h, const float* rays, int n, unsigned char* out_hit) {
    auto* rs = static_cast<RefScene*>(h);
    const BVH& bvh = *rs->scene.primitive;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        const float* r = rays + 7 * i;
        Ray ray(Vec3(r[0], r[1], r[2]), Vec3(r[3], r[4], r[5]), r[6]);
        out_hit[i] = bvh.intersect_any(ray) ? 1 : 0;
    }
}

// Dumps the tree BVH::build produced.  Walks it in the order
// BVHNode::intersect visits it (member `right` first, bvh.h:33-34).
//   leaf_order[k]  = insertion index of the k-th primitive met (size n_prims)
//   node_boxes     = 6 floats per internal node, pre-order (size 6*max_nodes)
//   node_parent    = parent internal node of each internal node (-1 at root)
//   prim_parent    = for each insertion index, internal node holding its leaf
// Returns the number of internal nodes.
int ref_bvh_dump(void* h, int* leaf_order, float* node_boxes, int* node_parent, int* prim_parent,
                 int max_nodes) {
    auto* rs = static_cast<RefScene*>(h);
    int n_nodes = 0, n_leaf = 0;
    struct Item { const Primitive* p; int parent; };
    std::vector<Item> stack;
    stack.push_back({rs->scene.primitive->root.get(), -1});
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        if (auto* node = dynamic_cast<const BVHNode*>(it.p)) {
            int id = n_nodes++;
            if (id < max_nodes) {
                const AABB& b = node->aabb;
                float* o = node_boxes + 6 * id;
                o[0] = b.min.x; o[1] = b.min.y; o[2] = b.min.z;
                o[3] = b.max.x; o[4] = b.max.y; o[5] = b.max.z;
                node_parent[id] = it.parent;
            }
            // visited first must be popped first
            stack.push_back({node->left.get(), id});
            stack.push_back({node->right.get(), id});
        } else if (auto* group = dynamic_cast<const SimpleGroup*>(it.p)) {
            for (auto& p : group->primitives) {
                int idx = rs->leaf_index.at(p.get());
                leaf_order[n_leaf++] = idx;
                prim_parent[idx] = it.parent;
            }
        }
    }
    return n_nodes;
}

// PathtracerMIS::render with the settings value `spp` (= samples per axis:
// spp*spp samples per pixel), a bounce limit and a column-seed offset.
// Writes width*height*3 floats, row-major from the top row.  Returns the
// render time in seconds measured like main.cpp:130-142.
double ref_render_mis(void* h, int spp_axis, int max_depth, int seed_offset, int threads,
                      const char* out_prefix, float* rgb_out) {
    auto* rs = static_cast<RefScene*>(h);
    cpppt_harness_max_depth = max_depth;
    cpppt_harness_seed_offset = seed_offset;
    if (threads > 0) omp_set_num_threads(threads);
    RenderSettings settings = rs->rs;
    settings.spp = spp_axis;
    PathtracerMIS renderer(settings);
    double seconds;
    {
        Quiet q;
        auto t1 = std::chrono::high_resolution_clock::now();
        renderer.render(rs->scene, out_prefix);
        auto t2 = std::chrono::high_resolution_clock::now();
        seconds = std::chrono::duration<double>(t2 - t1).count();
    }
    RgbImage& img = rs->scene.camera->get_image();
    for (int j = 0; j < img.res.y; j++)
        for (int i = 0; i < img.res.x; i++) {
            Vec3 p = *img.get_pixel(i, j);
            float* o = rgb_out + 3 * (i + j * img.res.x);
            o[0] = p.x; o[1] = p.y; o[2] = p.z;
        }
    return seconds;
}

// The reference's other two integrators on the same scene: which = 1
// Pathtracer (PT + NEE without MIS, pathtracer.h:27-102), which = 2 PurePt
// (no NEE, pure_pt.h:28-71).  Same settings as ref_render_mis.
double ref_render_variant(void* h, int which, int spp_axis, int max_depth, int seed_offset, int threads,
                          const char* out_prefix, float* rgb_out) {
    auto* rs = static_cast<RefScene*>(h);
    cpppt_harness_max_depth = max_depth;
    cpppt_harness_seed_offset = seed_offset;
    if (threads > 0) omp_set_num_threads(threads);
    if (which == 1) return render_with<Pathtracer>(rs, spp_axis, out_prefix, rgb_out);
    if (which == 2) return render_with<PurePt>(rs, spp_axis, out_prefix, rgb_out);
    return render_with<PathtracerMIS>(rs, spp_axis, out_prefix, rgb_out);
}

// PPG::render (SD-tree guided, no NEE; ppg.h:149-215).  The bounce limit of
// ppg.h:49 stays at the reference's 32.
double ref_render_ppg(void* h, int spp_axis, int seed_offset, int threads, const char* out_prefix,
                      float* rgb_out) {
    auto* rs = static_cast<RefScene*>(h);
    cpppt_harness_seed_offset = seed_offset;
    if (threads > 0) omp_set_num_threads(threads);
    RenderSettings settings = rs->rs;
    settings.spp = spp_axis;
    PPG renderer(settings);
    double seconds;
    {
        Quiet q;
        auto t1 = std::chrono::high_resolution_clock::now();
        renderer.render(rs->scene, out_prefix);
        auto t2 = std::chrono::high_resolution_clock::now();
        seconds = std::chrono::duration<double>(t2 - t1).count();
    }
    RgbImage& img = rs->scene.camera->get_image();
    for (int j = 0; j < img.res.y; j++)
        for (int i = 0; i < img.res.x; i++) {
            Vec3 p = *img.get_pixel(i, j);
            float* o = rgb_out + 3 * (i + j * img.res.x);
            o[0] = p.x; o[1] = p.y; o[2] = p.z;
        }
    return seconds;
}

int ref_max_threads(void) { return omp_get_max_threads(); }

// An image file through the reference's own Image<Vec3> (rgb = 1) or
// Image<float> (rgb = 0) with the colour space a material would give it
// (rgb_image.h:160-205, stb_image).  out (nullable) receives w * h * (rgb ?
// 3 : 1) floats.  Returns 0, or 2 when cap is too small.  Only call it on
// files stb can read: the reference does not check stbi_load's result.
int ref_image_load(const char* path, int rgb, int srgb, int* w, int* h, float* out, long long cap) {
    const auto cs = srgb ? ImageDef::SRGB : ImageDef::LINEAR;
    if (rgb) {
        Image<Vec3> im(path, cs);
        *w = im.res.x;
        *h = im.res.y;
        if (!out) return 0;
        if (cap < 3LL * im.res.x * im.res.y) return 2;
        for (size_t i = 0; i < im.pixels.size(); i++) {
            out[3 * i] = im.pixels[i].x;
            out[3 * i + 1] = im.pixels[i].y;
            out[3 * i + 2] = im.pixels[i].z;
        }
    } else {
        Image<float> im(path, cs);
        *w = im.res.x;
        *h = im.res.y;
        if (!out) return 0;
        if (cap < 1LL * im.res.x * im.res.y) return 2;
        for (size_t i = 0; i < im.pixels.size(); i++) out[i] = im.pixels[i];
    }
    return 0;
}

// Runs the reference's SDTree (src/algorithms/sdtree.h:268-674) through
// n_iters rounds of {splat the round's records, update()}.  splats: 7 floats
// each {radiance, pos xyz, dir xyz}.  Then dumps, for every spatial leaf in
// depth-first order (child 0 first), its sampling leaves (4 floats each:
// begin phi, begin cos, size phi, size cos), count and flux, and answers pdf
// queries (6 floats each: pos, dir).  Returns the number of spatial leaves.
int ref_sdtree_run(const float* lo, const float* hi, int n_iters, const int* n_splats, const float* splats,
                   int max_leaves, float* out_leaves, int* out_leaf_counts, int* out_counts, float* out_flux,
                   int n_queries, const float* queries, float* out_pdf) {
    SDTree st({Vec3(lo[0], lo[1], lo[2]), Vec3(hi[0], hi[1], hi[2])});
    {
        Quiet q;
        size_t off = 0;
        for (int it = 0; it < n_iters; it++) {
            for (int k = 0; k < n_splats[it]; k++, off++) {
                const float* s = splats + 7 * off;
                st.splat(s[0], Vec3(s[1], s[2], s[3]), Vec3(s[4], s[5], s[6]));
            }
            st.update();
        }
    }
    for (int k = 0; k < n_queries; k++) {
        const float* qv = queries + 6 * k;
        out_pdf[k] = st.pdf(Vec3(qv[0], qv[1], qv[2]), Vec3(qv[3], qv[4], qv[5]));
    }
    int n_sleaf = 0, n_out = 0;
    std::vector<const SNode*> stack{&st.root};
    while (!stack.empty()) {
        const SNode* n = stack.back();
        stack.pop_back();
        if (n->isLeaf) {
            const DTree& d = *n->leaf.pt;
            out_leaf_counts[n_sleaf] = (int)d.leaves.size();
            out_counts[n_sleaf] = d.count;
            out_flux[n_sleaf] = d.radiance;
            for (auto& l : d.leaves) {
                if (n_out < max_leaves) {
                    out_leaves[4 * n_out] = l.begin.x;
                    out_leaves[4 * n_out + 1] = l.begin.y;
                    out_leaves[4 * n_out + 2] = l.size.x;
                    out_leaves[4 * n_out + 3] = l.size.y;
                }
                n_out++;
            }
            n_sleaf++;
        } else {
            stack.push_back(&n->children->at(1));
            stack.push_back(&n->children->at(0));
        }
    }
    return n_sleaf;
}

}  // extern "C"
