// C ABI of the GB300 path tracer (declared in include/cpppt_gb300.h).
//
// Owns the device copy of a scene, the wavefront buffers and the CUDA graph
// that replays wavefront iterations.  No call throws across the ABI; errors
// are status codes plus a thread-local message.
#include "gpu_bvh.h"
#include "host_internal.h"
#include "image_io.h"
#include "loader.h"

#include <thread>
#include <iterator>

using namespace cpppt_gb300;
using namespace cpppt_gb300::hostimpl;

thread_local std::string cpppt_gb300::hostimpl::g_error;

namespace {

void check_device(pt_scene* s) {
    int dev = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    cudaDeviceProp prop;
    ck(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    if (prop.major * 10 + prop.minor != 103)
        throw Fail(PT_ERR_NO_DEVICE, "device " + std::string(prop.name) + " is not compute capability 10.3 (sm_103a)");
    s->device = dev;
    s->num_sms = prop.multiProcessorCount;
    ck(trace_kernels_setup(), "traversal shared memory limits");
    ck(nn_set_smem_limits(), "guided wavefront shared memory limits");
}

void create_scene(const pt_scene_desc* d, pt_scene* s, const SceneTextures* tx = nullptr) {
    if (!d) throw std::invalid_argument("null scene description");
    const int nv = d->n_vertices, nt = d->n_triangles, nm = d->n_materials;
    if (nv < 0 || nt < 0 || nm < 0) throw std::invalid_argument("negative count");
    if (nt > 0 && (!d->vertices || !d->normals || !d->triangles || !d->tri_material))
        throw std::invalid_argument("missing vertex or triangle arrays");
    if (nt > (1 << 27) - 1) throw std::invalid_argument("too many triangles (max 2^27-1)");
    if (nm > 0 && !d->materials) throw std::invalid_argument("missing materials");
    if (d->camera.width <= 0 || d->camera.height <= 0) throw std::invalid_argument("camera resolution must be positive");
    for (int i = 0; i < 3 * nt; i++)
        if (d->triangles[i] < 0 || d->triangles[i] >= nv) throw std::invalid_argument("triangle vertex index out of range");
    for (int i = 0; i < nt; i++)
        if (d->tri_material[i] < 0 || d->tri_material[i] >= nm) throw std::invalid_argument("triangle material out of range");
    for (int i = 0; i < nm; i++)
        if (d->materials[i].kind < 0 || d->materials[i].kind > 3) throw std::invalid_argument("unknown material kind");

    check_device(s);
    ck(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    s->n_tris = nt;
    s->width = d->camera.width;
    s->height = d->camera.height;

    // per-triangle vertex positions (a, b, c)
    std::vector<float> tv(9 * (size_t)nt);
    for (int t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++)
            std::memcpy(&tv[9 * (size_t)t + 3 * k], d->vertices + 3 * (size_t)d->triangles[3 * t + k], 12);

    // the two device builds are independent: the 4-wide SAH tree from a
    // second host thread on a stream of its own
    auto t0 = std::chrono::steady_clock::now();
    WideBVH wide;
    std::exception_ptr wide_err;
    std::chrono::steady_clock::time_point t2;
    const int dev = s->device;
    std::thread wide_th([&] {
        cudaStream_t ws = nullptr;
        try {
            ck(cudaSetDevice(dev), "cudaSetDevice");
            ck(cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking), "cudaStreamCreate");
            wide = build_wide_bvh_device(tv.data(), nt, 4, ws);
        } catch (...) {
            wide_err = std::current_exception();
        }
        if (ws) cudaStreamDestroy(ws);
        t2 = std::chrono::steady_clock::now();
    });
    RefTopology ref;
    try {
        ref = build_ref_topology_device(tv.data(), nt, s->stream);
    } catch (...) {
        wide_th.join();
        throw;
    }
    auto t1 = std::chrono::steady_clock::now();
    wide_th.join();
    if (wide_err) std::rethrow_exception(wide_err);
    s->build_ref_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    s->build_wide_ms = std::chrono::duration<double, std::milli>(t2 - t0).count();
    s->wide_depth = wide.max_depth;
    for (int k = 0; k < 3; k++) { s->bounds_lo[k] = INFINITY; s->bounds_hi[k] = -INFINITY; }
    for (size_t i = 0; i < tv.size(); i += 3)
        for (int k = 0; k < 3; k++) {
            s->bounds_lo[k] = std::min(s->bounds_lo[k], tv[i + k]);
            s->bounds_hi[k] = std::max(s->bounds_hi[k], tv[i + k]);
        }
    if (3 * wide.max_depth + 4 > 64) throw Fail(PT_ERR_LIMIT, "wide BVH too deep for the traversal stack");

    // traversal triangles in leaf order: {a, rank}, {b - a, parent}, {c - a, prim}
    std::vector<float4> tris(3 * (size_t)nt);
    for (int k = 0; k < nt; k++) {
        const int p = wide.tri_order[k];
        const float* v = &tv[9 * (size_t)p];
        float a[3] = {v[0], v[1], v[2]};
        float e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};  // triangle.h:40 (b - a)
        float e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};  // triangle.h:41 (c - a)
        int32_t rank = ref.rank[p], parent = ref.prim_parent[p];
        float rf, pf, idf;
        std::memcpy(&rf, &rank, 4);
        std::memcpy(&pf, &parent, 4);
        std::memcpy(&idf, &p, 4);
        tris[3 * (size_t)k] = make_float4(a[0], a[1], a[2], rf);
        tris[3 * (size_t)k + 1] = make_float4(e1[0], e1[1], e1[2], pf);
        tris[3 * (size_t)k + 2] = make_float4(e2[0], e2[1], e2[2], idf);
    }
    std::vector<float4> rbox(2 * ref.node_box.size());
    for (size_t i = 0; i < ref.node_box.size(); i++) {
        const Box3& b = ref.node_box[i];
        rbox[2 * i] = make_float4(b.lo[0], b.lo[1], b.lo[2], 0.f);
        rbox[2 * i + 1] = make_float4(b.hi[0], b.hi[1], b.hi[2], 0.f);
    }
    // shading data
    std::vector<int4> vidx(nt);
    for (int t = 0; t < nt; t++)
        vidx[t] = make_int4(d->triangles[3 * t], d->triangles[3 * t + 1], d->triangles[3 * t + 2], d->tri_material[t]);
    std::vector<float4> vpos(nv), vnrm(nv), vbt(nv);
    for (int v = 0; v < nv; v++) {
        const float* p = d->vertices + 3 * (size_t)v;
        const float* n = d->normals + 3 * (size_t)v;
        float tg[3];
        if (d->tangents) {
            std::memcpy(tg, d->tangents + 3 * (size_t)v, 12);
        } else {  // any vector perpendicular to the normal
            float ax[3] = {std::fabs(n[1]) < 0.9f ? 0.f : 1.f, std::fabs(n[1]) < 0.9f ? 1.f : 0.f, 0.f};
            fcross(ax, n, tg);
            fnorm3(tg);
        }
        float bt[3];
        fcross(n, tg, bt);  // loader.h:237
        vpos[v] = make_float4(p[0], p[1], p[2], 0.f);
        vnrm[v] = make_float4(n[0], n[1], n[2], 0.f);
        vbt[v] = make_float4(bt[0], bt[1], bt[2], 0.f);
    }
    std::vector<DevMaterial> mats(nm);
    for (int i = 0; i < nm; i++) {
        const pt_material& m = d->materials[i];
        DevMaterial dm{};
        dm.kind = m.kind;
        dm.r = m.rgb[0]; dm.g = m.rgb[1]; dm.b = m.rgb[2];
        if (m.kind == PT_MAT_EMISSIVE) { dm.r *= m.intensity; dm.g *= m.intensity; dm.b *= m.intensity; }
        float r2 = m.roughness * m.roughness;
        dm.alpha = std::max(r2, 0.01f);
        dm.delta = (double)m.roughness < 0.01 ? 1 : 0;
        dm.ior = m.ior;
        dm.tex = kNoTextures;
        if (tx && i < (int)tx->mat_tex.size()) {
            dm.tex = tx->mat_tex[i];
            if (m.kind == PT_MAT_EMISSIVE && (dm.tex & 0xffu) != kNoTex) dm.alpha = tx->emit_intensity[i];
        }
        mats[i] = dm;
    }
    std::vector<int32_t> lprim;
    std::vector<float> larea;
    for (int t = 0; t < nt; t++) {
        if (d->materials[d->tri_material[t]].kind != PT_MAT_EMISSIVE) continue;
        lprim.push_back(t);
        const float* v = &tv[9 * (size_t)t];
        float e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]}, e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]}, c[3];
        fcross(e1, e2, c);
        larea.push_back(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) * 0.5f);
    }
    std::vector<uint4> nodes(4 * wide.nodes.size());
    std::memcpy(nodes.data(), wide.nodes.data(), sizeof(WideNode) * wide.nodes.size());

    s->n_verts = nv;
    s->n_mats = nm;
    s->n_rbox = (int)ref.node_box.size();
    DevScene& S = s->dev;
    S.nodes = dupload(s->owned, nodes, s->stream);
    S.n_nodes = (int)wide.nodes.size();
    S.n_tris = nt;
    S.tris = dupload(s->owned, tris, s->stream);
    S.ref_box = dupload(s->owned, rbox, s->stream);
    S.tri_vidx = dupload(s->owned, vidx, s->stream);
    S.v_pos = dupload(s->owned, vpos, s->stream);
    S.v_nrm = dupload(s->owned, vnrm, s->stream);
    S.v_btan = dupload(s->owned, vbt, s->stream);
    S.mats = dupload(s->owned, mats, s->stream);
    s->h_mats = mats;
    S.light_prim = dupload(s->owned, lprim, s->stream);
    S.light_area = dupload(s->owned, larea, s->stream);
    S.n_lights = (int)lprim.size();
    // image textures and uv (zero uv and an empty texture table without them)
    std::vector<float2> uv(std::max(1, nv), make_float2(0.f, 0.f));
    if (tx && tx->uv.size() >= 2 * (size_t)nv)
        for (int v = 0; v < nv; v++) uv[v] = make_float2(tx->uv[2 * (size_t)v], tx->uv[2 * (size_t)v + 1]);
    S.v_uv = dupload(s->owned, uv, s->stream);
    std::vector<float> px = (tx && !tx->px.empty()) ? tx->px : std::vector<float>(1, 0.f);
    std::vector<int4> info = (tx && !tx->info.empty()) ? tx->info : std::vector<int4>(1, make_int4(0, 1, 1, 1));
    S.tex_px = dupload(s->owned, px, s->stream);
    S.tex_info = dupload(s->owned, info, s->stream);
    S.n_tex = tx ? (int)tx->info.size() : 0;
    s->h_tex_info.assign(info.begin(), info.begin() + S.n_tex);
    s->n_tex_px = tx ? tx->px.size() : 0;
    // camera: CameraPerspective(res, tan_fovy, origin, normalized(at - origin), up)
    const pt_camera& c = d->camera;
    float fwd[3] = {c.at[0] - c.origin[0], c.at[1] - c.origin[1], c.at[2] - c.origin[2]};
    fnorm3(fwd);
    float z[3] = {-fwd[0], -fwd[1], -fwd[2]}, x[3], y[3];
    fnorm3(z);
    fcross(c.up, z, x);
    fnorm3(x);
    fcross(z, x, y);
    fnorm3(y);
    DevCamera& C = S.cam;
    for (int k = 0; k < 3; k++) C.o[k] = c.origin[k];
    float m9[9] = {x[0], y[0], z[0], x[1], y[1], z[1], x[2], y[2], z[2]};
    std::memcpy(C.m, m9, sizeof(m9));
    C.tan_fovy = c.tan_fovy;
    C.aspect = (float)c.width / (float)c.height;
    C.width = c.width;
    C.height = c.height;

    s->d_counter = dalloc<int>(s->owned, 4);
    s->d_status = reinterpret_cast<uint32_t*>(s->d_counter + 1);
    s->d_ctr = dalloc<WaveCounters>(s->owned, 1);
    ck(cudaMallocHost(&s->h_ctr, sizeof(WaveCounters)), "cudaMallocHost");
    s->d_job = dalloc<DevBatchJob>(s->owned, 1);
    ck(cudaMallocHost(&s->h_job, sizeof(DevBatchJob)), "cudaMallocHost");
    s->d_nnjob = dalloc<DevNNJob>(s->owned, 1);
    ck(cudaMallocHost(&s->h_nnjob, sizeof(DevNNJob)), "cudaMallocHost");
    ck(cudaEventCreate(&s->ev0), "cudaEventCreate");
    ck(cudaEventCreate(&s->ev1), "cudaEventCreate");
    ck(cudaStreamSynchronize(s->stream), "scene upload");
}

void ensure_io(pt_scene* s, size_t bytes) {
    if (s->d_io_bytes >= bytes) return;
    if (s->d_io) cudaFree(s->d_io);
    s->d_io = nullptr;
    s->d_io_bytes = 0;
    ck(cudaMalloc(&s->d_io, bytes), "cudaMalloc");
    s->d_io_bytes = bytes;
}

void check_status(pt_scene* s, uint32_t status) {
    if (status & kStatusIterLimit) throw Fail(PT_ERR_LIMIT, "traversal step limit reached");
    if (status & kStatusStackOverflow) throw Fail(PT_ERR_LIMIT, "traversal stack overflow");
    if (status & kStatusQueueOverflow) throw Fail(PT_ERR_LIMIT, "wavefront queue overflow");
    if (status & kStatusTensorTimeout) throw Fail(PT_ERR_CUDA, "tensor-core completion wait timed out");
    if (status & kStatusRoundLimit) throw Fail(PT_ERR_LIMIT, "render did not converge within the iteration bound");
}

void trace_device(pt_scene* s, const pt_ray* rays, int n, void* out, bool any, cudaStream_t st) {
    if (n < 0) throw std::invalid_argument("negative ray count");
    if (n == 0) return;
    if (!rays || !out) throw std::invalid_argument("null buffer");
    ck(cudaMemsetAsync(s->d_counter, 0, 2 * sizeof(int), st), "memset");
    if (any)
        launch_trace_any(s->dev, reinterpret_cast<const float*>(rays), n, static_cast<uint8_t*>(out), s->d_counter,
                         s->d_status, s->num_sms, st);
    else
        launch_trace_closest(s->dev, reinterpret_cast<const float*>(rays), n, static_cast<float4*>(out), s->d_counter,
                             s->d_status, s->num_sms, st);
    ck(cudaGetLastError(), "trace launch");
}

void trace_host(pt_scene* s, const pt_ray* rays, int n, void* out, bool any) {
    if (n < 0) throw std::invalid_argument("negative ray count");
    if (n == 0) return;
    if (!rays || !out) throw std::invalid_argument("null buffer");
    const size_t in_bytes = sizeof(pt_ray) * (size_t)n;
    const size_t out_bytes = any ? (size_t)n : sizeof(pt_hit) * (size_t)n;
    const size_t out_off = (in_bytes + 255) & ~(size_t)255;
    ensure_io(s, out_off + out_bytes);
    char* base = static_cast<char*>(s->d_io);
    ck(cudaMemcpyAsync(base, rays, in_bytes, cudaMemcpyHostToDevice, s->stream), "copy rays");
    trace_device(s, reinterpret_cast<const pt_ray*>(base), n, base + out_off, any, s->stream);
    ck(cudaMemcpyAsync(out, base + out_off, out_bytes, cudaMemcpyDeviceToHost, s->stream), "copy hits");
    uint32_t status = 0;
    ck(cudaMemcpyAsync(&status, s->d_status, 4, cudaMemcpyDeviceToHost, s->stream), "copy status");
    ck(cudaStreamSynchronize(s->stream), "trace");
    check_status(s, status);
}

// Paths in flight of a single render.  Each traversal launch ends with a
// tail in which a few long rays hold their SMs, so larger wavefronts
// amortise it over more rays.  Measured on the 1M-triangle soup at 1080p,
// 64 spp: 2^20 279.5 Mpaths/s, 2^21 310.6, 2^22 328.5, 2^23 337.3, 2^24
// 342.6, 2^25 334.2 (2^24 paths hold 3.2 GB of path state).
#ifndef CPPPT_MAX_WAVE_LOG2
#define CPPPT_MAX_WAVE_LOG2 24
#endif
constexpr int kMaxCapacity = 1 << CPPPT_MAX_WAVE_LOG2;
// Paths in flight of the learned-guide (slot) wavefront, each with a vertex
// record per bounce for training (112 B x depth per path).  Larger
// wavefronts render faster (on the 200k-triangle slit room at 1280x720,
// depth 12, 8 spp per call: 2^20 guided and training 157.5 Mpaths/s, 2^22
// 204) but gave far worse images: with the record quota filled in finishing
// order the guide learned from short paths only (config 4 at 60 s: relMSE
// 3.3e-3 against 4.7e-4 at 2^20); with records sampled evenly (the keep
// probability) it learned faster but then took very bright samples
// (relMSE 8.8e-3 at 10 s).  So 2^20.
#ifndef CPPPT_NN_WAVE_LOG2
#define CPPPT_NN_WAVE_LOG2 20
#endif
constexpr int kItersPerGraph = 16;  // even: buffers alternate

// The scene's wavefront buffers for `capacity` paths in flight (192 B per
// path, kept for later renders).  Returns the paths in flight the render
// uses: `capacity`, or fewer when the device cannot hold that many (the
// request halved down to 2^20 paths; the images do not depend on it).
int ensure_wave(pt_scene* s, int capacity, int film_n) {
    if (s->pb.capacity < capacity) {
        PathBuffers& B = s->pb;
        auto release = [&] {
            for (void* p : s->pb_owned) cudaFree(p);
            s->pb_owned.clear();
            B.capacity = 0;
        };
        release();
        if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
        for (int c = capacity;; c = std::max(1 << 20, c / 2)) {
            try {
                for (int k = 0; k < 2; k++) {
                    B.o[k] = dalloc<float4>(s->pb_owned, c);
                    B.d[k] = dalloc<float4>(s->pb_owned, c);
                    B.thr[k] = dalloc<float4>(s->pb_owned, c);
                    B.info[k] = dalloc<int4>(s->pb_owned, c);
                }
                B.hit = dalloc<float4>(s->pb_owned, c);
                B.sh_o = dalloc<float4>(s->pb_owned, c);
                B.sh_d = dalloc<float4>(s->pb_owned, c);
                B.sh_c = dalloc<float4>(s->pb_owned, c);
                B.capacity = c;
                break;
            } catch (...) {
                release();
                cudaGetLastError();  // an allocation failure is not sticky
                if (c <= (1 << 20)) throw;
            }
        }
    }
    if (s->film_n != film_n) {
        if (s->film) cudaFree(s->film);
        if (s->d_out) cudaFree(s->d_out);
        s->film = nullptr; s->d_out = nullptr;
        ck(cudaMalloc(&s->film, sizeof(unsigned long long) * film_n), "cudaMalloc film");
        ck(cudaMalloc(&s->d_out, sizeof(float) * film_n), "cudaMalloc film");
        s->film_n = film_n;
        if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
    }
    return std::min(capacity, s->pb.capacity);
}

// PPG::render (src/renderer/ppg.h:149-215): passes of 1, 2, 4, ... spp while
// below spp in total; the SD-tree learns from every pass (splats on the GPU,
// SDTree::update on the host) and only the last pass's image is kept.
void render_ppg(pt_scene* s, const pt_render_desc* desc, float* d_dst) {
    cudaStream_t st = s->stream;
    std::vector<int> passes;
    for (int spp = 1;; spp *= 2) {
        passes.push_back(spp);
        if (spp * 2 >= desc->spp) break;
    }
    const int film_n = 3 * s->width * s->height;
    const int D = desc->max_depth;
    const unsigned long long max_pass = (unsigned long long)s->width * s->height * (unsigned long long)passes.back();
    const int capacity =
        ensure_wave(s, (int)std::min<unsigned long long>(1 << 20, (max_pass + 1023) / 1024 * 1024), film_n);
    std::vector<void*> tmp;  // per-render buffers
    struct Free {
        std::vector<void*>& v;
        ~Free() { for (void* p : v) cudaFree(p); }
    } free_guard{tmp};
    PPGVerts V;
    V.vp = dalloc<float4>(tmp, (size_t)capacity * D);
    V.vd = dalloc<float4>(tmp, (size_t)capacity * D);
    V.vr = dalloc<float>(tmp, (size_t)capacity * D);
    int* slots = dalloc<int>(tmp, capacity);
    SDTreeHost tree(s->bounds_lo, s->bounds_hi);
    RenderParams P{};
    P.max_depth = desc->max_depth;
    P.rr_start = desc->rr_start;
    P.width = s->width;
    P.height = s->height;
    P.spp_axis = 0;  // ppg.h:181-184: one jittered sample per pixel per pass
    pt_render_stats total{};
    ck(cudaEventRecord(s->ev0, st), "event");
    double launches = 0;
    for (size_t l = 0; l < passes.size(); l++) {
        const SDTreeFlat f = tree.flatten();
        std::vector<void*> tt;
        Free tguard{tt};
        DevSDTree T;
        for (int k = 0; k < 3; k++) { T.lo[k] = f.lo[k]; T.hi[k] = f.hi[k]; }
        std::vector<int2> sn(f.snode.size() / 2);
        for (size_t i = 0; i < sn.size(); i++) sn[i] = make_int2(f.snode[2 * i], f.snode[2 * i + 1]);
        T.snode = dupload(tt, sn, st);
        T.dnode = dupload(tt, f.dnode, st);
        T.dtree_root = dupload(tt, f.dtree_root, st);
        T.leaf_off = dupload(tt, f.dtree_leaf_off, st);
        T.leaf_cnt = dupload(tt, f.dtree_leaf_cnt, st);
        std::vector<float4> lv(f.leaves.size() / 4);
        for (size_t i = 0; i < lv.size(); i++)
            lv[i] = make_float4(f.leaves[4 * i], f.leaves[4 * i + 1], f.leaves[4 * i + 2], f.leaves[4 * i + 3]);
        T.leaves = dupload(tt, lv, st);
        const int n_dtree = (int)f.dtree_root.size();
        T.slot_value = dalloc<float>(tt, f.n_value_slots);
        T.dtree_count = dalloc<int>(tt, n_dtree);
        T.dtree_rad = dalloc<float>(tt, n_dtree);
        ck(cudaMemsetAsync(T.slot_value, 0, sizeof(float) * std::max(1, f.n_value_slots), st), "memset");
        ck(cudaMemsetAsync(T.dtree_count, 0, sizeof(int) * std::max(1, n_dtree), st), "memset");
        ck(cudaMemsetAsync(T.dtree_rad, 0, sizeof(float) * std::max(1, n_dtree), st), "memset");
        ck(cudaMemsetAsync(s->film, 0, sizeof(unsigned long long) * film_n, st), "memset film");
        launch_init_slots(slots, capacity, st);
        P.spp = passes[l];
        P.seed = desc->seed * 7919u + (uint32_t)l;
        const unsigned long long work = (unsigned long long)s->width * s->height * (unsigned long long)passes[l];
        WaveCounters init{};
        init.work_total = work;
        init.free_top = capacity;
        init.film_safe = film_safe_bound((double)passes[l] * (2.0 * D + 2.0));
        *s->h_ctr = init;
        ck(cudaMemcpyAsync(s->d_ctr, s->h_ctr, sizeof(WaveCounters), cudaMemcpyHostToDevice, st), "init counters");
        launch_generate_ppg(s->dev, s->pb, 1, P, s->d_ctr, slots, st);
        launches += 4;
        const unsigned long long max_rounds =
            64 + (work / (unsigned long long)capacity + 2) * (unsigned long long)(D + 2) * 4 / kItersPerGraph;
        for (unsigned long long round = 0;; round++) {
            for (int k = 0; k < kItersPerGraph; k++) {
                const int cur = k & 1;
                launch_extend(s->dev, s->pb, cur, s->d_ctr, s->num_sms, st);
                launch_shade_ppg(s->dev, s->pb, cur, P, s->d_ctr, s->film, T, V, slots, st);
                launch_generate_ppg(s->dev, s->pb, cur, P, s->d_ctr, slots, st);
            }
            launches += 4 * kItersPerGraph;
            ck(cudaMemcpyAsync(s->h_ctr, s->d_ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st), "read counters");
            ck(cudaStreamSynchronize(st), "render");
            check_status(s, s->h_ctr->status);
            if (s->h_ctr->n_cur == 0 && s->h_ctr->work_next >= s->h_ctr->work_total) break;
            if (round > max_rounds) throw Fail(PT_ERR_LIMIT, "guided render did not converge within the iteration bound");
        }
        total.paths += (double)s->h_ctr->stat_paths;
        total.closest_rays += (double)s->h_ctr->stat_closest;
        total.iterations += (double)s->h_ctr->stat_iters;
        total.nonfinite += (double)s->h_ctr->stat_nonfinite;
        total.film_overflow += (double)s->h_ctr->stat_film_overflow;
        if (l + 1 == passes.size()) {
            launch_film_resolve(s->film, d_dst ? d_dst : s->d_out, film_n, 1.0 / (double)passes[l], st);
            launches += 1;
        }
        std::vector<float> hv(std::max(1, f.n_value_slots)), hr(std::max(1, n_dtree));
        std::vector<int32_t> hc(std::max(1, n_dtree));
        ck(cudaMemcpyAsync(hv.data(), T.slot_value, sizeof(float) * hv.size(), cudaMemcpyDeviceToHost, st), "copy");
        ck(cudaMemcpyAsync(hc.data(), T.dtree_count, sizeof(int) * hc.size(), cudaMemcpyDeviceToHost, st), "copy");
        ck(cudaMemcpyAsync(hr.data(), T.dtree_rad, sizeof(float) * hr.size(), cudaMemcpyDeviceToHost, st), "copy");
        ck(cudaStreamSynchronize(st), "copy tree");
        tree.accumulate(hv.data(), hc.data(), hr.data());
        tree.update();
    }
    ck(cudaEventRecord(s->ev1, st), "event");
    ck(cudaStreamSynchronize(st), "render");
    ck(cudaGetLastError(), "render kernels");
    float ms = 0;
    ck(cudaEventElapsedTime(&ms, s->ev0, s->ev1), "elapsed");
    total.render_ms = ms;
    total.kernel_launches = launches;
    s->stats = total;
    check_film(total.film_overflow);
}

// ---------------------------------------------------------------------------
// Learned guide: network state and the NN / unbiased-MIS render driver
// ---------------------------------------------------------------------------
constexpr int kNNBatch = 1 << 18;               // largest training batch (records per Adam step)
constexpr int kNNRecordCap = 16 * kNNBatch;  // record buffer: 2^22 records (64 B each, 268 MB)
constexpr int kNNWeightCount = 3 * 64 * 64 + 64 * 48;
static_assert(kNNWeightCount == PT_NN_WEIGHTS, "weight count");
static_assert(PT_FLAG_THROUGHPUT_RR == 16, "mirrored by PT_FLAG_THROUGHPUT_RR_ in shade.cuh");

std::vector<float> nn_random_weights(uint32_t seed) {
    // He initialisation for the ReLU layers, a smaller output layer
    std::mt19937 g(seed);
    std::vector<float> w(kNNWeightCount);
    for (int l = 0; l < 4; l++) {
        const int nout = l == 3 ? 48 : 64;
        const float sd = l == 3 ? 0.05f : std::sqrt(2.0f / 64.0f);
        std::normal_distribution<float> nd(0.0f, sd);
        for (int k = 0; k < 64 * nout; k++) w[l * 64 * 64 + k] = nd(g);
    }
    return w;
}

void nn_alloc(std::vector<void*>& owned, NNWeights* W, NNTrainBuf* TB, float** grad, float** scalars, int cap) {
    W->master = dalloc<float>(owned, kNNWeightCount);
    W->m = dalloc<float>(owned, kNNWeightCount);
    W->v = dalloc<float>(owned, kNNWeightCount);
    W->wt = dalloc<__nv_bfloat16>(owned, nn_wcopy_elems());
    W->w = dalloc<__nv_bfloat16>(owned, nn_wcopy_elems());
    if (TB) {
        TB->cap = cap;
        TB->act = dalloc<__nv_bfloat16>(owned, (size_t)4 * cap * 64);
        TB->grad = dalloc<__nv_bfloat16>(owned, (size_t)4 * cap * 64);
    }
    *grad = dalloc<float>(owned, kNNWeightCount);
    *scalars = dalloc<float>(owned, 4);
    ck(nn_set_smem_limits(), "nn shared memory limits");
}

void nn_upload(const NNWeights& W, const float* host, cudaStream_t st) {
    ck(cudaMemcpyAsync(W.master, host, sizeof(float) * kNNWeightCount, cudaMemcpyHostToDevice, st), "nn upload");
    ck(cudaMemsetAsync(W.m, 0, sizeof(float) * kNNWeightCount, st), "memset");
    ck(cudaMemsetAsync(W.v, 0, sizeof(float) * kNNWeightCount, st), "memset");
    ck(cudaMemsetAsync(W.wt, 0, sizeof(__nv_bfloat16) * nn_wcopy_elems(), st), "memset");
    ck(cudaMemsetAsync(W.w, 0, sizeof(__nv_bfloat16) * nn_wcopy_elems(), st), "memset");
    launch_nn_pack(W, st);
}

void nn_ensure(pt_scene* s) {
    if (s->nn_ready) return;
    nn_alloc(s->nn_owned, &s->nnw, &s->nn_tb, &s->nn_grad, &s->nn_scalars, kNNBatch);
    for (int k = 0; k < 2; k++) {
        s->nn_rec_buf[k] = dalloc<float4>(s->nn_owned, (size_t)kNNRecordCap * 4);
        if (!s->nn_read_done[k])
            ck(cudaEventCreateWithFlags(&s->nn_read_done[k], cudaEventDisableTiming), "cudaEventCreate");
    }
    s->nn_rec_cur = 0;
    s->nn_rec = s->nn_rec_buf[0];
    if (!s->nn_tst) ck(cudaStreamCreateWithFlags(&s->nn_tst, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!s->nn_ev_records) ck(cudaEventCreateWithFlags(&s->nn_ev_records, cudaEventDisableTiming), "cudaEventCreate");
    s->nn_rec_count = 0;
    if (!s->h_rec_left) ck(cudaMallocHost(&s->h_rec_left, sizeof(int)), "cudaMallocHost");
    if (!s->h_scal) ck(cudaMallocHost(&s->h_scal, sizeof(float) * 4), "cudaMallocHost");
    if (!s->h_tasks)
        ck(cudaMallocHost(&s->h_tasks, sizeof(NNTrainTask) * kNNMaxStepsPerRound * kNNMaxPasses), "cudaMallocHost");
    s->d_tasks = dalloc<NNTrainTask>(s->nn_owned, kNNMaxStepsPerRound * kNNMaxPasses);
    std::vector<float> w = nn_random_weights(12345u);
    nn_upload(s->nnw, w.data(), s->stream);
    ck(cudaStreamSynchronize(s->stream), "nn init");
    s->nn_ready = true;
    s->nn_steps = 0;
}

NNNorm scene_norm(const pt_scene* s) {
    NNNorm N;
    for (int k = 0; k < 3; k++) {
        const float ext = std::max(s->bounds_hi[k] - s->bounds_lo[k], 1e-6f);
        N.lo[k] = s->bounds_lo[k];
        N.inv_ext[k] = 1.0f / ext;
    }
    N.c_lo = s->nn_cfg.bsdf_frac_min;
    N.c_hi = s->nn_cfg.bsdf_frac_max;
    N.encoding = s->nn_cfg.encoding;
    return N;
}

// Per-path buffers of the slot-based wavefront, kept by the scene and grown
// on demand (capacity paths; vertex records for `depth` vertices per path
// when training; guide parameters when the guide is used).
NNPathData nn_path_buffers(pt_scene* s, int capacity, int depth) {
    const bool grow = capacity > s->nnpd_cap || depth > s->nnpd_depth;
    if (grow) {
        for (void* p : s->nnpd_owned) cudaFree(p);
        s->nnpd_owned.clear();
        s->nnpd = NNPathData{};
        s->nn_params = nullptr;
        s->nnpd_cap = std::max(capacity, s->nnpd_cap);
        s->nnpd_depth = std::max(depth, s->nnpd_depth);
        const int cap = s->nnpd_cap;
        s->nnpd.vert = dalloc<float4>(s->nnpd_owned, (size_t)cap * std::max(1, s->nnpd_depth) * kNNVertFloat4);
        s->nnpd.acc = dalloc<float4>(s->nnpd_owned, cap);
        s->nnpd.slot_stack = dalloc<int>(s->nnpd_owned, cap);
        s->nnpd.slot_job = dalloc<int>(s->nnpd_owned, cap);
        s->nnpd.fin = dalloc<int4>(s->nnpd_owned, cap);
        s->nn_params = dalloc<float4>(s->nnpd_owned, (size_t)cap * kNNMixF4);
    }
    return s->nnpd;
}

// Overlapped training rounds of one or several scenes' guides (declared
// in host_internal.h): every scene's step j runs in the same fused launch.
void train_finish(NNTrainPending& P) {
    if (P.sc.empty()) return;
    ck(cudaStreamSynchronize(P.tst), "train");
    for (size_t k = 0; k < P.sc.size(); k++) {
        pt_scene* s = P.sc[k];
        uint32_t tstat;
        std::memcpy(&tstat, &s->h_scal[2], sizeof(tstat));
        check_status(s, tstat);
        s->nn_last_loss = s->h_scal[0];
        s->nn_records += (double)P.steps[k] * s->nn_cfg.batch;  // P.steps: batches trained on
    }
    P.sc.clear();
    P.steps.clear();
}

void train_enqueue(pt_scene* const* sc, const int* held, const int* caps, int* const* d_count, int n,
                   NNTrainTask* d_tasks, NNTrainTask* h_tasks, int num_sms, cudaStream_t st, cudaStream_t tst,
                   cudaEvent_t ev_records, double* launches, int* left, NNTrainPending& P) {
    train_finish(P);  // h_tasks, h_scal and the pinned counts are free again
    const NNAdam opt;
    // steps[k] = full batches x passes; step j of scene k uses batch j / passes
    std::vector<int> steps(n, 0), batches(n, 0);
    int max_steps = 0;
    for (int k = 0; k < n; k++) {
        left[k] = -1;
        if (!sc[k]) continue;
        batches[k] = std::min(held[k], caps[k]) / sc[k]->nn_cfg.batch;
        steps[k] = batches[k] * sc[k]->nn_cfg.passes;
        max_steps = std::max(max_steps, steps[k]);
    }
    if (max_steps == 0) return;
    // task table on the buffers the records are in now: step level j holds
    // the scenes with more than j steps
    std::vector<int> off(max_steps + 1, 0), max_n(max_steps, 0);
    int t = 0;
    for (int j = 0; j < max_steps; j++) {
        off[j] = t;
        for (int k = 0; k < n; k++) {
            if (steps[k] <= j) continue;
            pt_scene* s = sc[k];
            NNTrainTask& T = h_tasks[t++];
            T = NNTrainTask{};
            T.W = s->nnw;
            T.N = scene_norm(s);
            const int passes = s->nn_cfg.passes;
            T.rec = s->nn_rec + (size_t)4 * (j / passes) * s->nn_cfg.batch;
            T.n = s->nn_cfg.batch;
            T.prep = j % passes == 0 ? 1 : 0;  // later passes reuse the batch's prepared T and its sum
            T.chi2 = s->nn_cfg.divergence == PT_NN_CHI2 ? 1 : 0;
            T.scal = s->nn_scalars;
            T.TB = s->nn_tb;
            T.grad = s->nn_grad;
            T.lr = s->nn_cfg.learning_rate;
            const int step = s->nn_steps + j + 1;
            T.bc1 = 1.0f - powf(opt.b1, (float)step);
            T.bc2 = 1.0f - powf(opt.b2, (float)step);
            max_n[j] = std::max(max_n[j], T.n);
        }
    }
    off[max_steps] = t;
    // training waits for the round's records
    ck(cudaEventRecord(ev_records, st), "event");
    ck(cudaStreamWaitEvent(tst, ev_records, 0), "wait records");
    ck(cudaMemcpyAsync(d_tasks, h_tasks, sizeof(NNTrainTask) * t, cudaMemcpyHostToDevice, tst), "training tasks");
    for (int k = 0; k < n; k++)
        if (steps[k] > 0) ck(cudaMemsetAsync(sc[k]->nn_scalars + 2, 0, sizeof(float), tst), "memset status");
    bool oneblob = false;
    for (int k = 0; k < n; k++) oneblob = oneblob || (sc[k] && sc[k]->nn_cfg.encoding == PT_NN_ENC_ONEBLOB);
    for (int j = 0; j < max_steps; j++) {
        launch_nn_train_tasks(d_tasks + off[j], off[j + 1] - off[j], max_n[j], num_sms, tst, true, true, oneblob);
        if (launches) *launches += 5;
    }
    P.tst = tst;
    for (int k = 0; k < n; k++) {
        if (steps[k] == 0) continue;
        pt_scene* s = sc[k];
        const int batch = s->nn_cfg.batch, cur = s->nn_rec_cur, nxt = 1 - cur;
        ck(cudaMemcpyAsync(s->h_scal, s->nn_scalars, sizeof(float) * 4, cudaMemcpyDeviceToHost, tst), "copy");
        ck(cudaEventRecord(s->nn_read_done[cur], tst), "event");
        // the render stream continues in the other buffer once the training
        // that last read it has finished; the records after the last full
        // batch go to its front (this round's training does not read them)
        const int kept = std::min(held[k], caps[k]) - batches[k] * batch;
        ck(cudaStreamWaitEvent(st, s->nn_read_done[nxt], 0), "wait training");
        if (kept > 0)
            ck(cudaMemcpyAsync(s->nn_rec_buf[nxt], s->nn_rec_buf[cur] + (size_t)4 * batches[k] * batch,
                               sizeof(float4) * 4 * kept, cudaMemcpyDeviceToDevice, st), "keep records");
        *s->h_rec_left = kept;
        ck(cudaMemcpyAsync(d_count[k], s->h_rec_left, sizeof(int), cudaMemcpyHostToDevice, st), "records");
        s->nn_rec_cur = nxt;
        s->nn_rec = s->nn_rec_buf[nxt];
        s->nn_steps += steps[k];
        left[k] = kept;
        P.sc.push_back(s);
        P.steps.push_back(batches[k]);
    }
}

// PT + NEE + MIS on the slot-based wavefront (nn.cu).  guided: the learned
// mixture is sampled and trained online; otherwise the same estimator with
// the BSDF alone (PT_FLAG_UNBIASED_MIS).
void render_nn(pt_scene* s, const pt_render_desc* desc, float* d_dst, bool guided) {
    cudaStream_t st = s->stream;
    const bool train = guided && !(desc->flags & PT_FLAG_NN_FREEZE);
    if (guided) nn_ensure(s);
    if (s->nn_tst) ck(cudaStreamSynchronize(s->nn_tst), "train");  // nothing of an earlier call is left queued
    RenderParams P{};
    P.spp = desc->spp;
    int ax = (int)std::lround(std::sqrt((double)desc->spp));
    P.spp_axis = (ax * ax == desc->spp) ? ax : 0;
    P.max_depth = desc->max_depth;
    P.rr_start = desc->rr_start;
    P.seed = desc->seed;
    P.width = s->width;
    P.height = s->height;
    P.flags = desc->flags;
    const unsigned long long total = (unsigned long long)s->width * s->height * (unsigned long long)desc->spp;
    const int film_n = 3 * s->width * s->height;
    const int capacity =
        ensure_wave(s, (int)std::min<unsigned long long>(1 << CPPPT_NN_WAVE_LOG2, (total + 1023) / 1024 * 1024), film_n);
    NNPathData PD = nn_path_buffers(s, capacity, train ? P.max_depth : 0);
    const int batch = s->nn_cfg.batch;
    const int rec_cap = std::min(kNNRecordCap, s->nn_cfg.steps_per_round * batch);
    PD.rec_cap = train ? rec_cap : 0;
    float4* params = guided ? s->nn_params : nullptr;
    const NNNorm N = scene_norm(s);
    // one-entry job tables (render parameters; the scene's network and records)
    *s->h_job = single_job(s->dev, P);
    DevNNJob& nj = *s->h_nnjob;
    nj = DevNNJob{};
    nj.wt = guided ? s->nnw.wt : nullptr;
    for (int k = 0; k < 3; k++) { nj.lo[k] = N.lo[k]; nj.inv_ext[k] = N.inv_ext[k]; }
    nj.c_lo = N.c_lo;
    nj.c_hi = N.c_hi;
    nj.encoding = N.encoding;
    nj.rec = train ? s->nn_rec : nullptr;
    nj.rec_cap = train ? rec_cap : 0;
    nj.n_rec = &s->d_ctr->n_rec;
    nj.keep = s->nn_keep;
    ck(cudaMemcpyAsync(s->d_job, s->h_job, sizeof(DevBatchJob), cudaMemcpyHostToDevice, st), "job table");
    ck(cudaMemcpyAsync(s->d_nnjob, s->h_nnjob, sizeof(DevNNJob), cudaMemcpyHostToDevice, st), "guide job table");
    ck(cudaEventRecord(s->ev0, st), "event");
    ck(cudaMemsetAsync(s->film, 0, sizeof(unsigned long long) * film_n, st), "memset film");
    launch_init_slots(PD.slot_stack, capacity, st);
    WaveCounters init{};
    init.work_total = total;
    init.free_top = capacity;
    init.n_rec = train ? s->nn_rec_count : 0;
    init.film_safe = film_safe_bound((double)desc->spp * (2.0 * desc->max_depth + 2.0));
    *s->h_ctr = init;
    ck(cudaMemcpyAsync(s->d_ctr, s->h_ctr, sizeof(WaveCounters), cudaMemcpyHostToDevice, st), "init counters");
    launch_nn_generate(s->dev, s->pb, 1, s->d_ctr, PD, s->d_job, 1, st);
    double launches = 3;
    const unsigned long long max_rounds =
        64 + (total / (unsigned long long)capacity + 2) * (unsigned long long)(desc->max_depth + 2) * 4 / kItersPerGraph;
    double records = 0;
    int rec_left = -1;  // records kept after the last round's training (-1: that round did not train)
    int n0 = init.n_rec;  // records held when the round started
    NNTrainPending pending;
    for (unsigned long long round = 0;; round++) {
        for (int k = 0; k < kItersPerGraph; k++) {
            const int cur = k & 1;
            launch_extend(s->dev, s->pb, cur, s->d_ctr, s->num_sms, st);
            if (guided)
                launch_nn_infer(s->dev, s->pb, cur, s->d_ctr, s->d_nnjob, params, s->num_sms, st,
                                s->nn_cfg.encoding == PT_NN_ENC_ONEBLOB);
            launch_nn_shade(s->dev, s->pb, cur, P, s->d_ctr, s->film, params, PD, guided, s->d_job, st);
            launch_nn_shadow(s->dev, s->pb, s->d_ctr, s->film, PD, s->d_job, s->num_sms, st);
            launch_nn_finish(PD, s->d_ctr, s->d_nnjob, P.max_depth, capacity, st);
            launch_nn_generate(s->dev, s->pb, cur, s->d_ctr, PD, s->d_job, 1, st);
            launches += guided ? 7 : 6;
        }
        ck(cudaMemcpyAsync(s->h_ctr, s->d_ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st), "read counters");
        ck(cudaStreamSynchronize(st), "render");
        check_status(s, s->h_ctr->status);
        rec_left = -1;
        if (train) {
            // the paths' share that leaves records, set so that a round's
            // records (sampled evenly over its paths) fill about 80 % of
            // the round's quota
            const int got = s->h_ctr->n_rec - n0;
            const double q = (double)s->nn_keep * 0.8 * rec_cap / std::max(1, got);
            s->nn_keep = (float)std::min(1.0, std::max(1.0 / 1024.0, q));
            nj.keep = s->nn_keep;
        }
        if (train && s->h_ctr->n_rec >= batch) {
            // this round's full batches train on the training stream while
            // the next round fills the other record buffer
            int* d_count = &s->d_ctr->n_rec;
            train_enqueue(&s, &s->h_ctr->n_rec, &rec_cap, &d_count, 1, s->d_tasks, s->h_tasks, s->num_sms, st,
                          s->nn_tst, s->nn_ev_records, &launches, &rec_left, pending);
            records += (double)(std::min(s->h_ctr->n_rec, rec_cap) - rec_left);
            nj.rec = s->nn_rec;
        }
        if (train)
            ck(cudaMemcpyAsync(s->d_nnjob, s->h_nnjob, sizeof(DevNNJob), cudaMemcpyHostToDevice, st),
               "guide job table");
        n0 = rec_left >= 0 ? rec_left : s->h_ctr->n_rec;
        if (s->h_ctr->n_cur == 0 && s->h_ctr->work_next >= s->h_ctr->work_total) break;
        if (round > max_rounds) throw Fail(PT_ERR_LIMIT, "render did not converge within the iteration bound");
    }
    if (train) s->nn_rec_count = rec_left >= 0 ? rec_left : std::min(s->h_ctr->n_rec, rec_cap);
    train_finish(pending);  // the network is complete before the render returns
    launch_film_resolve(s->film, d_dst ? d_dst : s->d_out, film_n, 1.0 / (double)desc->spp, st);
    ck(cudaEventRecord(s->ev1, st), "event");
    ck(cudaStreamSynchronize(st), "render");
    ck(cudaGetLastError(), "render kernels");
    float ms = 0;
    ck(cudaEventElapsedTime(&ms, s->ev0, s->ev1), "elapsed");
    pt_render_stats& R = s->stats;
    R = pt_render_stats{};
    R.paths = (double)s->h_ctr->stat_paths;
    R.closest_rays = (double)s->h_ctr->stat_closest;
    R.shadow_rays = (double)s->h_ctr->stat_shadow;
    R.iterations = (double)s->h_ctr->stat_iters;
    R.render_ms = ms;
    R.kernel_launches = launches + 1;
    R.nonfinite = (double)s->h_ctr->stat_nonfinite;
    R.film_overflow = (double)s->h_ctr->stat_film_overflow;
    (void)records;
    check_film(R.film_overflow);
}

void render_impl(pt_scene* s, const pt_render_desc* desc, float* d_dst) {
    if (!desc) throw std::invalid_argument("null render description");
    if (desc->spp < 1) throw std::invalid_argument("spp must be >= 1");
    if (desc->max_depth < 1 || desc->max_depth > 0xffff) throw std::invalid_argument("max_depth must be in [1, 65535]");
    if (desc->mode == PT_MODE_NN) {
        if (desc->flags & ~(PT_FLAG_NN_FREEZE | PT_FLAG_UNBIASED_MIS | PT_FLAG_THROUGHPUT_RR))
            throw Fail(PT_ERR_INVALID, "unsupported flags for the learned-guide render");
        render_nn(s, desc, d_dst, true);
        return;
    }
    if (desc->mode == PT_MODE_MIS && (desc->flags & PT_FLAG_UNBIASED_MIS)) {
        if (desc->flags & ~(PT_FLAG_UNBIASED_MIS | PT_FLAG_THROUGHPUT_RR))
            throw Fail(PT_ERR_INVALID, "PT_FLAG_UNBIASED_MIS combines only with PT_FLAG_THROUGHPUT_RR");
        render_nn(s, desc, d_dst, false);
        return;
    }
    if (desc->flags & PT_FLAG_THROUGHPUT_RR)
        throw Fail(PT_ERR_INVALID, "PT_FLAG_THROUGHPUT_RR needs PT_MODE_NN or PT_FLAG_UNBIASED_MIS");
    if (desc->mode == PT_MODE_SDTREE) {
        if (desc->flags != 0) throw Fail(PT_ERR_INVALID, "flags are not supported by the SD-tree guided render");
        render_ppg(s, desc, d_dst);
        return;
    }
    if (desc->mode != PT_MODE_MIS && desc->mode != PT_MODE_NEE && desc->mode != PT_MODE_PT)
        throw Fail(PT_ERR_INVALID, "unknown render mode");
    RenderParams P{};
    P.spp = desc->spp;
    int ax = (int)std::lround(std::sqrt((double)desc->spp));
    P.spp_axis = (ax * ax == desc->spp) ? ax : 0;
    P.max_depth = desc->max_depth;
    P.rr_start = desc->rr_start;
    P.seed = desc->seed;
    P.width = s->width;
    P.height = s->height;
    const unsigned long long total = (unsigned long long)s->width * s->height * (unsigned long long)desc->spp;
    const int film_n = 3 * s->width * s->height;
    const int capacity =
        ensure_wave(s, (int)std::min<unsigned long long>(kMaxCapacity, (total + 1023) / 1024 * 1024), film_n);
    cudaStream_t st = s->stream;
    const bool timed = (desc->flags & PT_FLAG_TIME_KERNELS) != 0;
    const bool count = (desc->flags & PT_FLAG_COUNT) != 0;
    const bool direct = timed || count;
    // the render parameters live in the scene's one-entry job table and the
    // counters, so the graph stays valid across renders
    if (!direct && !s->graph)
        ck(build_render_graph(s->dev, s->pb, s->d_ctr, s->film, s->d_job, 1, kItersPerGraph, s->num_sms, st,
                              &s->graph),
           "render graph");
    ck(cudaEventRecord(s->ev0, st), "event");
    ck(cudaMemsetAsync(s->film, 0, sizeof(unsigned long long) * film_n, st), "memset film");
    const unsigned long long max_rounds = 64 + (total / (unsigned long long)capacity + 2) *
                                                   (unsigned long long)(desc->max_depth + 2) * 4 / kItersPerGraph;
    WaveCounters init{};
    init.work_total = total;
    init.film_safe = film_safe_bound((double)desc->spp * (2.0 * desc->max_depth + 2.0));
    init.max_rounds = (uint32_t)std::min<unsigned long long>(max_rounds, 0xffffffffull);
    *s->h_ctr = init;
    ck(cudaMemcpyAsync(s->d_ctr, s->h_ctr, sizeof(WaveCounters), cudaMemcpyHostToDevice, st), "init counters");
    *s->h_job = single_job(s->dev, P);
    s->h_job->integrator = desc->mode == PT_MODE_NEE ? kIntegratorNEE
                           : desc->mode == PT_MODE_PT ? kIntegratorPT : kIntegratorMIS;
    ck(cudaMemcpyAsync(s->d_job, s->h_job, sizeof(DevBatchJob), cudaMemcpyHostToDevice, st), "job table");
    launch_generate(s->dev, s->pb, 1, s->d_ctr, s->d_job, 1, st);  // fills buffer 0
    double launches = 2;
    std::vector<cudaEvent_t> tev;
    unsigned long long rounds = 0;
    if (!direct) {
        // the whole loop on the device: one graph launch, one read of the counters
        ck(cudaGraphLaunch(s->graph, st), "graph launch");
        ck(cudaMemcpyAsync(s->h_ctr, s->d_ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st), "read counters");
        ck(cudaStreamSynchronize(st), "render");
        check_status(s, s->h_ctr->status);
        rounds = s->h_ctr->rounds;
        launches += (double)rounds * (kKernelsPerIteration * kItersPerGraph + 1);
    }
    while (direct) {
        {
            // the graph's work, launched one kernel at a time
            for (int k = 0; k < kItersPerGraph; k++) {
                const int cur = k & 1;
                cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
                if (timed)
                    for (int q = 0; q < 4; q++) { ck(cudaEventCreate(&e[q]), "event"); tev.push_back(e[q]); }
                if (timed) ck(cudaEventRecord(e[0], st), "event");
                launch_extend(s->dev, s->pb, cur, s->d_ctr, s->num_sms, st, count);
                if (timed) ck(cudaEventRecord(e[1], st), "event");
                launch_shade(s->dev, s->pb, cur, s->d_ctr, s->film, s->d_job, st);
                if (timed) ck(cudaEventRecord(e[2], st), "event");
                launch_shadow(s->dev, s->pb, s->d_ctr, s->film, s->num_sms, st);
                if (timed) ck(cudaEventRecord(e[3], st), "event");
                launch_generate(s->dev, s->pb, cur, s->d_ctr, s->d_job, 1, st);
            }
        }
        launches += kKernelsPerIteration * kItersPerGraph;
        ck(cudaMemcpyAsync(s->h_ctr, s->d_ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st), "read counters");
        ck(cudaStreamSynchronize(st), "render");
        check_status(s, s->h_ctr->status);
        rounds++;
        if (s->h_ctr->n_cur == 0 && s->h_ctr->work_next >= s->h_ctr->work_total) break;
        if (rounds > max_rounds) throw Fail(PT_ERR_LIMIT, "render did not converge within the iteration bound");
    }
    launch_film_resolve(s->film, d_dst ? d_dst : s->d_out, film_n, 1.0 / (double)desc->spp, st);
    ck(cudaEventRecord(s->ev1, st), "event");
    ck(cudaStreamSynchronize(st), "render");
    ck(cudaGetLastError(), "render kernels");
    float ms = 0;
    ck(cudaEventElapsedTime(&ms, s->ev0, s->ev1), "elapsed");
    pt_render_stats& R = s->stats;
    R = pt_render_stats{};
    R.paths = (double)s->h_ctr->stat_paths;
    R.closest_rays = (double)s->h_ctr->stat_closest;
    R.shadow_rays = (double)s->h_ctr->stat_shadow;
    R.iterations = (double)s->h_ctr->stat_iters;
    R.render_ms = ms;
    R.kernel_launches = launches + 1;
    R.extend_nodes = (double)s->h_ctr->stat_nodes;
    R.extend_tris = (double)s->h_ctr->stat_tris;
    R.nonfinite = (double)s->h_ctr->stat_nonfinite;
    R.h2d_bytes = (double)sizeof(WaveCounters);
    R.d2h_bytes = (double)((direct ? rounds : 1) * sizeof(WaveCounters));
    if (timed) {
        double ext = 0, sh = 0;
        for (size_t q = 0; q + 3 < tev.size(); q += 4) {
            float a = 0, b = 0;
            cudaEventElapsedTime(&a, tev[q], tev[q + 1]);
            cudaEventElapsedTime(&b, tev[q + 2], tev[q + 3]);
            ext += a;
            sh += b;
        }
        for (cudaEvent_t e : tev) cudaEventDestroy(e);
        R.trace_closest_ms = ext;
        R.trace_shadow_ms = sh;
    }
    R.film_overflow = (double)s->h_ctr->stat_film_overflow;
    check_film(R.film_overflow);
}


// ---------------------------------------------------------------------------
// Image output (Image::save, rgb_image.h:300-318): 8-bit sRGB PNG and RGBE.
// PNG is written with stored (uncompressed) deflate blocks.
// ---------------------------------------------------------------------------
uint32_t crc32_update(uint32_t crc, const unsigned char* p, size_t n) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
    return ~crc;
}

void put_be32(std::vector<unsigned char>& v, uint32_t x) {
    v.push_back((unsigned char)(x >> 24)); v.push_back((unsigned char)(x >> 16));
    v.push_back((unsigned char)(x >> 8)); v.push_back((unsigned char)x);
}

void png_chunk(FILE* f, const char* type, const std::vector<unsigned char>& data) {
    std::vector<unsigned char> b;
    put_be32(b, (uint32_t)data.size());
    b.insert(b.end(), type, type + 4);
    b.insert(b.end(), data.begin(), data.end());
    uint32_t crc = crc32_update(0, b.data() + 4, b.size() - 4);
    put_be32(b, crc);
    fwrite(b.data(), 1, b.size(), f);
}

float linear2srgb(float a) { return a > 0.0031308f ? 1.055f * std::pow(a, 1.0f / 2.4f) - 0.055f : 12.92f * a; }

void save_png(const std::string& path, const float* rgb, int W, int H) {
    std::vector<unsigned char> raw;
    raw.reserve((size_t)H * (3 * W + 1));
    for (int j = 0; j < H; j++) {
        raw.push_back(0);
        for (int i = 0; i < 3 * W; i++) {
            float a = linear2srgb(rgb[(size_t)j * 3 * W + i]);
            if (!(a > 0.0f)) a = 0.0f;  // put2char1 (rgb_image.h:23-35)
            if (a >= 0.99999f) a = 0.99999f;
            raw.push_back((unsigned char)(unsigned int)(a * 255.0f));
        }
    }
    std::vector<unsigned char> z = {0x78, 0x01};
    uint32_t s1 = 1, s2 = 0;
    for (unsigned char c : raw) { s1 = (s1 + c) % 65521; s2 = (s2 + s1) % 65521; }
    size_t pos = 0;
    do {
        size_t len = std::min<size_t>(65535, raw.size() - pos);
        z.push_back(pos + len == raw.size() ? 1 : 0);
        z.push_back((unsigned char)(len & 0xff)); z.push_back((unsigned char)(len >> 8));
        z.push_back((unsigned char)(~len & 0xff)); z.push_back((unsigned char)((~len >> 8) & 0xff));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    put_be32(z, (s2 << 16) | s1);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Fail(PT_ERR_IO, "cannot write " + path);
    const unsigned char sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    fwrite(sig, 1, 8, f);
    std::vector<unsigned char> ihdr;
    put_be32(ihdr, (uint32_t)W);
    put_be32(ihdr, (uint32_t)H);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
    png_chunk(f, "IHDR", ihdr);
    png_chunk(f, "IDAT", z);
    png_chunk(f, "IEND", {});
    std::fclose(f);
}

void save_hdr(const std::string& path, const float* rgb, int W, int H) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Fail(PT_ERR_IO, "cannot write " + path);
    std::fprintf(f, "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n", H, W);
    std::vector<unsigned char> row(4 * (size_t)W);
    for (int j = 0; j < H; j++) {
        for (int i = 0; i < W; i++) {
            const float* p = rgb + 3 * ((size_t)j * W + i);
            float m = std::max(p[0], std::max(p[1], p[2]));
            unsigned char* o = &row[4 * (size_t)i];
            if (!(m >= 1e-32f)) { o[0] = o[1] = o[2] = o[3] = 0; continue; }
            int e;
            float scale = std::frexp(m, &e) * 256.0f / m;
            o[0] = (unsigned char)std::max(0.0f, p[0] * scale);
            o[1] = (unsigned char)std::max(0.0f, p[1] * scale);
            o[2] = (unsigned char)std::max(0.0f, p[2] * scale);
            o[3] = (unsigned char)(e + 128);
        }
        fwrite(row.data(), 1, row.size(), f);
    }
    std::fclose(f);
}

}  // namespace

// The learned-guide helpers above, for the multi-scene batch (batch.cpp).
namespace cpppt_gb300 {
namespace hostimpl {
void nn_ensure_scene(pt_scene* s) { nn_ensure(s); }
NNNorm nn_scene_norm(const pt_scene* s) { return scene_norm(s); }
int nn_record_cap(const pt_scene* s) { return std::min(kNNRecordCap, s->nn_cfg.steps_per_round * s->nn_cfg.batch); }
void nn_train_enqueue(pt_scene* const* scenes, const int* held, const int* caps, int* const* d_count, int n,
                      NNTrainTask* d_tasks, NNTrainTask* h_tasks, int num_sms, cudaStream_t st, cudaStream_t tst,
                      cudaEvent_t ev_records, double* launches, int* left, NNTrainPending& pending) {
    train_enqueue(scenes, held, caps, d_count, n, d_tasks, h_tasks, num_sms, st, tst, ev_records, launches, left,
                  pending);
}
void nn_train_finish(NNTrainPending& pending) { train_finish(pending); }
}  // namespace hostimpl
}  // namespace cpppt_gb300


extern "C" {

pt_status scene_create_with(const pt_scene_desc* desc, const SceneTextures* tx, pt_scene** out) {
    if (!out) { g_error = "null output pointer"; return PT_ERR_INVALID; }
    *out = nullptr;
    pt_scene* s = new (std::nothrow) pt_scene();
    if (!s) { g_error = "host allocation failed"; return PT_ERR_MEMORY; }
    pt_status st = guarded([&] { create_scene(desc, s, tx); });
    if (st != PT_OK) { delete s; return st; }
    *out = s;
    return PT_OK;
}

pt_status pt_scene_create(const pt_scene_desc* desc, pt_scene** out) { return scene_create_with(desc, nullptr, out); }

pt_status pt_scene_load(const char* settings_file, pt_scene** out, pt_render_desc* settings, char* output_name,
                        int32_t output_name_len) {
    if (!out || !settings_file) { g_error = "null argument"; return PT_ERR_INVALID; }
    *out = nullptr;
    LoadedScene L;
    pt_render_desc rs{};
    std::string output;
    pt_status st = guarded([&] { load_files(settings_file, L, &rs, output); });
    if (st != PT_OK) return st;
    pt_scene_desc d{};
    d.n_vertices = (int32_t)(L.v.size() / 3);
    d.vertices = L.v.data();
    d.normals = L.n.data();
    d.tangents = L.t.data();
    d.n_triangles = (int32_t)L.tri_mat.size();
    d.triangles = L.tri.data();
    d.tri_material = L.tri_mat.data();
    d.n_materials = (int32_t)L.mats.size();
    d.materials = L.mats.data();
    d.camera = L.cam;
    st = scene_create_with(&d, &L.tx, out);
    if (st != PT_OK) return st;
    if (settings) *settings = rs;
    if (output_name && output_name_len > 0) {
        std::snprintf(output_name, (size_t)output_name_len, "%s", output.c_str());
    }
    return PT_OK;
}

void pt_scene_destroy(pt_scene* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(lifetime_mutex());
        if (s->batch_refs > 0) {  // the last batch holding the scene deletes it
            s->destroy_pending = true;
            return;
        }
    }
    delete s;
}

pt_status pt_scene_info(pt_scene* s, int32_t* width, int32_t* height, int32_t* n_triangles, int32_t* n_lights) {
    if (!s) { g_error = "null scene"; return PT_ERR_INVALID; }
    if (width) *width = s->width;
    if (height) *height = s->height;
    if (n_triangles) *n_triangles = s->n_tris;
    if (n_lights) *n_lights = s->dev.n_lights;
    return PT_OK;
}

pt_status pt_trace_closest(pt_scene* s, const pt_ray* rays, int32_t n, pt_hit* hits) {
    if (!s) { g_error = "null scene"; return PT_ERR_INVALID; }
    return guarded([&] { trace_host(s, rays, n, hits, false); });
}

pt_status pt_trace_any(pt_scene* s, const pt_ray* rays, int32_t n, uint8_t* occluded) {
    if (!s) { g_error = "null scene"; return PT_ERR_INVALID; }
    return guarded([&] { trace_host(s, rays, n, occluded, true); });
}

pt_status pt_trace_closest_device(pt_scene* s, const pt_ray* d_rays, int32_t n, pt_hit* d_hits, void* stream) {
    if (!s) { g_error = "null scene"; return PT_ERR_INVALID; }
    return guarded([&] { trace_device(s, d_rays, n, d_hits, false, static_cast<cudaStream_t>(stream)); });
}

pt_status pt_trace_any_device(pt_scene* s, const pt_ray* d_rays, int32_t n, uint8_t* d_occ, void* stream) {
    if (!s) { g_error = "null scene"; return PT_ERR_INVALID; }
    return guarded([&] { trace_device(s, d_rays, n, d_occ, true, static_cast<cudaStream_t>(stream)); });
}

pt_status pt_render(pt_scene* s, const pt_render_desc* desc, float* rgb_out) {
    if (!s || !rgb_out) { g_error = "null argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        render_impl(s, desc, nullptr);
        ck(cudaMemcpyAsync(rgb_out, s->d_out, sizeof(float) * s->film_n, cudaMemcpyDeviceToHost, s->stream), "copy image");
        ck(cudaStreamSynchronize(s->stream), "copy image");
        s->stats.d2h_bytes += (double)(sizeof(float) * s->film_n);
    });
}

pt_status pt_render_device(pt_scene* s, const pt_render_desc* desc, float* d_rgb_out) {
    if (!s || !d_rgb_out) { g_error = "null argument"; return PT_ERR_INVALID; }
    return guarded([&] { render_impl(s, desc, d_rgb_out); });
}

// For callers that must not allocate device memory during a render (see the
// header): same wavefront and same image as pt_render_device, scratch in the
// library's fixed __device__ array.  The scene (created earlier) is read only.
pt_status pt_render_device_noalloc(pt_scene* s, const pt_render_desc* desc, float* d_rgb_out, void* stream) {
    if (!s || !d_rgb_out) { g_error = "null argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        if (!desc) throw std::invalid_argument("null render description");
        if (desc->spp < 1) throw std::invalid_argument("spp must be >= 1");
        if (desc->max_depth < 1 || desc->max_depth > 0xffff)
            throw std::invalid_argument("max_depth must be in [1, 65535]");
        if (desc->mode != PT_MODE_MIS) throw Fail(PT_ERR_INVALID, "the allocation-free render supports PT_MODE_MIS only");
        if (desc->flags != 0) throw Fail(PT_ERR_INVALID, "the allocation-free render takes no flags");
        int cur_dev = -1;
        ck(cudaGetDevice(&cur_dev), "cudaGetDevice");
        if (cur_dev != s->device)
            throw Fail(PT_ERR_INVALID, "the scene was created on device " + std::to_string(s->device) +
                                       " but device " + std::to_string(cur_dev) + " is current");
        const long long pixels = (long long)s->width * s->height;
        if (pixels > noalloc_max_pixels())
            throw Fail(PT_ERR_LIMIT, "image of " + std::to_string(pixels) + " pixels exceeds the allocation-free render's "
                                     "maximum of " + std::to_string(noalloc_max_pixels()) + " pixels");
        RenderParams P{};
        P.spp = desc->spp;
        int ax = (int)std::lround(std::sqrt((double)desc->spp));
        P.spp_axis = (ax * ax == desc->spp) ? ax : 0;
        P.max_depth = desc->max_depth;
        P.rr_start = desc->rr_start;
        P.seed = desc->seed;
        P.width = s->width;
        P.height = s->height;
        WaveCounters h{};
        int limit = 0;
        ck(render_noalloc(s->dev, P, s->num_sms, desc->max_depth, d_rgb_out, static_cast<cudaStream_t>(stream), &h,
                          &limit),
           "allocation-free render");
        pt_render_stats R{};
        R.paths = (double)h.stat_paths;
        R.closest_rays = (double)h.stat_closest;
        R.shadow_rays = (double)h.stat_shadow;
        R.iterations = (double)h.stat_iters;
        R.nonfinite = (double)h.stat_nonfinite;
        R.film_overflow = (double)h.stat_film_overflow;
        s->stats = R;
        check_film(R.film_overflow);
        check_status(s, h.status);
        if (limit) throw Fail(PT_ERR_LIMIT, "render did not converge within the iteration bound");
    });
}

pt_status pt_nn_get_weights(pt_scene* s, float* w) {
    if (!s || !w) { g_error = "null argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        nn_ensure(s);
        ck(cudaMemcpyAsync(w, s->nnw.master, sizeof(float) * kNNWeightCount, cudaMemcpyDeviceToHost, s->stream), "copy");
        ck(cudaStreamSynchronize(s->stream), "copy");
    });
}

pt_status pt_nn_set_weights(pt_scene* s, const float* w) {
    if (!s || !w) { g_error = "null argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        nn_ensure(s);
        nn_upload(s->nnw, w, s->stream);
        ck(cudaStreamSynchronize(s->stream), "upload");
        s->nn_steps = 0;
    });
}

pt_status pt_nn_reset(pt_scene* s, uint32_t seed) {
    if (!s) { g_error = "null argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        nn_ensure(s);
        std::vector<float> w = nn_random_weights(seed);
        nn_upload(s->nnw, w.data(), s->stream);
        ck(cudaStreamSynchronize(s->stream), "upload");
        s->nn_steps = 0;
        s->nn_last_loss = 0;
        s->nn_records = 0;
        s->nn_rec_count = 0;
        s->nn_keep = 1.0f;
    });
}

pt_status pt_nn_configure(pt_scene* s, const pt_nn_config* c) {
    if (!s || !c) { g_error = "null argument"; return PT_ERR_INVALID; }
    if (!(c->learning_rate > 0.f) || !(c->learning_rate < 1.f)) {
        g_error = "learning_rate must be in (0, 1)";
        return PT_ERR_INVALID;
    }
    if (!(c->bsdf_frac_min >= 0.1f) || !(c->bsdf_frac_max >= c->bsdf_frac_min) || !(c->bsdf_frac_max <= 1.f)) {
        g_error = "need 0.1 <= bsdf_frac_min <= bsdf_frac_max <= 1";
        return PT_ERR_INVALID;
    }
    if (c->batch < 1024 || c->batch > kNNBatch) {
        g_error = "batch must be in [1024, 262144]";
        return PT_ERR_INVALID;
    }
    if (c->divergence != PT_NN_KL && c->divergence != PT_NN_CHI2) {
        g_error = "divergence must be PT_NN_KL or PT_NN_CHI2";
        return PT_ERR_INVALID;
    }
    if (c->steps_per_round < 1 || c->steps_per_round > kNNMaxStepsPerRound) {
        g_error = "steps_per_round must be in [1, 64]";
        return PT_ERR_INVALID;
    }
    if (c->encoding != PT_NN_ENC_FREQ && c->encoding != PT_NN_ENC_ONEBLOB) {
        g_error = "encoding must be PT_NN_ENC_FREQ or PT_NN_ENC_ONEBLOB";
        return PT_ERR_INVALID;
    }
    if (c->passes < 1 || c->passes > kNNMaxPasses) {
        g_error = "passes must be in [1, 8]";
        return PT_ERR_INVALID;
    }
    s->nn_cfg = *c;
    s->nn_rec_count = 0;  // records of the previous batch size are dropped
    s->nn_keep = 1.0f;
    return PT_OK;
}

pt_status pt_nn_config_get(pt_scene* s, pt_nn_config* c) {
    if (!s || !c) { g_error = "null argument"; return PT_ERR_INVALID; }
    *c = s->nn_cfg;
    return PT_OK;
}

pt_status pt_nn_stats(pt_scene* s, double* steps, double* last_loss, double* records_used) {
    if (!s) { g_error = "null argument"; return PT_ERR_INVALID; }
    if (steps) *steps = s->nn_steps;
    if (last_loss) *last_loss = s->nn_last_loss;
    if (records_used) *records_used = s->nn_records;
    return PT_OK;
}

namespace {
struct DebugCtx {
    cudaStream_t st = nullptr;
    std::vector<void*> owned;
    int sms = 0;
    DebugCtx() {
        int dev = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        cudaDeviceProp prop;
        ck(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
        if (prop.major * 10 + prop.minor != 103) throw Fail(PT_ERR_NO_DEVICE, "not a compute capability 10.3 device");
        sms = prop.multiProcessorCount;
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    }
    ~DebugCtx() {
        if (st) cudaStreamSynchronize(st);
        for (void* p : owned) cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
};
NNNorm norm_from(const float* lo, const float* hi) {
    NNNorm N;
    for (int k = 0; k < 3; k++) {
        N.lo[k] = lo[k];
        N.inv_ext[k] = 1.0f / std::max(hi[k] - lo[k], 1e-6f);
    }
    return N;
}
}  // namespace

pt_status pt_debug_nn_forward_ex(const float* weights, const float* lo, const float* hi, const float* inputs,
                                 int32_t n, int32_t encoding, float* out) {
    if (!weights || !lo || !hi || n < 0 || (n > 0 && (!inputs || !out))) { g_error = "bad argument"; return PT_ERR_INVALID; }
    if (encoding != PT_NN_ENC_FREQ && encoding != PT_NN_ENC_ONEBLOB) { g_error = "unknown encoding"; return PT_ERR_INVALID; }
    return guarded([&] {
        if (n == 0) return;
        DebugCtx c;
        NNWeights W;
        NNTrainBuf* none = nullptr;
        float *grad, *scal;
        nn_alloc(c.owned, &W, none, &grad, &scal, 0);
        nn_upload(W, weights, c.st);
        float* din = dalloc<float>(c.owned, (size_t)9 * n);
        float* dout = dalloc<float>(c.owned, (size_t)41 * n);
        uint32_t* dstat = dalloc<uint32_t>(c.owned, 1);
        ck(cudaMemsetAsync(dstat, 0, sizeof(uint32_t), c.st), "memset");
        ck(cudaMemcpyAsync(din, inputs, sizeof(float) * 9 * n, cudaMemcpyHostToDevice, c.st), "copy");
        const NNNorm N = norm_from(lo, hi);
        DevNNJob hj{};
        hj.wt = W.wt;
        for (int k = 0; k < 3; k++) { hj.lo[k] = N.lo[k]; hj.inv_ext[k] = N.inv_ext[k]; }
        hj.c_lo = N.c_lo;
        hj.c_hi = N.c_hi;
        hj.encoding = encoding;
        DevNNJob* dj = dalloc<DevNNJob>(c.owned, 1);
        ck(cudaMemcpyAsync(dj, &hj, sizeof(hj), cudaMemcpyHostToDevice, c.st), "copy");
        launch_nn_forward_debug(dj, din, n, dout, dstat, c.sms, c.st, encoding == PT_NN_ENC_ONEBLOB);
        ck(cudaMemcpyAsync(out, dout, sizeof(float) * 41 * n, cudaMemcpyDeviceToHost, c.st), "copy");
        uint32_t hstat = 0;
        ck(cudaMemcpyAsync(&hstat, dstat, sizeof(uint32_t), cudaMemcpyDeviceToHost, c.st), "copy");
        ck(cudaStreamSynchronize(c.st), "forward");
        ck(cudaGetLastError(), "forward");
        if (hstat & kStatusTensorTimeout) throw Fail(PT_ERR_CUDA, "tensor-core completion wait timed out");
    });
}

pt_status pt_debug_traversal_limits(pt_scene* s, int32_t step_limit, int32_t stack_limit) {
    if (!s) { g_error = "null scene"; return PT_ERR_INVALID; }
    if (step_limit < 0 || (uint32_t)step_limit > kTraversalStepLimit || stack_limit < 0 ||
        stack_limit > kTraversalStackSize) {
        g_error = "limits must lie in [0, default] (0: the default)";
        return PT_ERR_INVALID;
    }
    return guarded([&] {
        ck(cudaStreamSynchronize(s->stream), "sync");
        s->dev.step_limit = step_limit ? (uint32_t)step_limit : kTraversalStepLimit;
        s->dev.stack_limit = stack_limit ? stack_limit : kTraversalStackSize;
        // the captured iteration graph holds the scene description by value
        if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
    });
}

pt_status pt_debug_tensor_wait_timeout(void) {
    return guarded([&] {
        DebugCtx c;
        uint32_t* dstat = dalloc<uint32_t>(c.owned, 1);
        ck(cudaMemsetAsync(dstat, 0, sizeof(uint32_t), c.st), "memset");
        launch_debug_tc_timeout(dstat, c.st);
        ck(cudaGetLastError(), "launch");
        uint32_t h = 0;
        ck(cudaMemcpyAsync(&h, dstat, sizeof(h), cudaMemcpyDeviceToHost, c.st), "copy");
        ck(cudaStreamSynchronize(c.st), "timeout kernel");
        if (h & kStatusTensorTimeout) throw Fail(PT_ERR_CUDA, "tensor-core completion wait timed out");
    });
}

pt_status pt_debug_bsdf(int32_t n, const float* cases, float* out) {
    if (n < 0 || (n > 0 && (!cases || !out))) { g_error = "bad argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        if (n == 0) return;
        for (int32_t i = 0; i < n; i++) {
            const float k = cases[(size_t)kDebugBsdfIn * i];
            if (!(k == 0.f || k == 1.f || k == 2.f || k == 3.f)) throw std::invalid_argument("unknown material kind");
        }
        DebugCtx c;
        float* din = dalloc<float>(c.owned, (size_t)kDebugBsdfIn * n);
        float* dout = dalloc<float>(c.owned, (size_t)kDebugBsdfOut * n);
        ck(cudaMemcpyAsync(din, cases, sizeof(float) * kDebugBsdfIn * n, cudaMemcpyHostToDevice, c.st), "copy");
        launch_debug_bsdf(din, dout, n, c.st);
        ck(cudaGetLastError(), "debug bsdf launch");
        ck(cudaMemcpyAsync(out, dout, sizeof(float) * kDebugBsdfOut * n, cudaMemcpyDeviceToHost, c.st), "copy");
        ck(cudaStreamSynchronize(c.st), "debug bsdf");
    });
}

pt_status pt_debug_light_sample(pt_scene* s, int32_t n, const float* cases, float* out) {
    if (!s || n < 0 || (n > 0 && (!cases || !out))) { g_error = "bad argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        if (n == 0) return;
        if (s->dev.n_lights <= 0) throw std::invalid_argument("the scene has no emissive triangles");
        std::vector<void*> owned;
        struct Free {
            std::vector<void*>& v;
            ~Free() { for (void* p : v) cudaFree(p); }
        } guard{owned};
        float* din = dalloc<float>(owned, (size_t)kDebugLightIn * n);
        float* dout = dalloc<float>(owned, (size_t)kDebugLightOut * n);
        ck(cudaMemcpyAsync(din, cases, sizeof(float) * kDebugLightIn * n, cudaMemcpyHostToDevice, s->stream), "copy");
        launch_debug_light(s->dev, din, dout, n, s->stream);
        ck(cudaGetLastError(), "debug light launch");
        ck(cudaMemcpyAsync(out, dout, sizeof(float) * kDebugLightOut * n, cudaMemcpyDeviceToHost, s->stream), "copy");
        ck(cudaStreamSynchronize(s->stream), "debug light");
    });
}

pt_status pt_debug_nn_forward(const float* weights, const float* lo, const float* hi, const float* inputs, int32_t n,
                              float* out) {
    return pt_debug_nn_forward_ex(weights, lo, hi, inputs, n, PT_NN_ENC_FREQ, out);
}

namespace {
// One gradient evaluation of the training kernels on a host batch.  prep:
// the renderer's own step (T summed, and squared for chi-square, on the
// device); otherwise the host sums T and the KL weights are used.
void nn_grad_debug(const float* weights, const float* lo, const float* hi, const float* records, int32_t n, bool prep,
                   int divergence, float c_lo, float c_hi, int encoding, float* out_grad, float* out_loss) {
    DebugCtx c;
    NNWeights W;
    NNTrainBuf TB;
    float *grad, *scal;
    nn_alloc(c.owned, &W, &TB, &grad, &scal, n);
    nn_upload(W, weights, c.st);
    float4* drec = dalloc<float4>(c.owned, (size_t)4 * n);
    ck(cudaMemcpyAsync(drec, records, sizeof(float) * 16 * n, cudaMemcpyHostToDevice, c.st), "copy");
    double tsum = 0;
    if (!prep)
        for (int i = 0; i < n; i++) tsum += records[16 * i + 13];
    const float sc0[4] = {0.f, (float)tsum, 0.f, 0.f};
    ck(cudaMemcpyAsync(scal, sc0, sizeof(sc0), cudaMemcpyHostToDevice, c.st), "copy");
    NNTrainTask task{};
    task.W = W;
    task.N = norm_from(lo, hi);
    task.N.c_lo = c_lo;
    task.N.c_hi = c_hi;
    task.N.encoding = encoding;
    task.rec = drec;
    task.n = n;
    task.chi2 = divergence == PT_NN_CHI2 ? 1 : 0;
    task.prep = 1;
    task.scal = scal;
    task.TB = TB;
    task.grad = grad;
    NNTrainTask* dtask = dalloc<NNTrainTask>(c.owned, 1);
    ck(cudaMemcpyAsync(dtask, &task, sizeof(task), cudaMemcpyHostToDevice, c.st), "copy");
    launch_nn_train_tasks(dtask, 1, n, c.sms, c.st, prep, false, encoding == PT_NN_ENC_ONEBLOB);
    ck(cudaMemcpyAsync(out_grad, grad, sizeof(float) * kNNWeightCount, cudaMemcpyDeviceToHost, c.st), "copy");
    float sc[4] = {0.f, 0.f, 0.f, 0.f};
    ck(cudaMemcpyAsync(sc, scal, sizeof(sc), cudaMemcpyDeviceToHost, c.st), "copy");
    ck(cudaStreamSynchronize(c.st), "grad");
    ck(cudaGetLastError(), "grad");
    uint32_t tstat;
    std::memcpy(&tstat, &sc[2], sizeof(tstat));
    if (tstat & kStatusTensorTimeout) throw Fail(PT_ERR_CUDA, "tensor-core completion wait timed out");
    if (out_loss) *out_loss = sc[0];
}
}  // namespace

pt_status pt_debug_nn_grad_ex(const float* weights, const float* lo, const float* hi, const float* records, int32_t n,
                              int32_t divergence, float c_lo, float c_hi, int32_t encoding, float* out_grad,
                              float* out_loss) {
    if (!weights || !lo || !hi || n <= 0 || !records || !out_grad) { g_error = "bad argument"; return PT_ERR_INVALID; }
    if (divergence != PT_NN_KL && divergence != PT_NN_CHI2) { g_error = "unknown divergence"; return PT_ERR_INVALID; }
    if (!(c_lo >= 0.1f && c_lo <= c_hi && c_hi <= 1.0f)) { g_error = "need 0.1 <= c_lo <= c_hi <= 1"; return PT_ERR_INVALID; }
    if (encoding != PT_NN_ENC_FREQ && encoding != PT_NN_ENC_ONEBLOB) { g_error = "unknown encoding"; return PT_ERR_INVALID; }
    return guarded([&] {
        nn_grad_debug(weights, lo, hi, records, n, true, divergence, c_lo, c_hi, encoding, out_grad, out_loss);
    });
}

pt_status pt_debug_nn_grad(const float* weights, const float* lo, const float* hi, const float* records, int32_t n,
                           float* out_grad, float* out_loss) {
    if (!weights || !lo || !hi || n <= 0 || !records || !out_grad) { g_error = "bad argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        nn_grad_debug(weights, lo, hi, records, n, false, PT_NN_KL, 0.1f, 0.9f, PT_NN_ENC_FREQ, out_grad, out_loss);
    });
}

pt_status pt_render_stats_get(pt_scene* s, pt_render_stats* out) {
    if (!s || !out) { g_error = "null argument"; return PT_ERR_INVALID; }
    *out = s->stats;
    return PT_OK;
}

void pt_set_mesh_cache(int32_t enabled) { set_mesh_cache(enabled != 0); }

pt_status pt_image_save(const char* prefix, const float* rgb, int32_t w, int32_t h) {
    if (!prefix || !rgb || w <= 0 || h <= 0) { g_error = "bad argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        save_png(std::string(prefix) + ".png", rgb, w, h);
        save_hdr(std::string(prefix) + ".hdr", rgb, w, h);
    });
}

const char* pt_last_error(void) { return g_error.c_str(); }

pt_status pt_debug_sdtree_run(const float* lo, const float* hi, int32_t n_iters, const int32_t* n_splats,
                              const float* splats, int32_t max_leaves, float* out_leaves, int32_t* out_leaf_counts,
                              int32_t* out_counts, float* out_flux, int32_t n_queries, const float* queries,
                              float* out_pdf, int32_t* n_spatial) {
    if (!lo || !hi || n_iters < 0 || (n_iters > 0 && (!n_splats || !splats)) || !n_spatial ||
        (n_queries > 0 && (!queries || !out_pdf))) {
        g_error = "bad argument";
        return PT_ERR_INVALID;
    }
    return guarded([&] {
        SDTreeHost t(lo, hi);
        size_t off = 0;
        for (int it = 0; it < n_iters; it++) {
            for (int k = 0; k < n_splats[it]; k++, off++) {
                const float* sp = splats + 7 * off;
                t.splat(sp[0], sp + 1, sp + 4);
            }
            t.update();
        }
        for (int q = 0; q < n_queries; q++) out_pdf[q] = t.pdf(queries + 6 * q, queries + 6 * q + 3);
        std::vector<DLeafRegion> leaves;
        std::vector<int> lc, cnt;
        std::vector<float> flux;
        t.dump(&leaves, &lc, &cnt, &flux);
        *n_spatial = (int32_t)lc.size();
        for (size_t i = 0; i < leaves.size() && (int32_t)i < max_leaves; i++) {
            out_leaves[4 * i] = leaves[i].bx;
            out_leaves[4 * i + 1] = leaves[i].by;
            out_leaves[4 * i + 2] = leaves[i].sx;
            out_leaves[4 * i + 3] = leaves[i].sy;
        }
        for (size_t i = 0; i < lc.size(); i++) {
            if (out_leaf_counts) out_leaf_counts[i] = lc[i];
            if (out_counts) out_counts[i] = cnt[i];
            if (out_flux) out_flux[i] = flux[i];
        }
    });
}

pt_status pt_debug_image_load(const char* path, int32_t rgb, int32_t srgb, int32_t* w, int32_t* h, float* out,
                              int64_t cap) {
    if (!path || !w || !h) { g_error = "null argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        DecodedImage im;
        try {
            im = decode_image_file(path);
        } catch (std::runtime_error& e) {
            throw Fail(PT_ERR_IO, e.what());
        }
        *w = im.w;
        *h = im.h;
        if (!out) return;
        std::vector<float> px;
        texture_pixels(im, rgb != 0, srgb != 0, px);
        if ((int64_t)px.size() > cap) throw Fail(PT_ERR_LIMIT, "output buffer too small");
        std::memcpy(out, px.data(), sizeof(float) * px.size());
    });
}

pt_status pt_debug_ref_topology_device(const float* tri_v, int32_t n, int32_t* leaf_order, int32_t* prim_parent,
                                       float* node_boxes, int32_t max_nodes, int32_t* n_nodes, int32_t* levels) {
    if (n < 0 || (n > 0 && (!tri_v || !leaf_order || !prim_parent)) || !n_nodes) {
        g_error = "bad argument";
        return PT_ERR_INVALID;
    }
    return guarded([&] {
        DebugCtx c;
        RefBuildStats rs;
        RefTopology t = build_ref_topology_device(tri_v, n, c.st, &rs);
        if (levels) *levels = rs.levels;
        *n_nodes = (int32_t)t.node_box.size();
        if ((int32_t)t.node_box.size() > max_nodes) throw Fail(PT_ERR_LIMIT, "node buffer too small");
        for (int i = 0; i < n; i++) {
            leaf_order[i] = t.leaf_order[i];
            prim_parent[i] = t.prim_parent[i];
        }
        for (size_t i = 0; i < t.node_box.size(); i++) {
            std::memcpy(node_boxes + 6 * i, t.node_box[i].lo, 12);
            std::memcpy(node_boxes + 6 * i + 3, t.node_box[i].hi, 12);
        }
    });
}

pt_status pt_debug_wide_bvh(const float* tri_v, int32_t n, int32_t max_leaf, int32_t on_device, int32_t host_threads,
                            uint32_t* nodes, int32_t max_nodes, int32_t* n_nodes, int32_t* tri_order,
                            int32_t* max_depth, float* inflate) {
    if (n < 0 || (n > 0 && (!tri_v || !tri_order)) || !n_nodes || max_leaf < 1 || max_leaf > 16) {
        g_error = "bad argument";
        return PT_ERR_INVALID;
    }
    return guarded([&] {
        WideBVH w;
        if (on_device) {
            DebugCtx c;
            w = build_wide_bvh_device(tri_v, n, max_leaf, c.st);
        } else {
            w = build_wide_bvh(tri_v, n, max_leaf, host_threads);
        }
        *n_nodes = (int32_t)w.nodes.size();
        if (max_depth) *max_depth = w.max_depth;
        if (inflate) *inflate = w.inflate;
        if ((int32_t)w.nodes.size() > max_nodes || (!nodes && !w.nodes.empty()))
            throw Fail(PT_ERR_LIMIT, "node buffer too small");
        if (!w.nodes.empty()) std::memcpy(nodes, w.nodes.data(), sizeof(WideNode) * w.nodes.size());
        if (n > 0) std::memcpy(tri_order, w.tri_order.data(), sizeof(int32_t) * (size_t)n);
    });
}

pt_status pt_debug_ref_topology(const float* tri_v, int32_t n, int32_t* leaf_order, int32_t* prim_parent,
                                float* node_boxes, int32_t max_nodes, int32_t* n_nodes) {
    if (n < 0 || (n > 0 && (!tri_v || !leaf_order || !prim_parent)) || !n_nodes) {
        g_error = "bad argument";
        return PT_ERR_INVALID;
    }
    return guarded([&] {
        RefTopology t = build_ref_topology(tri_v, n);
        *n_nodes = (int32_t)t.node_box.size();
        if ((int32_t)t.node_box.size() > max_nodes) throw Fail(PT_ERR_LIMIT, "node buffer too small");
        for (int i = 0; i < n; i++) {
            leaf_order[i] = t.leaf_order[i];
            prim_parent[i] = t.prim_parent[i];
        }
        for (size_t i = 0; i < t.node_box.size(); i++) {
            std::memcpy(node_boxes + 6 * i, t.node_box[i].lo, 12);
            std::memcpy(node_boxes + 6 * i + 3, t.node_box[i].hi, 12);
        }
    });
}

}  // extern "C"
