// Internal declarations shared by the C ABI's translation units (host.cpp,
// batch.cpp): error plumbing, device allocation helpers and the scene object.
#pragma once
#include <algorithm>
#include <mutex>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cpppt_gb300.h"
#include "bvh.h"
#include "dev_types.h"
#include "guide.h"
#include "kernels.h"
#include "nn.h"
#include "sdtree.h"
#include <random>

namespace cpppt_gb300 {
namespace hostimpl {
extern thread_local std::string g_error;

// Serialises the scene/batch lifetime bookkeeping (pt_scene::batch_refs and
// destroy_pending) across threads.
inline std::mutex& lifetime_mutex() {
    static std::mutex m;
    return m;
}

struct Fail : std::runtime_error {
    pt_status code;
    Fail(pt_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// A render whose film could not hold a contribution (stat_film_overflow) has
// a wrong image: fail it (the counter stays in the render's statistics).
inline void check_film(double overflow) {
    if (overflow > 0)
        throw Fail(PT_ERR_LIMIT, "film overflow: " + std::to_string((long long)overflow) +
                                     " contributions did not fit the film's 32.32 fixed-point range "
                                     "(a pixel's sum must stay below 2^31)");
}

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Fail(e == cudaErrorMemoryAllocation ? PT_ERR_MEMORY : PT_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
    }
}

template <class F>
pt_status guarded(F&& f) {
    try {
        f();
        g_error.clear();
        return PT_OK;
    } catch (const Fail& e) {
        g_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_error = "host allocation failed";
        return PT_ERR_MEMORY;
    } catch (const std::exception& e) {
        g_error = e.what();
        return PT_ERR_INVALID;
    }
}

template <class T>
T* dalloc(std::vector<void*>& owned, size_t count) {
    void* p = nullptr;
    if (count == 0) count = 1;
    ck(cudaMalloc(&p, sizeof(T) * count), "cudaMalloc");
    owned.push_back(p);
    return static_cast<T*>(p);
}

template <class T>
T* dupload(std::vector<void*>& owned, const std::vector<T>& v, cudaStream_t st) {
    T* p = dalloc<T>(owned, v.size());
    if (!v.empty()) ck(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st), "upload");
    return p;
}

inline float fnorm3(float* v) {
    float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    float inv = 1.0f / l;
    v[0] *= inv; v[1] *= inv; v[2] *= inv;
    return l;
}
inline void fcross(const float* a, const float* b, float* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

}  // namespace hostimpl
}  // namespace cpppt_gb300

using namespace cpppt_gb300;  // internal header of the ABI's own translation units

// Image textures of a file scene (the loader's image(...) textures): pixels
// of every texture back to back, {first float, width, height, channels} per
// texture, per-vertex uv, and each material's texture slots (DevMaterial::tex).
struct SceneTextures {
    std::vector<float> px;
    std::vector<int4> info;
    std::vector<float> uv;         // 2 per vertex (empty: all zero)
    std::vector<uint32_t> mat_tex;  // per material (empty: no textures)
    std::vector<float> emit_intensity;  // per material: intensity of a textured emitter
};

struct pt_scene {
    // counts of the device arrays (a multi-scene batch copies them)
    int n_verts = 0, n_mats = 0, n_rbox = 0;
    int batch_refs = 0;           // batches made from this scene (they use its learned guide);
                                  // read and changed under lifetime_mutex() only
    bool destroy_pending = false;  // pt_scene_destroy came while batches still held the scene
    std::vector<int4> h_tex_info;  // host copy of dev.tex_info (batch arena merge)
    std::vector<DevMaterial> h_mats;  // host copy of dev.mats (batch arena merge)
    size_t n_tex_px = 0;           // floats in dev.tex_px
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> owned;  // scene data
    DevScene dev{};
    int n_tris = 0, width = 0, height = 0;
    double build_ref_ms = 0, build_wide_ms = 0;
    float bounds_lo[3] = {0, 0, 0}, bounds_hi[3] = {0, 0, 0};  // union of the triangles' boxes
    int wide_depth = 0;

    // ray-batch scratch
    int* d_counter = nullptr;
    uint32_t* d_status = nullptr;
    void* d_io = nullptr;
    size_t d_io_bytes = 0;

    // wavefront state
    PathBuffers pb{};
    std::vector<void*> pb_owned;
    unsigned long long* film = nullptr;  // 32.32 fixed point
    float* d_out = nullptr;
    int film_n = 0;
    WaveCounters* d_ctr = nullptr;
    WaveCounters* h_ctr = nullptr;  // pinned
    cudaGraphExec_t graph = nullptr;
    DevBatchJob* d_job = nullptr;  // one-entry job table of the wavefront kernels
    DevBatchJob* h_job = nullptr;  // pinned staging copy
    DevNNJob* d_nnjob = nullptr;   // one-entry learned-guide job table
    DevNNJob* h_nnjob = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    pt_render_stats stats{};

    // learned guide
    bool nn_ready = false;
    std::vector<void*> nn_owned;
    NNWeights nnw{};
    NNTrainBuf nn_tb{};
    float* nn_grad = nullptr;
    float* nn_scalars = nullptr;  // [0] loss, [1] sum of T, [2] status bits
    float* h_scal = nullptr;      // pinned copy of nn_scalars
    NNTrainTask* d_tasks = nullptr;  // training task table (one per step of a round)
    NNTrainTask* h_tasks = nullptr;  // pinned
    int nn_steps = 0;
    double nn_last_loss = 0, nn_records = 0;
    float4* nn_rec = nullptr;  // training records being collected (one of nn_rec_buf)
    float4* nn_rec_buf[2] = {nullptr, nullptr};  // double buffer: one collects while the other trains
    int nn_rec_cur = 0;
    cudaStream_t nn_tst = nullptr;                   // training stream (overlaps the wavefront)
    cudaEvent_t nn_read_done[2] = {nullptr, nullptr};  // last training that read nn_rec_buf[k] completed
    cudaEvent_t nn_ev_records = nullptr;             // a round's records are complete (render stream)
    int nn_rec_count = 0;
    float nn_keep = 1.0f;  // probability that a finished path leaves training records (adapted per round)
    int* h_rec_left = nullptr;  // pinned staging word for the kept-record count
    NNPathData nnpd{};          // per-path buffers of the slot-based wavefront (grown on demand)
    float4* nn_params = nullptr;
    int nnpd_cap = 0, nnpd_depth = 0;
    std::vector<void*> nnpd_owned;
    pt_nn_config nn_cfg{3e-3f, 0.3f, 0.9f, 1 << 16, PT_NN_CHI2, 16, PT_NN_ENC_FREQ, 1};

    ~pt_scene() {
        for (void* p : nn_owned) cudaFree(p);
        for (void* p : nnpd_owned) cudaFree(p);
        if (graph) cudaGraphExecDestroy(graph);
        for (void* p : owned) cudaFree(p);
        for (void* p : pb_owned) cudaFree(p);
        if (film) cudaFree(film);
        if (d_out) cudaFree(d_out);
        if (d_io) cudaFree(d_io);
        if (h_ctr) cudaFreeHost(h_ctr);
        if (h_job) cudaFreeHost(h_job);
        if (h_nnjob) cudaFreeHost(h_nnjob);
        if (h_rec_left) cudaFreeHost(h_rec_left);
        if (h_scal) cudaFreeHost(h_scal);
        if (h_tasks) cudaFreeHost(h_tasks);
        if (nn_tst) { cudaStreamSynchronize(nn_tst); cudaStreamDestroy(nn_tst); }
        for (cudaEvent_t e : nn_read_done) if (e) cudaEventDestroy(e);
        if (nn_ev_records) cudaEventDestroy(nn_ev_records);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace cpppt_gb300 {
namespace hostimpl {
// Learned-guide state of a scene (host.cpp), for the multi-scene batch.
void nn_ensure_scene(pt_scene* s);               // network, Adam state, record and training buffers
NNNorm nn_scene_norm(const pt_scene* s);         // position normalisation and BSDF-fraction range
int nn_record_cap(const pt_scene* s);            // records collected per round (steps_per_round batches, <= 2^22)
// Training of the learned guides overlaps the wavefront.  After a round,
// nn_train_enqueue queues on the training stream `tst` (after the records
// the render stream `st` has produced so far) as many Adam steps per scene
// as it holds full batches (held[k] counted, at most caps[k] written), the
// steps of all scenes fused per step level; it moves each trained scene's
// records beyond its last full batch to the front of its other record
// buffer (on `st`, after the training that last read that buffer),
// switches the scene to that buffer and sets *d_count[k] and left[k] to the
// records kept (-1: no full batch, nothing changed).  It returns at once;
// nn_train_finish waits for the queued steps and takes their status and
// loss (done at the start of the next enqueue and at the end of a render).
struct NNTrainPending {
    std::vector<pt_scene*> sc;
    std::vector<int> steps;
    cudaStream_t tst = nullptr;
};
void nn_train_enqueue(pt_scene* const* scenes, const int* held, const int* caps, int* const* d_count, int n,
                      NNTrainTask* d_tasks, NNTrainTask* h_tasks, int num_sms, cudaStream_t st, cudaStream_t tst,
                      cudaEvent_t ev_records, double* launches, int* left, NNTrainPending& pending);
void nn_train_finish(NNTrainPending& pending);
}  // namespace hostimpl
}  // namespace cpppt_gb300
