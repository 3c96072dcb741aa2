// Multi-scene batches (pt_batch_*): many scenes of uneven size, resolution
// and spp rendered by one wavefront.
//
// pt_batch_create merges the scenes' device arrays into one arena with the
// cross-references rebased (batch.cu), so the traversal kernels run on the
// arena unchanged; each path carries its job, whose table entry gives the
// scene root, camera, light list, film range and render parameters.  Jobs are
// laid out back to back in one work range: while the last paths of a job
// drain, the first paths of the next one fill the freed wavefront slots, so
// the GPU stays full across scenes and the whole batch is one chain of
// graph-captured iterations.  The RNG is keyed by (job seed, sample, pixel,
// bounce) and the film is fixed point, so each job's image is bit-identical
// to pt_render of the same scene with the same parameters.
#include "batch.h"
#include "host_internal.h"

using namespace cpppt_gb300::hostimpl;

struct pt_batch {
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> owned;  // arena
    DevScene arena{};
    struct Member {
        pt_scene* scene;  // its learned guide serves guided batch renders
        uint32_t root;
        int light_off, n_lights, width, height;
        DevCamera cam;
    };
    std::vector<Member> members;

    pt_batch_tuning tuning{1 << 21, 16, 1, 1};
    PathBuffers pb{};
    std::vector<void*> pb_owned;
    unsigned long long* film = nullptr;
    size_t film_cap = 0;  // u64 elements
    float* d_out = nullptr;
    size_t out_cap = 0;
    DevBatchJob* d_jobs = nullptr;
    DevBatchJob* h_jobs = nullptr;  // pinned
    int jobs_cap = 0;
    WaveCounters* d_ctr = nullptr;
    WaveCounters* h_ctr = nullptr;  // pinned
    cudaGraphExec_t graph = nullptr;
    struct GraphKey {
        const void* film;
        int n_jobs, capacity, iters;
        bool operator==(const GraphKey& o) const {
            return film == o.film && n_jobs == o.n_jobs && capacity == o.capacity && iters == o.iters;
        }
    } graph_key{nullptr, 0, 0, 0};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    pt_render_stats stats{};

    // slot wavefront (learned guide, PT_FLAG_UNBIASED_MIS): per-path vertex
    // records and slots, guide parameters, per-job guide table, per-scene
    // record counters
    NNPathData pd{};
    std::vector<void*> pd_owned;
    int pd_cap = 0, pd_depth = 0;
    float4* nn_params = nullptr;
    DevNNJob* d_nnjobs = nullptr;
    DevNNJob* h_nnjobs = nullptr;  // pinned
    int nnjobs_cap = 0;
    int* d_nrec = nullptr;  // one per member scene (in `owned`)
    int* h_nrec = nullptr;  // pinned
    NNTrainTask* d_tasks = nullptr;  // fused training steps: kNNMaxStepsPerRound x kNNMaxPasses per member scene (in `owned`)
    NNTrainTask* h_tasks = nullptr;  // pinned
    cudaStream_t nn_tst = nullptr;       // training stream (overlaps the wavefront)
    cudaEvent_t nn_ev_records = nullptr;  // a round's records are complete

    ~pt_batch() {
        if (stream) cudaStreamSynchronize(stream);
        if (graph) cudaGraphExecDestroy(graph);
        for (void* p : owned) cudaFree(p);
        for (void* p : pb_owned) cudaFree(p);
        if (film) cudaFree(film);
        if (d_out) cudaFree(d_out);
        if (d_jobs) cudaFree(d_jobs);
        if (h_jobs) cudaFreeHost(h_jobs);
        if (h_ctr) cudaFreeHost(h_ctr);  // d_ctr is in pb_owned
        for (void* p : pd_owned) cudaFree(p);
        if (d_nnjobs) cudaFree(d_nnjobs);
        if (h_nnjobs) cudaFreeHost(h_nnjobs);
        if (h_nrec) cudaFreeHost(h_nrec);
        if (h_tasks) cudaFreeHost(h_tasks);
        if (nn_tst) { cudaStreamSynchronize(nn_tst); cudaStreamDestroy(nn_tst); }
        if (nn_ev_records) cudaEventDestroy(nn_ev_records);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

constexpr int kMaxBatchCapacity = 1 << 24;
constexpr int kMaxSlotCapacity = 1 << 22;  // learned-guide batches: vertex records per path and bounce
constexpr unsigned long long kMaxBatchPixels = 1ull << 30;  // film pixel index travels as a 32-bit word

template <class T>
void d2d(T* dst, const T* src, size_t n, cudaStream_t st) {
    if (n) ck(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDeviceToDevice, st), "arena copy");
}

void create_batch(pt_scene* const* scenes, int n, pt_batch* b) {
    if (!scenes || n < 1) throw std::invalid_argument("a batch needs at least one scene");
    for (int i = 0; i < n; i++)
        if (!scenes[i]) throw std::invalid_argument("null scene in batch");
    b->device = scenes[0]->device;
    b->num_sms = scenes[0]->num_sms;
    int cur = 0;
    ck(cudaGetDevice(&cur), "cudaGetDevice");
    for (int i = 0; i < n; i++)
        if (scenes[i]->device != b->device) throw std::invalid_argument("batch scenes live on different devices");
    if (cur != b->device) throw std::invalid_argument("the current device is not the scenes' device");
    ck(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    // arena sizes and offsets
    unsigned long long nn = 0, nt = 0, nr = 0, nv = 0, nm = 0, nl = 0, ntex = 0, npx = 0;
    for (int i = 0; i < n; i++) {
        const pt_scene* s = scenes[i];
        nn += s->dev.n_nodes;
        nt += s->n_tris;
        nr += s->n_rbox;
        nv += s->n_verts;
        nm += s->n_mats;
        nl += s->dev.n_lights;
        ntex += s->h_tex_info.size();
        npx += s->n_tex_px;
    }
    if (ntex >= kNoTex) throw Fail(PT_ERR_LIMIT, "a batch holds at most 254 image textures");
    if (nt >= (1ull << 27)) throw Fail(PT_ERR_LIMIT, "batch exceeds 2^27 - 1 triangles (leaf reference range)");
    if (nn >= (1ull << 31) || nr >= (1ull << 31) || nv >= (1ull << 31) || nm >= (1ull << 31))
        throw Fail(PT_ERR_LIMIT, "batch arena exceeds 32-bit indices");
    DevScene& A = b->arena;
    uint4* nodes = dalloc<uint4>(b->owned, 4 * nn);
    float4* tris = dalloc<float4>(b->owned, 3 * nt);
    float4* rbox = dalloc<float4>(b->owned, 2 * nr);
    int4* vidx = dalloc<int4>(b->owned, nt);
    float4* vpos = dalloc<float4>(b->owned, nv);
    float4* vnrm = dalloc<float4>(b->owned, nv);
    float4* vbt = dalloc<float4>(b->owned, nv);
    DevMaterial* mats = dalloc<DevMaterial>(b->owned, nm);
    float2* vuv = dalloc<float2>(b->owned, std::max<unsigned long long>(1, nv));
    float* tpx = dalloc<float>(b->owned, std::max<unsigned long long>(1, npx));
    std::vector<int4> tinfo;
    std::vector<DevMaterial> hmats;
    tinfo.reserve(ntex + 1);
    hmats.reserve(nm);
    int32_t* lprim = dalloc<int32_t>(b->owned, nl);
    float* larea = dalloc<float>(b->owned, nl);
    cudaStream_t st = b->stream;
    int on = 0, ot = 0, orb = 0, ov = 0, om = 0, ol = 0;
    for (int i = 0; i < n; i++) {
        const pt_scene* s = scenes[i];
        const DevScene& S = s->dev;
        // the source scene's uploads ran on its own stream
        ck(cudaStreamSynchronize(s->stream), "scene stream");
        launch_rebase_nodes(nodes + 4 * (size_t)on, S.nodes, S.n_nodes, (uint32_t)on, (uint32_t)ot, st);
        launch_rebase_tris(tris + 3 * (size_t)ot, S.tris, s->n_tris, orb, ot, st);
        d2d(rbox + 2 * (size_t)orb, S.ref_box, 2 * (size_t)s->n_rbox, st);
        launch_rebase_vidx(vidx + ot, S.tri_vidx, s->n_tris, ov, om, st);
        d2d(vpos + ov, S.v_pos, s->n_verts, st);
        d2d(vnrm + ov, S.v_nrm, s->n_verts, st);
        d2d(vbt + ov, S.v_btan, s->n_verts, st);
        d2d(vuv + ov, S.v_uv, s->n_verts, st);
        // textures: pixels appended, offsets and material slots rebased
        const int tex_base = (int)tinfo.size();
        size_t px_off = 0;
        for (const int4& t : tinfo) px_off = std::max(px_off, (size_t)t.x + (size_t)t.y * t.z * t.w);
        if (s->n_tex_px) d2d(tpx + px_off, S.tex_px, s->n_tex_px, st);
        for (int4 t : s->h_tex_info) {
            t.x += (int)px_off;
            tinfo.push_back(t);
        }
        for (DevMaterial m : s->h_mats) {
            if (m.tex != kNoTextures)
                for (int k = 0; k < 4; k++) {
                    const uint32_t id = (m.tex >> (8 * k)) & 0xffu;
                    if (id != kNoTex) m.tex = (m.tex & ~(0xffu << (8 * k))) | ((id + (uint32_t)tex_base) << (8 * k));
                }
            hmats.push_back(m);
        }
        launch_offset_i32(lprim + ol, S.light_prim, S.n_lights, ot, st);
        d2d(larea + ol, S.light_area, S.n_lights, st);
        pt_batch::Member m;
        m.scene = scenes[i];
        m.root = s->n_tris > 0 ? (uint32_t)on : 0xffffffffu;
        m.light_off = ol;
        m.n_lights = S.n_lights;
        m.width = s->width;
        m.height = s->height;
        m.cam = S.cam;
        b->members.push_back(m);
        on += S.n_nodes;
        ot += s->n_tris;
        orb += s->n_rbox;
        ov += s->n_verts;
        om += s->n_mats;
        ol += S.n_lights;
    }
    ck(cudaGetLastError(), "arena merge");
    A.nodes = nodes;
    A.n_nodes = on;
    A.n_tris = ot;
    A.tris = tris;
    A.ref_box = rbox;
    A.tri_vidx = vidx;
    A.v_pos = vpos;
    A.v_nrm = vnrm;
    A.v_btan = vbt;
    A.mats = mats;
    A.light_prim = lprim;
    A.light_area = larea;
    A.n_lights = ol;
    if (!hmats.empty())
        ck(cudaMemcpyAsync(mats, hmats.data(), sizeof(DevMaterial) * hmats.size(), cudaMemcpyHostToDevice, st),
           "arena materials");
    if (tinfo.empty()) tinfo.push_back(make_int4(0, 1, 1, 1));
    int4* dinfo = dalloc<int4>(b->owned, tinfo.size());
    ck(cudaMemcpyAsync(dinfo, tinfo.data(), sizeof(int4) * tinfo.size(), cudaMemcpyHostToDevice, st), "arena textures");
    A.v_uv = vuv;
    A.tex_px = tpx;
    A.tex_info = dinfo;
    A.n_tex = (int)ntex;
    A.cam = b->members[0].cam;  // unused by the batch kernels
    b->d_ctr = dalloc<WaveCounters>(b->pb_owned, 1);
    ck(cudaMallocHost(&b->h_ctr, sizeof(WaveCounters)), "cudaMallocHost");
    b->d_nrec = dalloc<int>(b->owned, n);
    ck(cudaMallocHost(&b->h_nrec, sizeof(int) * n), "cudaMallocHost");
    b->d_tasks = dalloc<NNTrainTask>(b->owned, (size_t)n * kNNMaxStepsPerRound * kNNMaxPasses);
    ck(cudaMallocHost(&b->h_tasks, sizeof(NNTrainTask) * n * kNNMaxStepsPerRound * kNNMaxPasses), "cudaMallocHost");
    ck(cudaStreamCreateWithFlags(&b->nn_tst, cudaStreamNonBlocking), "cudaStreamCreate");
    ck(cudaEventCreateWithFlags(&b->nn_ev_records, cudaEventDisableTiming), "cudaEventCreate");
    ck(cudaEventCreate(&b->ev0), "cudaEventCreate");
    ck(cudaEventCreate(&b->ev1), "cudaEventCreate");
    ck(cudaStreamSynchronize(st), "arena merge");
}

void check_tuning(const pt_batch_tuning& t) {
    if (t.capacity < 1024 || t.capacity > kMaxBatchCapacity || t.capacity % 1024)
        throw std::invalid_argument("capacity must be a multiple of 1024 in [1024, 16777216]");
    if (t.iters_per_graph < 2 || t.iters_per_graph > 256 || t.iters_per_graph % 2)
        throw std::invalid_argument("iters_per_graph must be even, in [2, 256]");
    if (t.tile_w < 1 || t.tile_h < 1 || t.tile_w * t.tile_h > 1024)
        throw std::invalid_argument("tile sides must be >= 1 with at most 1024 pixels per tile");
}

void ensure_buffers(pt_batch* b, int capacity, size_t film_n, int n_jobs) {
    if (b->pb.capacity != capacity) {
        // keep the counters block (first entry), drop the path buffers
        void* ctr = b->d_ctr;
        for (void* p : b->pb_owned)
            if (p != ctr) cudaFree(p);
        b->pb_owned.assign(1, ctr);
        PathBuffers& B = b->pb;
        for (int k = 0; k < 2; k++) {
            B.o[k] = dalloc<float4>(b->pb_owned, capacity);
            B.d[k] = dalloc<float4>(b->pb_owned, capacity);
            B.thr[k] = dalloc<float4>(b->pb_owned, capacity);
            B.info[k] = dalloc<int4>(b->pb_owned, capacity);
        }
        B.hit = dalloc<float4>(b->pb_owned, capacity);
        B.sh_o = dalloc<float4>(b->pb_owned, capacity);
        B.sh_d = dalloc<float4>(b->pb_owned, capacity);
        B.sh_c = dalloc<float4>(b->pb_owned, capacity);
        B.capacity = capacity;
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    }
    if (b->film_cap < film_n) {
        if (b->film) cudaFree(b->film);
        if (b->d_out) cudaFree(b->d_out);
        b->film = nullptr;
        b->d_out = nullptr;
        ck(cudaMalloc(&b->film, sizeof(unsigned long long) * film_n), "cudaMalloc film");
        ck(cudaMalloc(&b->d_out, sizeof(float) * film_n), "cudaMalloc film");
        b->film_cap = film_n;
        b->out_cap = film_n;
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    }
    if (b->jobs_cap < n_jobs) {
        if (b->d_jobs) cudaFree(b->d_jobs);
        if (b->h_jobs) cudaFreeHost(b->h_jobs);
        b->d_jobs = nullptr;
        b->h_jobs = nullptr;
        ck(cudaMalloc(&b->d_jobs, sizeof(DevBatchJob) * n_jobs), "cudaMalloc jobs");
        ck(cudaMallocHost(&b->h_jobs, sizeof(DevBatchJob) * n_jobs), "cudaMallocHost jobs");
        b->jobs_cap = n_jobs;
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    }
}

// Builds the job table; returns total work and total film pixels.
void build_jobs(pt_batch* b, const pt_batch_job* jobs, int n_jobs, const pt_batch_tuning& t, int integrator,
                std::vector<DevBatchJob>& out, unsigned long long* work, unsigned long long* pixels) {
    if (!jobs || n_jobs < 1) throw std::invalid_argument("a batch render needs at least one job");
    out.resize(n_jobs);
    unsigned long long w = 0, px = 0;
    for (int i = 0; i < n_jobs; i++) {
        const pt_batch_job& j = jobs[i];
        if (j.scene < 0 || j.scene >= (int)b->members.size()) throw std::invalid_argument("job scene out of range");
        if (j.spp < 1) throw std::invalid_argument("spp must be >= 1");
        if (j.max_depth < 1 || j.max_depth > 0xffff) throw std::invalid_argument("max_depth must be in [1, 65535]");
        const pt_batch::Member& m = b->members[j.scene];
        DevBatchJob& d = out[i];
        d = DevBatchJob{};
        d.cam = m.cam;
        d.work_begin = w;
        d.film_off = px;
        d.root = m.root;
        d.light_off = m.light_off;
        d.n_lights = m.n_lights;
        d.spp = j.spp;
        const int ax = (int)std::lround(std::sqrt((double)j.spp));
        d.spp_axis = (ax * ax == j.spp) ? ax : 0;  // as pt_render
        d.max_depth = j.max_depth;
        d.rr_start = j.rr_start;
        d.seed = j.seed;
        d.integrator = integrator;
        const bool tiles = m.width % t.tile_w == 0 && m.height % t.tile_h == 0;
        d.tile_w = tiles ? t.tile_w : 1;
        d.tile_h = tiles ? t.tile_h : 1;
        const unsigned long long npx = (unsigned long long)m.width * m.height;
        w += npx * (unsigned long long)j.spp;
        px += npx;
    }
    if (px > kMaxBatchPixels) throw Fail(PT_ERR_LIMIT, "batch film exceeds 2^30 pixels");
    *work = w;
    *pixels = px;
}

// Renders the jobs; d_dst[i] (device, 3 floats per pixel) receive the images,
// or the batch's own output buffer when d_dst is null.
void render_batch(pt_batch* b, const pt_batch_job* jobs, int n_jobs, float* const* d_dst, const pt_batch_tuning& t,
                  int integrator = kIntegratorMIS) {
    check_tuning(t);
    std::vector<DevBatchJob> table;
    unsigned long long total = 0, pixels = 0;
    build_jobs(b, jobs, n_jobs, t, integrator, table, &total, &pixels);
    const int capacity = (int)std::min<unsigned long long>(t.capacity, (total + 1023) / 1024 * 1024);
    ensure_buffers(b, capacity, 3 * pixels, n_jobs);
    cudaStream_t st = b->stream;
    std::memcpy(b->h_jobs, table.data(), sizeof(DevBatchJob) * n_jobs);
    ck(cudaMemcpyAsync(b->d_jobs, b->h_jobs, sizeof(DevBatchJob) * n_jobs, cudaMemcpyHostToDevice, st), "jobs");
    const pt_batch::GraphKey key{b->film, n_jobs, capacity, t.iters_per_graph};
    if (!b->graph || !(b->graph_key == key)) {
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
        ck(build_render_graph(b->arena, b->pb, b->d_ctr, b->film, b->d_jobs, n_jobs, t.iters_per_graph, b->num_sms, st,
                              &b->graph),
           "render graph");
        b->graph_key = key;
    }
    ck(cudaEventRecord(b->ev0, st), "event");
    ck(cudaMemsetAsync(b->film, 0, sizeof(unsigned long long) * 3 * pixels, st), "memset film");
    int max_depth = 1;
    for (const DevBatchJob& j : table) max_depth = std::max(max_depth, j.max_depth);
    const unsigned long long max_rounds =
        64 + (total / (unsigned long long)capacity + 2 + (unsigned long long)n_jobs) *
                 (unsigned long long)(max_depth + 2) * 4 / (unsigned long long)t.iters_per_graph;
    WaveCounters init{};
    init.work_total = total;
    init.max_rounds = (uint32_t)std::min<unsigned long long>(max_rounds, 0xffffffffull);
    {
        double per_pixel = 1.0;
        for (const DevBatchJob& j : table) per_pixel = std::max(per_pixel, (double)j.spp * (2.0 * j.max_depth + 2.0));
        init.film_safe = film_safe_bound(per_pixel);
    }
    *b->h_ctr = init;
    ck(cudaMemcpyAsync(b->d_ctr, b->h_ctr, sizeof(WaveCounters), cudaMemcpyHostToDevice, st), "init counters");
    launch_generate(b->arena, b->pb, 1, b->d_ctr, b->d_jobs, n_jobs, st);  // fills buffer 0
    // the whole loop on the device: one graph launch, one read of the counters
    ck(cudaGraphLaunch(b->graph, st), "graph launch");
    ck(cudaMemcpyAsync(b->h_ctr, b->d_ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st), "read counters");
    ck(cudaStreamSynchronize(st), "batch render");
    {
        const uint32_t status = b->h_ctr->status;
        if (status & kStatusStackOverflow) throw Fail(PT_ERR_LIMIT, "traversal stack overflow");
        if (status & kStatusIterLimit) throw Fail(PT_ERR_LIMIT, "traversal step limit reached");
        if (status & kStatusQueueOverflow) throw Fail(PT_ERR_LIMIT, "wavefront queue overflow");
        if (status & kStatusRoundLimit) throw Fail(PT_ERR_LIMIT, "batch render did not converge within the iteration bound");
    }
    const unsigned long long rounds = b->h_ctr->rounds;
    double launches = 2 + (double)rounds * (kKernelsPerIteration * t.iters_per_graph + 1);
    for (int i = 0; i < n_jobs; i++) {
        const pt_batch::Member& m = b->members[jobs[i].scene];
        const size_t off = 3 * (size_t)table[i].film_off;
        float* dst = (d_dst && d_dst[i]) ? d_dst[i] : b->d_out + off;
        launch_film_resolve(b->film + off, dst, 3 * m.width * m.height, 1.0 / (double)jobs[i].spp, st);
        launches += 1;
    }
    ck(cudaEventRecord(b->ev1, st), "event");
    ck(cudaStreamSynchronize(st), "batch render");
    ck(cudaGetLastError(), "batch kernels");
    float ms = 0;
    ck(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "elapsed");
    pt_render_stats& R = b->stats;
    R = pt_render_stats{};
    R.paths = (double)b->h_ctr->stat_paths;
    R.closest_rays = (double)b->h_ctr->stat_closest;
    R.shadow_rays = (double)b->h_ctr->stat_shadow;
    R.iterations = (double)b->h_ctr->stat_iters;
    R.render_ms = ms;
    R.kernel_launches = launches;
    R.nonfinite = (double)b->h_ctr->stat_nonfinite;
    R.film_overflow = (double)b->h_ctr->stat_film_overflow;
    R.h2d_bytes = (double)(sizeof(WaveCounters) + sizeof(DevBatchJob) * n_jobs);
    R.d2h_bytes = (double)sizeof(WaveCounters);
    check_film(R.film_overflow);
}

// Per-path buffers of the slot wavefront, grown on demand.
NNPathData slot_buffers(pt_batch* b, int capacity, int depth, bool params) {
    if (capacity > b->pd_cap || depth > b->pd_depth || (params && !b->nn_params)) {
        for (void* p : b->pd_owned) cudaFree(p);
        b->pd_owned.clear();
        b->pd = NNPathData{};
        b->nn_params = nullptr;
        b->pd_cap = std::max(capacity, b->pd_cap);
        b->pd_depth = std::max(depth, b->pd_depth);
        const int cap = b->pd_cap;
        b->pd.vert = dalloc<float4>(b->pd_owned, (size_t)cap * std::max(1, b->pd_depth) * kNNVertFloat4);
        b->pd.acc = dalloc<float4>(b->pd_owned, cap);
        b->pd.slot_stack = dalloc<int>(b->pd_owned, cap);
        b->pd.slot_job = dalloc<int>(b->pd_owned, cap);
        b->pd.fin = dalloc<int4>(b->pd_owned, cap);
        if (params) b->nn_params = dalloc<float4>(b->pd_owned, (size_t)cap * kNNMixF4);
    }
    return b->pd;
}

// The jobs on the slot wavefront (nn.cu): PT + NEE + MIS with each job's
// scene's learned guide (guided; trained online from the batch's paths
// unless PT_FLAG_NN_FREEZE, each scene's network on its own records), or the
// same estimator with BSDF sampling alone (PT_FLAG_UNBIASED_MIS).  Each
// job's image equals pt_render of its scene with the same parameters and
// mode when the guides are frozen (training order depends on the batch).
void render_batch_slot(pt_batch* b, const pt_batch_job* jobs, int n_jobs, float* const* d_dst,
                       const pt_batch_tuning& t, bool guided, uint32_t flags) {
    check_tuning(t);
    if (n_jobs > kNNMaxJobs) throw Fail(PT_ERR_LIMIT, "the slot wavefront takes at most 32768 jobs");
    const bool train = guided && !(flags & PT_FLAG_NN_FREEZE);
    std::vector<DevBatchJob> table;
    unsigned long long total = 0, pixels = 0;
    build_jobs(b, jobs, n_jobs, t, kIntegratorMIS, table, &total, &pixels);
    int max_depth = 1;
    for (const DevBatchJob& j : table) max_depth = std::max(max_depth, j.max_depth);
    const int capacity = (int)std::min<unsigned long long>(std::min(t.capacity, kMaxSlotCapacity), (total + 1023) / 1024 * 1024);
    ensure_buffers(b, capacity, 3 * pixels, n_jobs);
    cudaStream_t st = b->stream;
    const int n_members = (int)b->members.size();
    std::vector<char> used(n_members, 0);
    for (int i = 0; i < n_jobs; i++) used[jobs[i].scene] = 1;
    std::vector<int> cap(n_members, 0);
    int max_cap = 0;
    if (guided)
        for (int m = 0; m < n_members; m++) {
            if (!used[m]) continue;
            pt_scene* s = b->members[m].scene;
            nn_ensure_scene(s);
            cap[m] = train ? nn_record_cap(s) : 0;
            max_cap = std::max(max_cap, cap[m]);
        }
    NNPathData PD = slot_buffers(b, capacity, train ? max_depth : 0, guided);
    PD.rec_cap = max_cap;
    if (b->nnjobs_cap < n_jobs) {
        if (b->d_nnjobs) cudaFree(b->d_nnjobs);
        if (b->h_nnjobs) cudaFreeHost(b->h_nnjobs);
        b->d_nnjobs = nullptr;
        b->h_nnjobs = nullptr;
        ck(cudaMalloc(&b->d_nnjobs, sizeof(DevNNJob) * n_jobs), "cudaMalloc guide jobs");
        ck(cudaMallocHost(&b->h_nnjobs, sizeof(DevNNJob) * n_jobs), "cudaMallocHost guide jobs");
        b->nnjobs_cap = n_jobs;
    }
    bool oneblob = false;  // some guide of the batch uses the one-blob encoding
    for (int i = 0; i < n_jobs; i++) {
        const int m = jobs[i].scene;
        DevNNJob& nj = b->h_nnjobs[i];
        nj = DevNNJob{};
        nj.n_rec = b->d_nrec + m;
        if (!guided) continue;
        pt_scene* s = b->members[m].scene;
        const NNNorm N = nn_scene_norm(s);
        nj.wt = s->nnw.wt;
        for (int k = 0; k < 3; k++) {
            nj.lo[k] = N.lo[k];
            nj.inv_ext[k] = N.inv_ext[k];
        }
        nj.c_lo = N.c_lo;
        nj.c_hi = N.c_hi;
        nj.encoding = N.encoding;
        oneblob = oneblob || N.encoding == PT_NN_ENC_ONEBLOB;
        nj.rec = train ? s->nn_rec : nullptr;
        nj.rec_cap = cap[m];
    }
    for (int m = 0; m < n_members; m++) b->h_nrec[m] = train && used[m] ? b->members[m].scene->nn_rec_count : 0;
    std::memcpy(b->h_jobs, table.data(), sizeof(DevBatchJob) * n_jobs);
    ck(cudaMemcpyAsync(b->d_jobs, b->h_jobs, sizeof(DevBatchJob) * n_jobs, cudaMemcpyHostToDevice, st), "jobs");
    ck(cudaMemcpyAsync(b->d_nnjobs, b->h_nnjobs, sizeof(DevNNJob) * n_jobs, cudaMemcpyHostToDevice, st),
       "guide jobs");
    ck(cudaMemcpyAsync(b->d_nrec, b->h_nrec, sizeof(int) * n_members, cudaMemcpyHostToDevice, st), "records");
    RenderParams P{};
    P.max_depth = max_depth;  // vertex-record stride of a slot
    P.flags = flags;
    ck(cudaEventRecord(b->ev0, st), "event");
    ck(cudaMemsetAsync(b->film, 0, sizeof(unsigned long long) * 3 * pixels, st), "memset film");
    launch_init_slots(PD.slot_stack, capacity, st);
    WaveCounters init{};
    init.work_total = total;
    init.free_top = capacity;
    {
        double per_pixel = 1.0;
        for (int k = 0; k < n_jobs; k++) per_pixel = std::max(per_pixel, (double)jobs[k].spp * (2.0 * jobs[k].max_depth + 2.0));
        init.film_safe = film_safe_bound(per_pixel);
    }
    *b->h_ctr = init;
    ck(cudaMemcpyAsync(b->d_ctr, b->h_ctr, sizeof(WaveCounters), cudaMemcpyHostToDevice, st), "init counters");
    launch_nn_generate(b->arena, b->pb, 1, b->d_ctr, PD, b->d_jobs, n_jobs, st);  // fills buffer 0
    const unsigned long long max_rounds =
        64 + (total / (unsigned long long)capacity + 2 + (unsigned long long)n_jobs) *
                 (unsigned long long)(max_depth + 2) * 4 / (unsigned long long)t.iters_per_graph;
    std::vector<int> left(n_members, -1);  // records kept after a scene's last training round (-1: none)
    NNTrainPending pending;
    ck(cudaStreamSynchronize(b->nn_tst), "train");  // nothing of an earlier call is left queued
    double launches = 5;
    unsigned long long rounds = 0;
    while (true) {
        for (int k = 0; k < t.iters_per_graph; k++) {
            const int cur = k & 1;
            launch_extend(b->arena, b->pb, cur, b->d_ctr, b->num_sms, st);
            if (guided)
                launch_nn_infer(b->arena, b->pb, cur, b->d_ctr, b->d_nnjobs, b->nn_params, b->num_sms, st, oneblob);
            launch_nn_shade(b->arena, b->pb, cur, P, b->d_ctr, b->film, b->nn_params, PD, guided, b->d_jobs, st);
            launch_nn_shadow(b->arena, b->pb, b->d_ctr, b->film, PD, b->d_jobs, b->num_sms, st);
            launch_nn_finish(PD, b->d_ctr, b->d_nnjobs, max_depth, capacity, st);
            launch_nn_generate(b->arena, b->pb, cur, b->d_ctr, PD, b->d_jobs, n_jobs, st);
            launches += guided ? 7 : 6;
        }
        ck(cudaMemcpyAsync(b->h_ctr, b->d_ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st), "read counters");
        if (train)
            ck(cudaMemcpyAsync(b->h_nrec, b->d_nrec, sizeof(int) * n_members, cudaMemcpyDeviceToHost, st),
               "read records");
        ck(cudaStreamSynchronize(st), "batch render");
        const uint32_t status = b->h_ctr->status;
        if (status & kStatusStackOverflow) throw Fail(PT_ERR_LIMIT, "traversal stack overflow");
        if (status & kStatusIterLimit) throw Fail(PT_ERR_LIMIT, "traversal step limit reached");
        if (status & kStatusQueueOverflow) throw Fail(PT_ERR_LIMIT, "wavefront queue overflow");
        if (status & kStatusTensorTimeout) throw Fail(PT_ERR_CUDA, "tensor-core completion wait timed out");
        if (status) throw Fail(PT_ERR_CUDA, "batch render reported an error status");
        if (train) {
            // every scene with a full batch of records trains, all in the same
            // fused steps on the training stream, while the next round fills
            // the scenes' other record buffers
            std::vector<pt_scene*> sc(n_members, nullptr);
            std::vector<int*> d_count(n_members);
            for (int m = 0; m < n_members; m++) {
                if (used[m]) sc[m] = b->members[m].scene;
                d_count[m] = b->d_nrec + m;
            }
            nn_train_enqueue(sc.data(), b->h_nrec, cap.data(), d_count.data(), n_members, b->d_tasks, b->h_tasks,
                             b->num_sms, st, b->nn_tst, b->nn_ev_records, &launches, left.data(), pending);
            bool moved = false;
            for (int m = 0; m < n_members; m++) moved = moved || left[m] >= 0;
            if (moved) {
                for (int i = 0; i < n_jobs; i++) b->h_nnjobs[i].rec = b->members[jobs[i].scene].scene->nn_rec;
                ck(cudaMemcpyAsync(b->d_nnjobs, b->h_nnjobs, sizeof(DevNNJob) * n_jobs, cudaMemcpyHostToDevice, st),
                   "guide jobs");
            }
        }
        rounds++;
        if (b->h_ctr->n_cur == 0 && b->h_ctr->work_next >= b->h_ctr->work_total) break;
        if (rounds > max_rounds) throw Fail(PT_ERR_LIMIT, "batch render did not converge within the iteration bound");
    }
    if (train)
        for (int m = 0; m < n_members; m++)
            if (used[m])
                b->members[m].scene->nn_rec_count = left[m] >= 0 ? left[m] : std::min(b->h_nrec[m], cap[m]);
    nn_train_finish(pending);  // the networks are complete before the render returns
    for (int i = 0; i < n_jobs; i++) {
        const pt_batch::Member& m = b->members[jobs[i].scene];
        const size_t off = 3 * (size_t)table[i].film_off;
        float* dst = (d_dst && d_dst[i]) ? d_dst[i] : b->d_out + off;
        launch_film_resolve(b->film + off, dst, 3 * m.width * m.height, 1.0 / (double)jobs[i].spp, st);
        launches += 1;
    }
    ck(cudaEventRecord(b->ev1, st), "event");
    ck(cudaStreamSynchronize(st), "batch render");
    ck(cudaGetLastError(), "batch kernels");
    float ms = 0;
    ck(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "elapsed");
    pt_render_stats& R = b->stats;
    R = pt_render_stats{};
    R.paths = (double)b->h_ctr->stat_paths;
    R.closest_rays = (double)b->h_ctr->stat_closest;
    R.shadow_rays = (double)b->h_ctr->stat_shadow;
    R.iterations = (double)b->h_ctr->stat_iters;
    R.render_ms = ms;
    R.kernel_launches = launches;
    R.nonfinite = (double)b->h_ctr->stat_nonfinite;
    R.h2d_bytes = (double)(sizeof(WaveCounters) + (sizeof(DevBatchJob) + sizeof(DevNNJob)) * n_jobs +
                           sizeof(int) * n_members);
    R.d2h_bytes = (double)(rounds * (sizeof(WaveCounters) + (train ? sizeof(int) * n_members : 0)));
    R.film_overflow = (double)b->h_ctr->stat_film_overflow;
    check_film(R.film_overflow);
}

// Dispatch on the render mode (as pt_render's modes, without the SD-tree).
void render_batch_mode(pt_batch* b, const pt_batch_job* jobs, int n_jobs, float* const* d_dst, int32_t mode,
                       uint32_t flags) {
    if (mode == PT_MODE_NN) {
        if (flags & ~(PT_FLAG_NN_FREEZE | PT_FLAG_UNBIASED_MIS | PT_FLAG_THROUGHPUT_RR))
            throw Fail(PT_ERR_INVALID, "unsupported flags for the learned-guide render");
        render_batch_slot(b, jobs, n_jobs, d_dst, b->tuning, true, flags);
        return;
    }
    if (mode == PT_MODE_MIS && (flags & PT_FLAG_UNBIASED_MIS)) {
        if (flags & ~(PT_FLAG_UNBIASED_MIS | PT_FLAG_THROUGHPUT_RR))
            throw Fail(PT_ERR_INVALID, "PT_FLAG_UNBIASED_MIS combines only with PT_FLAG_THROUGHPUT_RR");
        render_batch_slot(b, jobs, n_jobs, d_dst, b->tuning, false, flags);
        return;
    }
    if (flags != 0) throw Fail(PT_ERR_INVALID, "unsupported flags for a batch render in this mode");
    if (mode == PT_MODE_SDTREE) throw Fail(PT_ERR_INVALID, "the SD-tree guide does not render in batches");
    if (mode != PT_MODE_MIS && mode != PT_MODE_NEE && mode != PT_MODE_PT) throw Fail(PT_ERR_INVALID, "unknown render mode");
    render_batch(b, jobs, n_jobs, d_dst, b->tuning,
                 mode == PT_MODE_NEE ? kIntegratorNEE : mode == PT_MODE_PT ? kIntegratorPT : kIntegratorMIS);
}

// Copies the batch's own output images to host buffers (null entries skipped).
void copy_out(pt_batch* b, const pt_batch_job* jobs, int n_jobs, float* const* rgb_out) {
    if (!rgb_out) return;
    size_t off = 0, bytes = 0;
    for (int i = 0; i < n_jobs; i++) {
        const pt_batch::Member& m = b->members[jobs[i].scene];
        const size_t n = 3 * (size_t)m.width * m.height;
        if (rgb_out[i]) {
            ck(cudaMemcpyAsync(rgb_out[i], b->d_out + off, sizeof(float) * n, cudaMemcpyDeviceToHost, b->stream),
               "copy image");
            bytes += sizeof(float) * n;
        }
        off += n;
    }
    ck(cudaStreamSynchronize(b->stream), "copy images");
    b->stats.d2h_bytes += (double)bytes;
}

}  // namespace

pt_status pt_batch_create(pt_scene* const* scenes, int32_t n_scenes, pt_batch** out) {
    if (!out) { g_error = "null argument"; return PT_ERR_INVALID; }
    *out = nullptr;
    pt_batch* b = new (std::nothrow) pt_batch;
    if (!b) { g_error = "host allocation failed"; return PT_ERR_MEMORY; }
    const pt_status r = guarded([&] { create_batch(scenes, n_scenes, b); });
    if (r != PT_OK) { delete b; return r; }
    {
        std::lock_guard<std::mutex> lock(lifetime_mutex());
        for (const pt_batch::Member& m : b->members) m.scene->batch_refs++;  // kept alive until the batch goes
    }
    *out = b;
    return PT_OK;
}

void pt_batch_destroy(pt_batch* b) {
    if (!b) return;
    std::vector<pt_scene*> held;
    for (const pt_batch::Member& m : b->members) held.push_back(m.scene);
    delete b;
    std::vector<pt_scene*> dead;
    {
        std::lock_guard<std::mutex> lock(lifetime_mutex());
        for (pt_scene* s : held)
            if (--s->batch_refs == 0 && s->destroy_pending) dead.push_back(s);
    }
    for (pt_scene* s : dead) delete s;
}

pt_status pt_batch_render_device(pt_batch* b, const pt_batch_job* jobs, int32_t n_jobs, float* const* d_rgb_out) {
    if (!b) { g_error = "null batch"; return PT_ERR_INVALID; }
    return guarded([&] { render_batch(b, jobs, n_jobs, d_rgb_out, b->tuning); });
}

pt_status pt_batch_render(pt_batch* b, const pt_batch_job* jobs, int32_t n_jobs, float* const* rgb_out) {
    if (!b) { g_error = "null batch"; return PT_ERR_INVALID; }
    return guarded([&] {
        render_batch(b, jobs, n_jobs, nullptr, b->tuning);
        copy_out(b, jobs, n_jobs, rgb_out);
    });
}

pt_status pt_batch_render_ex(pt_batch* b, const pt_batch_job* jobs, int32_t n_jobs, int32_t mode, uint32_t flags,
                             float* const* rgb_out) {
    if (!b) { g_error = "null batch"; return PT_ERR_INVALID; }
    return guarded([&] {
        render_batch_mode(b, jobs, n_jobs, nullptr, mode, flags);
        copy_out(b, jobs, n_jobs, rgb_out);
    });
}

pt_status pt_batch_render_ex_device(pt_batch* b, const pt_batch_job* jobs, int32_t n_jobs, int32_t mode,
                                    uint32_t flags, float* const* d_rgb_out) {
    if (!b) { g_error = "null batch"; return PT_ERR_INVALID; }
    return guarded([&] { render_batch_mode(b, jobs, n_jobs, d_rgb_out, mode, flags); });
}

pt_status pt_batch_set_tuning(pt_batch* b, const pt_batch_tuning* t) {
    if (!b || !t) { g_error = "null argument"; return PT_ERR_INVALID; }
    return guarded([&] {
        check_tuning(*t);
        b->tuning = *t;
    });
}

pt_status pt_batch_get_tuning(pt_batch* b, pt_batch_tuning* t) {
    if (!b || !t) { g_error = "null argument"; return PT_ERR_INVALID; }
    *t = b->tuning;
    return PT_OK;
}

pt_status pt_batch_stats(pt_batch* b, pt_render_stats* out) {
    if (!b || !out) { g_error = "null argument"; return PT_ERR_INVALID; }
    *out = b->stats;
    return PT_OK;
}

// Autotuner: renders a reduced copy of the job list (spp divided by
// spp_divisor, at least 1) once per candidate setting and keeps the one with
// the highest paths per second.  Candidates: wavefront capacity 2^22 or 2^24
// (scanline order), then scanline or 8x4 / 4x8 / 16x2 pixel tiles at the
// better capacity: five settings.  The render loop runs on the device
// (build_render_graph), so the iterations per loop body only set how often
// its control kernel runs and are kept (16); smaller capacities are clamped
// to the work anyway and never won on the batches measured.
pt_status pt_batch_autotune(pt_batch* b, const pt_batch_job* jobs, int32_t n_jobs, int32_t spp_divisor,
                            pt_batch_tuning* best_out, double* best_mpaths) {
    if (!b) { g_error = "null batch"; return PT_ERR_INVALID; }
    return guarded([&] {
        if (!jobs || n_jobs < 1) throw std::invalid_argument("a batch render needs at least one job");
        if (spp_divisor < 1) throw std::invalid_argument("spp_divisor must be >= 1");
        std::vector<pt_batch_job> sample(jobs, jobs + n_jobs);
        for (pt_batch_job& j : sample) j.spp = std::max(1, j.spp / spp_divisor);
        const int caps[] = {1 << 22, 1 << 24};
        const int tiles[][2] = {{1, 1}, {8, 4}, {4, 8}, {16, 2}};
        const int iters = b->tuning.iters_per_graph;
        pt_batch_tuning best = b->tuning;
        double best_rate = -1.0;
        auto trial = [&](const pt_batch_tuning& t) {
            render_batch(b, sample.data(), n_jobs, nullptr, t);  // warm-up: buffers and graph
            render_batch(b, sample.data(), n_jobs, nullptr, t);
            const double rate = b->stats.paths / (b->stats.render_ms * 1e3);
            if (rate > best_rate) { best_rate = rate; best = t; }
        };
        // capacity first (scanline order), then the tile shape
        for (int c : caps) trial(pt_batch_tuning{c, iters, 1, 1});
        const pt_batch_tuning base = best;
        for (const auto& tl : tiles) {
            if (tl[0] == 1 && tl[1] == 1) continue;
            trial(pt_batch_tuning{base.capacity, base.iters_per_graph, tl[0], tl[1]});
        }
        b->tuning = best;
        if (best_out) *best_out = best;
        if (best_mpaths) *best_mpaths = best_rate;
    });
}
