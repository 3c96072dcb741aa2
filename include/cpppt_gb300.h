/*
 * cpppt_gb300.h -- C ABI of the GB300 path tracer (PT + NEE + MIS and its BVH).
 *
 * Drop-in for the reference's path-tracing path (drcd1/cpp-pt):
 *   - the renderer behind `class Renderer { virtual void render(Scene&,
 *     std::string) = 0; }` (src/renderer/renderer.h:30-33), selected by the
 *     settings key `renderer pathtracer_mis` (src/loader/loader.h:280-281) and
 *     implemented by PathtracerMIS (src/renderer/pathtracerMIS.h:17-168);
 *   - the geometry queries Primitive::intersect / intersect_any
 *     (src/primitive/primitive.h:10-15) of its BVH (src/primitive/bvh.h:50-229).
 *
 * Conventions: plain pointers and sizes, no C++ types.  Every call returns a
 * pt_status and never throws; pt_last_error() describes the last failure on
 * the calling thread.  The caller owns host buffers; the library owns device
 * buffers.  A pt_scene is not safe for concurrent use from several threads.
 */
#ifndef CPPPT_GB300_H
#define CPPPT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t pt_status;
typedef struct pt_scene pt_scene; /* opaque */
#define PT_OK 0
#define PT_ERR_INVALID 1   /* bad argument or scene description */
#define PT_ERR_CUDA 2      /* CUDA runtime error (message in pt_last_error) */
#define PT_ERR_MEMORY 3    /* device allocation failed */
#define PT_ERR_LIMIT 4     /* a bounded loop or queue ran out (kernel status word) */
#define PT_ERR_IO 5        /* scene / settings file could not be read or parsed */
#define PT_ERR_NO_DEVICE 6 /* no CUDA device of compute capability 10.3 */

/* Material kinds of the reference scene model:
 *  DIFFUSE   StandardMaterial with metal < 0.1 -> DiffuseBxDF (diffuse_bxdf.h:25-49)
 *  GGX       StandardMaterial with metal >= 0.1 -> GlossyBxDF(roughness) (glossy_bxdf.h:23-79)
 *  DIELECTRIC RefractionBxDF(ior) (refraction_bxdf.h:17-61)
 *  EMISSIVE  EmissiveMaterial rgb * intensity (emissive_material.h:28-34) */
#define PT_MAT_DIFFUSE 0
#define PT_MAT_GGX 1
#define PT_MAT_DIELECTRIC 2
#define PT_MAT_EMISSIVE 3

typedef struct {
    int32_t kind;
    float rgb[3];     /* albedo, or emission colour */
    float roughness;  /* GGX */
    float ior;        /* dielectric */
    float intensity;  /* emissive: radiance = rgb * intensity */
    float reserved;
} pt_material;        /* 32 bytes */

/* CameraPerspective(res, tan_fovy, origin, normalize(at - origin), up)
 * as Loader::parse_camera builds it (loader.h:117-128). */
typedef struct {
    float origin[3];
    float at[3];
    float up[3];
    float tan_fovy;
    int32_t width, height;
} pt_camera;

/* Flat scene in the reference's insertion order (loader.h:353-367): the
 * global primitive index of a triangle is its position in `triangles`, and
 * emissive triangles become lights in that order. */
typedef struct {
    int32_t n_vertices;
    const float* vertices;     /* 3 per vertex */
    const float* normals;      /* 3 per vertex (the .ptobj normal) */
    const float* tangents;     /* 3 per vertex (the .ptobj tangent); NULL: any perpendicular */
    int32_t n_triangles;
    const int32_t* triangles;  /* 3 vertex indices per triangle */
    const int32_t* tri_material;
    int32_t n_materials;
    const pt_material* materials;
    pt_camera camera;
} pt_scene_desc;

/* Ray as the reference's Ray (src/primitive/ray.h:8-20): origin, direction,
 * max_t; 7 packed floats. */
typedef struct {
    float o[3];
    float d[3];
    float max_t;
} pt_ray;

/* Closest hit: prim = insertion index of the triangle BVH::intersect reports
 * (-1: none); t = the ray's max_t after the query (triangle.h:106);
 * beta/gamma = barycentrics of the hit (triangle.h:63-74). */
typedef struct {
    float t;
    int32_t prim;
    float beta, gamma;
} pt_hit;

/* Integrator modes. */
#define PT_MODE_MIS 0       /* PathtracerMIS, reference estimator (default) */
#define PT_MODE_SDTREE 1    /* SD-tree guided (practical path guiding) */
#define PT_MODE_NN 2        /* learned (MLP, vMF mixture) guiding */
#define PT_MODE_NEE 3       /* Pathtracer: NEE without MIS (pathtracer.h:27-102) */
#define PT_MODE_PT 4        /* PurePt: BSDF sampling only, no NEE (pure_pt.h:28-71) */

typedef struct {
    int32_t spp;        /* samples per pixel (the reference settings value `spp N` means N*N) */
    int32_t max_depth;  /* maximum path segments; reference: 32 (pathtracerMIS.h:36) */
    int32_t rr_start;   /* Russian roulette from this bounce index; reference: 3 (i > 2, :118) */
    uint32_t seed;      /* random stream of this render */
    int32_t mode;       /* PT_MODE_* */
    int32_t flags;      /* PT_FLAG_* bits (below); 0 = the reference's estimator */
} pt_render_desc;

/* Counters of the last render on a scene. */
typedef struct {
    double paths;            /* camera paths traced */
    double closest_rays;     /* closest-hit queries (extension rays) */
    double shadow_rays;      /* any-hit queries (NEE shadow rays) */
    double render_ms;        /* device time of the render loop (CUDA events) */
    double trace_closest_ms; /* device time inside the closest-hit kernel */
    double trace_shadow_ms;  /* device time inside the any-hit kernel */
    double iterations;       /* wavefront iterations */
    double kernel_launches;  /* kernels launched by the render */
    double extend_nodes;     /* wide-BVH nodes visited by extension rays (PT_FLAG_COUNT renders) */
    double extend_tris;      /* triangles tested by extension rays (PT_FLAG_COUNT renders) */
    double h2d_bytes;        /* host-to-device bytes copied by the call */
    double d2h_bytes;        /* device-to-host bytes copied by the call */
    double nonfinite;        /* contributions dropped because they were inf or NaN */
    double film_overflow;    /* contributions the film could not hold: the film keeps signed 32.32
                                fixed-point sums (a pixel's sum below 2^31); when non-zero the
                                render returned PT_ERR_LIMIT */
} pt_render_stats;

/* pt_render_desc.flags */
#define PT_FLAG_TIME_KERNELS 1 /* launch iterations directly with CUDA events around the traversal kernels */
#define PT_FLAG_COUNT 2        /* counting build of the extension kernel (visited nodes / tested triangles) */
#define PT_FLAG_UNBIASED_MIS 4 /* PT_MODE_MIS with MIS weights on the unscaled pdf, Russian roulette
                                  survival min(rr, 1) and full NEE weight at the last vertex: the
                                  unbiased estimator of the depth-limited image that the learned guide
                                  also uses (the default keeps the reference's RR-scaled weights,
                                  pathtracerMIS.h:118-124, and its MIS weight at the last vertex) */
#define PT_FLAG_NN_FREEZE 8    /* PT_MODE_NN: use the current network without training it */
#define PT_FLAG_THROUGHPUT_RR 16 /* PT_MODE_NN or PT_FLAG_UNBIASED_MIS: Russian roulette on the path
                                    throughput (survival min(1, max component of the throughput after
                                    the bounce); survivors are not boosted above 1) instead of the
                                    reference's survival on the BSDF value (pathtracerMIS.h:118-124) */

/* Replaces: Loader::load_scene + BVH::add/build (loader.h:314-374,
 * bvh.h:205-216) for a scene given as flat arrays.  Builds the
 * reference-topology BVH (for tie-breaks; on the device, bit-identical to
 * BVH::build) and the wide traversal BVH, and uploads the scene to the
 * current CUDA device. */
pt_status pt_scene_create(const pt_scene_desc* desc, pt_scene** scene);

/* Replaces: Loader::load_render_settings + Loader::load_scene
 * (loader.h:256-374) -- reads a render-settings file and the .ptscene /
 * .ptobj / .ptmat files it names.  `settings` receives spp (= N*N for
 * `spp N`), max_depth 32, rr_start 3.  width/height come from `resolution`. */
pt_status pt_scene_load(const char* settings_file, pt_scene** scene, pt_render_desc* settings,
                        char* output_name, int32_t output_name_len);

/* Frees the scene; for a member of a live batch (pt_batch_create) the
 * release waits until the last such batch is destroyed. */
void pt_scene_destroy(pt_scene* scene);

/* Image resolution of the scene's camera, its triangle and light counts. */
pt_status pt_scene_info(pt_scene* scene, int32_t* width, int32_t* height, int32_t* n_triangles, int32_t* n_lights);

/* Replaces: BVH::intersect(Ray&, Intersection*) (bvh.h:219-221) on a batch of
 * rays in host memory.  Same hit and same tie-break as the reference: the
 * smallest t among the triangles the reference tests; on equal t the one it
 * visits last. */
pt_status pt_trace_closest(pt_scene* scene, const pt_ray* rays, int32_t n, pt_hit* hits);

/* Replaces: BVH::intersect_any(Ray&) (bvh.h:222-224) on a host batch;
 * occluded[i] = 1 when the reference reports a hit. */
pt_status pt_trace_any(pt_scene* scene, const pt_ray* rays, int32_t n, uint8_t* occluded);

/* Device-pointer variants: rays/hits in device memory, enqueued on `stream`
 * (a cudaStream_t, NULL for the legacy default stream); asynchronous. */
pt_status pt_trace_closest_device(pt_scene* scene, const pt_ray* d_rays, int32_t n, pt_hit* d_hits, void* stream);
pt_status pt_trace_any_device(pt_scene* scene, const pt_ray* d_rays, int32_t n, uint8_t* d_occluded, void* stream);

/* Replaces: PathtracerMIS::render(Scene&, filename) (pathtracerMIS.h:135-167)
 * without the file writes: renders desc->spp samples per pixel and writes
 * width*height*3 floats (row-major from the top row, as Image::put_pixel,
 * rgb_image.h:208-210) to the host buffer rgb_out. */
pt_status pt_render(pt_scene* scene, const pt_render_desc* desc, float* rgb_out);

/* Device variant: leaves the average in a device buffer of width*height*3
 * floats; enqueued on the scene's stream and synchronised before return. */
pt_status pt_render_device(pt_scene* scene, const pt_render_desc* desc, float* d_rgb_out);

/* Allocation-free render; it has no counterpart in the reference (whose
 * renderer runs on the CPU).  For callers that cannot allocate device memory
 * when they render: a host whose GPU memory is reserved up front by another
 * allocator or an engine's budget (a further cudaMalloc would fail or evict
 * its pools), or a frame loop that must stay off the driver's allocation
 * path.  Same arguments, algorithm and image as pt_render_device
 * (bit-identical for the same desc), enqueued on `stream` and synchronised
 * before return (the host polls the wavefront's counters between rounds of
 * iterations), but it calls no cudaMalloc/cudaFree: its scratch (path state,
 * queues, film, counters) is one fixed array of about 19 MB in the library's
 * device memory, which every GPU that loads the library holds until the
 * process exits.  Limits: at most 262144 pixels (e.g. 512 x 512),
 * PT_MODE_MIS, flags 0; larger images return PT_ERR_LIMIT.  The scene must
 * belong to the current device (PT_ERR_INVALID otherwise).  The first call on
 * a device looks up the array's device address; make that first call before
 * any stream capture begins.  All calls share the array: calls that overlap
 * on the GPU (other threads or streams) race on it.  The call fills the
 * scene's pt_render_stats (paths, rays, iterations) like pt_render. */
pt_status pt_render_device_noalloc(pt_scene* scene, const pt_render_desc* desc, float* d_rgb_out, void* stream);

pt_status pt_render_stats_get(pt_scene* scene, pt_render_stats* stats);

/* Multi-scene batches.  No counterpart in the reference, which renders one
 * scene per process (main.cpp); each job of a batch is the equivalent of one
 * pt_render call (PathtracerMIS::render, pathtracerMIS.h:145-167) and gives
 * the bit-identical image, but all jobs share one wavefront on the GPU.
 * pt_batch_create copies the scenes' device data into one merged arena (the
 * scenes stay valid and independent; at most 2^27 - 1 triangles in total).
 * A job renders scene `scene` (index into the creation list) with spp,
 * max_depth, rr_start and seed as pt_render_desc with PT_MODE_MIS, flags 0.
 * rgb_out[i] / d_rgb_out[i]: 3 floats per pixel of job i's scene (host or
 * device memory; a null entry skips that copy). */
typedef struct pt_batch pt_batch;
typedef struct pt_batch_job {
    int32_t scene;
    int32_t spp;
    int32_t max_depth;
    int32_t rr_start;
    uint32_t seed;
} pt_batch_job;
/* Launch shape of a batch: paths in flight (multiple of 1024, <= 2^24; a
 * learned-guide batch uses at most 2^22),
 * wavefront iterations per CUDA graph launch (even), pixel tile of the
 * path order (1 x 1 = scanline; used where it divides the resolution).
 * None of them changes the images. */
typedef struct pt_batch_tuning {
    int32_t capacity;
    int32_t iters_per_graph;
    int32_t tile_w;
    int32_t tile_h;
} pt_batch_tuning;
pt_status pt_batch_create(pt_scene* const* scenes, int32_t n_scenes, pt_batch** batch);
void pt_batch_destroy(pt_batch* batch);
pt_status pt_batch_render(pt_batch* batch, const pt_batch_job* jobs, int32_t n_jobs, float* const* rgb_out);
pt_status pt_batch_render_device(pt_batch* batch, const pt_batch_job* jobs, int32_t n_jobs, float* const* d_rgb_out);
/* pt_batch_render with a render mode and flags as pt_render_desc (all
 * modes but PT_MODE_SDTREE).  PT_MODE_NN: every job is guided by its scene's
 * own learned guide (pt_nn_configure / pt_nn_reset / pt_nn_stats of that
 * scene), and each scene's guide trains online on the records of that
 * scene's paths unless PT_FLAG_NN_FREEZE; PT_MODE_MIS with
 * PT_FLAG_UNBIASED_MIS: the same estimator with BSDF sampling only.  With
 * frozen guides each job's image is bit-identical to pt_render of the same
 * scene, mode and flags.  The guides live in the member scenes, which the
 * batch keeps alive (see pt_scene_destroy).  Replaces nothing in the
 * reference (it renders one scene at a time). */
pt_status pt_batch_render_ex(pt_batch* batch, const pt_batch_job* jobs, int32_t n_jobs, int32_t mode, uint32_t flags,
                             float* const* rgb_out);
pt_status pt_batch_render_ex_device(pt_batch* batch, const pt_batch_job* jobs, int32_t n_jobs, int32_t mode,
                                    uint32_t flags, float* const* d_rgb_out);
pt_status pt_batch_set_tuning(pt_batch* batch, const pt_batch_tuning* tuning);
pt_status pt_batch_get_tuning(pt_batch* batch, pt_batch_tuning* tuning);
/* Statistics of the last batch render (paths, rays, time; per batch). */
pt_status pt_batch_stats(pt_batch* batch, pt_render_stats* stats);
/* Times every candidate launch shape on the jobs with spp / spp_divisor
 * (at least 1) and keeps the fastest; returns it and its Mpaths/s. */
pt_status pt_batch_autotune(pt_batch* batch, const pt_batch_job* jobs, int32_t n_jobs, int32_t spp_divisor,
                            pt_batch_tuning* best, double* best_mpaths);

/* pt_scene_load caches each parsed .ptobj mesh next to it as <file>.gbbin
 * (positions, normals, tangents, faces; keyed by the source's size and
 * modification time) and reads the cache instead of the text when it is
 * current.  Enabled by default; 0 turns reading and writing the cache off
 * for later loads in this process.  Replaces nothing in the reference (its
 * text parser, loader.h:209-251, has no cache). */
void pt_set_mesh_cache(int32_t enabled);

/* Writes <prefix>.png (sRGB, 8-bit, clipped as pixel_ops::put2char1) and
 * <prefix>.hdr (Radiance RGBE), as Image::save (rgb_image.h:300-318). */
pt_status pt_image_save(const char* prefix, const float* rgb, int32_t width, int32_t height);

/* Learned guide (PT_MODE_NN) state of a scene: the network's FP32 weights
 * (15360 floats: 64x64, 64x64, 64x64, 64x48, each row-major [in][out]).
 * Has no counterpart in the reference (its only guide is the SD-tree). */
#define PT_NN_WEIGHTS 15360
pt_status pt_nn_get_weights(pt_scene* scene, float* weights);
pt_status pt_nn_set_weights(pt_scene* scene, const float* weights); /* also resets Adam */
pt_status pt_nn_reset(pt_scene* scene, uint32_t seed);                 /* fresh random weights */
/* training steps taken and the mean loss of the last step */
pt_status pt_nn_stats(pt_scene* scene, double* steps, double* last_loss, double* records_used);

/* Online training and sampling settings of a scene's learned guide.  The
 * BSDF selection probability is c = bsdf_frac_min + (bsdf_frac_max -
 * bsdf_frac_min) sigmoid(logit); 0.1 <= bsdf_frac_min <= bsdf_frac_max <= 1
 * (equal values fix c).  batch: training records per Adam step, in
 * [1024, 262144].  divergence: PT_NN_KL weighs each record by its target
 * T (Kullback-Leibler), PT_NN_CHI2 by T^2 (Pearson chi-square: the variance
 * of the estimator; it favours the rare bright directions).  Records are
 * collected for up to steps_per_round batches (in [1, 64], at most 2^22
 * records) between the host's checks of the wavefront (every 16
 * iterations); each full batch is one Adam step.
 * Defaults: 3e-3, 0.3, 0.9, 65536, PT_NN_CHI2, 16 (a BSDF fraction of at least
 * 0.3 bounds the growth of a path's throughput through poorly guided
 * bounces, the main source of rare very bright samples; batches of 2^16
 * take four times the Adam steps of 2^18 on the same records and learned
 * faster per second of rendering on the occluded-light room). */
#define PT_NN_KL 0
#define PT_NN_CHI2 1
typedef struct pt_nn_config {
    float learning_rate;
    float bsdf_frac_min;
    float bsdf_frac_max;
    int32_t batch;
    int32_t divergence;
    int32_t steps_per_round; /* batches at most per wavefront round (16 iterations), 1..64 */
    int32_t encoding;        /* PT_NN_ENC_FREQ (default) or PT_NN_ENC_ONEBLOB; reset the weights
                                (pt_nn_reset) after changing it */
    int32_t passes;          /* Adam steps taken on each batch of records, 1..8 (default 1);
                                steps_per_round counts batches */
} pt_nn_config;
/* Input encodings of the learned guide (64 inputs, the last constant 1):
 * FREQ: sin / cos of the position normalised to the scene box at 8
 *   octaves per axis (48), then the shading normal and wo as they are;
 * ONEBLOB: the position at 6 octaves per axis (36), then the normal's and
 *   wo's cos theta and phi, each mapped to [0, 1] and spread over 6
 *   Gaussian bins (one-blob encoding, sigma = 1/6; phi wraps around). */
#define PT_NN_ENC_FREQ 0
#define PT_NN_ENC_ONEBLOB 1
pt_status pt_nn_configure(pt_scene* scene, const pt_nn_config* config);
pt_status pt_nn_config_get(pt_scene* scene, pt_nn_config* config);

/* Diagnostics of the learned guide on the current CUDA device (no scene):
 * forward: inputs 9 floats per sample (position, shading normal, wo),
 *   positions normalised with lo/hi; out 41 floats per sample (8 lobes x
 *   (mean xyz, kappa, weight), BSDF selection probability).
 * grad: records 16 floats each (pos, normal, wo, wi, p_bsdf(wi), T, 0, 0);
 *   out_grad receives dL/dW (PT_NN_WEIGHTS floats) of
 *   L = -sum T log(c p_bsdf + (1-c) q(wi)) / sum T, out_loss receives L. */
pt_status pt_debug_nn_forward(const float* weights, const float* lo, const float* hi, const float* inputs, int32_t n,
                              float* out);
pt_status pt_debug_nn_grad(const float* weights, const float* lo, const float* hi, const float* records, int32_t n,
                           float* out_grad, float* out_loss);
/* The renderer's own training step on a host batch (without the Adam
 * update): T summed on the device and, for PT_NN_CHI2, squared first
 * (records weighted by T^2), with the BSDF selection probability in
 * [c_lo, c_hi] (pt_nn_configure's range; 0.1 <= c_lo <= c_hi <= 1). */
pt_status pt_debug_nn_grad_ex(const float* weights, const float* lo, const float* hi, const float* records, int32_t n,
                              int32_t divergence, float c_lo, float c_hi, int32_t encoding, float* out_grad,
                              float* out_loss);
/* pt_debug_nn_forward with the input encoding (PT_NN_ENC_*). */
pt_status pt_debug_nn_forward_ex(const float* weights, const float* lo, const float* hi, const float* inputs,
                                 int32_t n, int32_t encoding, float* out);

/* Unit-test hooks of the integrator's own device functions, checked against
 * the oracle on the same numbers.  pt_debug_bsdf runs BxDF::eval, ::pdf,
 * ::sample and BxDF::same_hemisphere (diffuse_bxdf.h:25-49,
 * glossy_bxdf.h:23-79, microfacet_distribution.h:9-168,
 * refraction_bxdf.h:17-61, bxdf.h:42-57) on the current device.  Per case,
 * 20 floats: kind (PT_MAT_*), rgb, roughness, ior, the vertex normal and
 * tangent of a flat triangle (the shading frame of a path's first hit),
 * wo, wi, and the two uniform numbers of the sample.  Per case out, 10
 * floats: eval(wo, wi) (3, the cosine included), pdf(wo, wi),
 * same_hemisphere(wo, wi) (0/1), the sampled wi (3), its pdf, delta (0/1).
 * pt_debug_light_sample runs LightGroup::connect_eye_path
 * (light_group.h:25-30, shape_light.h:24-44, triangle.h:209-269) on the
 * scene's emitters: 6 floats per case in (the shaded point, then the
 * numbers picking the light and the point on it), 10 out (position,
 * normal, Le |n_l . w|, pdf). */
pt_status pt_debug_bsdf(int32_t n, const float* cases, float* out);

/* Error-path hooks.  pt_debug_traversal_limits lowers the scene's kernel-side
 * traversal bounds (steps of a ray's loop, default 2^22; entries of its
 * stack, default 64; 0 restores a default): a query or render that runs out
 * returns PT_ERR_LIMIT and leaves the context usable.
 * pt_debug_tensor_wait_timeout runs one CTA that waits, bounded, on a
 * tensor-core completion barrier nothing arrives on, through the timeout
 * path of the learned guide's kernels: it returns PT_ERR_CUDA ("tensor-core
 * completion wait timed out") and leaves the context usable. */
pt_status pt_debug_traversal_limits(pt_scene* scene, int32_t step_limit, int32_t stack_limit);
pt_status pt_debug_tensor_wait_timeout(void);
pt_status pt_debug_light_sample(pt_scene* scene, int32_t n, const float* cases, float* out);

/* Message of the last failed call on this thread ("" when none). */
const char* pt_last_error(void);

/* Diagnostic, host only (no CUDA call): the reference BVH topology the
 * library derives for a triangle list -- BVH::build (bvh.h:151-216) --
 * as used for the tie-break.  tri_v: 9 floats per triangle (a, b, c).
 * Outputs: leaf_order[n] (insertion indices in the order BVHNode::intersect
 * visits leaves), prim_parent[n] (innermost internal node above each
 * triangle, -1 when the root is a leaf), node_boxes[6 * max_nodes]
 * (min xyz, max xyz per internal node, pre-order); *n_nodes receives the
 * internal-node count (PT_ERR_LIMIT when it exceeds max_nodes). */
/* Diagnostic, host only (no CUDA call): the library's SD-tree update
 * (SDTree::splat / update / pdf, src/algorithms/sdtree.h:445-537) run for
 * n_iters rounds of {splat that round's records, update}.  splats: 7 floats
 * each {radiance, pos xyz, dir xyz}.  Outputs per spatial leaf (depth
 * first, child 0 first): its sampling leaves (4 floats: begin phi, begin
 * cos theta, size phi, size cos theta, into out_leaves up to max_leaves),
 * their number, the splat count and flux; and the pdf of each query
 * (6 floats: pos, dir).  *n_spatial receives the spatial-leaf count. */
pt_status pt_debug_sdtree_run(const float* lo, const float* hi, int32_t n_iters, const int32_t* n_splats,
                              const float* splats, int32_t max_leaves, float* out_leaves, int32_t* out_leaf_counts,
                              int32_t* out_counts, float* out_flux, int32_t n_queries, const float* queries,
                              float* out_pdf, int32_t* n_spatial);

/* Texture decoding as a material's image(...) texture sees it (host only):
 * the file's pixels as the reference's Image<Vec3> (rgb = 1) or
 * Image<float> (rgb = 0) holds them after loading (rgb_image.h:160-205),
 * sRGB-converted when srgb = 1.  PNG and Radiance .hdr files.  out: w * h *
 * (rgb ? 3 : 1) floats, top row first; with out = NULL (or cap too small)
 * only *w and *h are set (PT_ERR_LIMIT when out is given but too small). */
pt_status pt_debug_image_load(const char* path, int32_t rgb, int32_t srgb, int32_t* w, int32_t* h, float* out,
                              int64_t cap);
pt_status pt_debug_ref_topology(const float* tri_v, int32_t n, int32_t* leaf_order, int32_t* prim_parent,
                                float* node_boxes, int32_t max_nodes, int32_t* n_nodes);
/* The same topology built on the current device (level-synchronous binning
 * kernels, bit-identical to the host build and to BVH::build); *levels
 * receives the number of tree levels. */
pt_status pt_debug_ref_topology_device(const float* tri_v, int32_t n, int32_t* leaf_order, int32_t* prim_parent,
                                       float* node_boxes, int32_t max_nodes, int32_t* n_nodes, int32_t* levels);

/* The 4-wide traversal tree the library builds for a triangle list (binned
 * SAH, 32 bins, leaves of at most max_leaf triangles, collapsed to 64-byte
 * compressed nodes), built on the current device (on_device = 1, as scenes
 * are) or on the host with host_threads threads (on_device = 0; 0 = all
 * hardware threads; no CUDA call).  Both builds give the same bytes.
 * Outputs: nodes[16 * max_nodes] (16 words per node, breadth first),
 * *n_nodes, tri_order[n] (leaf order -> insertion index), *max_depth (tree
 * levels), *inflate (the absolute box inflation).  PT_ERR_LIMIT when the
 * tree has more than max_nodes nodes (*n_nodes is set). */
pt_status pt_debug_wide_bvh(const float* tri_v, int32_t n, int32_t max_leaf, int32_t on_device, int32_t host_threads,
                            uint32_t* nodes, int32_t max_nodes, int32_t* n_nodes, int32_t* tri_order,
                            int32_t* max_depth, float* inflate);

#ifdef __cplusplus
}
#endif
#endif /* CPPPT_GB300_H */
