/*
 * pt_oracle.c -- CPU restatement of the reference path tracer's hot path
 * (drcd1/cpp-pt: PathtracerMIS + its BVH).  TEST INFRASTRUCTURE ONLY: the
 * tests, the golden-fixture script and bench.py's CPU-baseline leg load it
 * through ctypes as a checker.  Nothing in the product links or calls it.
 *
 * Parity is pinned against the reference itself: tests/golden holds outputs
 * of the compiled reference (oracle/ref_harness.cpp) for the BVH topology,
 * closest/any-hit queries and small renders; test_oracle_pins.py checks this
 * file reproduces them bit for bit.
 *
 * Arithmetic follows the reference expression by expression, including its
 * implicit float<->double promotions (EPS is the double literal 1e-4,
 * src/math/math.h:11; Vec3 / s multiplies by float(1.0/s), math.h:105-107).
 * Build with -ffp-contract=off so no multiply-add is fused.
 *
 * Deliberate difference: BVH::build_node (bvh.h:151-202) recurses forever when
 * a split leaves one side empty (e.g. >=4 primitives with equal centroids).
 * Here such a node becomes a leaf holding all its primitives.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_EPS 1e-4 /* math.h:11, a double */
#define OR_PI 3.14159265358979323846

typedef struct { float x, y, z; } v3;

static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vscale(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
/* Vector3::operator/(T a): (*this) * (1.0 / a), the double quotient
 * converted to the float parameter of operator*(T) (math.h:105-107). */
static inline v3 vdivs(v3 a, float s) { return vscale(a, (float)(1.0 / (double)s)); }
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
    return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float vlen(v3 a) { return sqrtf(vdot(a, a)); }
static inline v3 vnorm(v3 a) { return vdivs(a, vlen(a)); }
static inline v3 vneg(v3 a) { return vscale(a, (float)-1.0); }
static inline v3 vminf(v3 a, v3 b) { return V(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z); }
static inline v3 vmaxf(v3 a, v3 b) { return V(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z); }
static inline float vget(v3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

/* Mat3 stored row-major as in math.h:224-260; Mat3(x,y,z) takes columns. */
typedef struct { float m[9]; } m3;
static inline m3 mcols(v3 x, v3 y, v3 z) {
    m3 r = {{x.x, y.x, z.x, x.y, y.y, z.y, x.z, y.z, z.z}};
    return r;
}
static inline v3 mmul(const m3* M, v3 a) { /* math.h:319-325 */
    const float* v = M->m;
    return V(v[0] * a.x + v[1] * a.y + v[2] * a.z, v[3] * a.x + v[4] * a.y + v[5] * a.z,
             v[6] * a.x + v[7] * a.y + v[8] * a.z);
}
static inline m3 mtranspose(const m3* M) { /* math.h:366-382 */
    const float* v = M->m;
    m3 r = {{v[0], v[3], v[6], v[1], v[4], v[7], v[2], v[5], v[8]}};
    return r;
}

/* ----------------------------------------------------------------------- */
/* mt19937 + libstdc++ uniform_real_distribution<float>(0,1)               */
/* (RandomSampler, src/math/sampler.h:13-23).  MT19937 is the published     */
/* generator of Matsumoto & Nishimura (1998); the float draw follows        */
/* generate_canonical<float,24>: one 32-bit word w, float(w) * 2^-32,       */
/* mapped to the largest float below 1 when it rounds to 1.                 */
/* ----------------------------------------------------------------------- */
typedef struct { uint32_t s[624]; int i; } mt19937;

static void mt_seed(mt19937* g, uint32_t seed) {
    g->s[0] = seed;
    for (int i = 1; i < 624; i++) g->s[i] = 1812433253u * (g->s[i - 1] ^ (g->s[i - 1] >> 30)) + (uint32_t)i;
    g->i = 624;
}

static uint32_t mt_next(mt19937* g) {
    if (g->i >= 624) {
        for (int k = 0; k < 624; k++) {
            uint32_t y = (g->s[k] & 0x80000000u) | (g->s[(k + 1) % 624] & 0x7fffffffu);
            uint32_t v = g->s[(k + 397) % 624] ^ (y >> 1);
            if (y & 1u) v ^= 0x9908b0dfu;
            g->s[k] = v;
        }
        g->i = 0;
    }
    uint32_t y = g->s[g->i++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

static float mt_float(mt19937* g) {
    float sum = (float)mt_next(g);
    float r = sum / 4294967296.0f;
    if (r >= 1.0f) r = nextafterf(1.0f, 0.0f);
    return r;
}

/* ----------------------------------------------------------------------- */
/* Scene                                                                    */
/* ----------------------------------------------------------------------- */
enum { MAT_DIFFUSE = 0, MAT_GGX = 1, MAT_DIELECTRIC = 2, MAT_EMISSIVE = 3 };

typedef struct {
    int n_tris, n_verts;
    v3* pos;    /* per vertex */
    v3* nrm;    /* per vertex, as given */
    v3* btan;   /* per vertex: cross(normal, tangent), loader.h:237 */
    int* tri;   /* 3 global vertex indices per triangle */
    int* tri_mat;
    int n_mats;
    int* mat_kind;
    float* mat_params; /* 8 per material: r g b roughness ior intensity - - */
    /* lights: one per emissive triangle in insertion order (loader.h:362-364) */
    int n_lights;
    int* light_tri;
    int* tri_light; /* -1 when not emissive */
    /* BVH replica */
    int n_nodes;      /* internal nodes, pre-order */
    float* node_box;  /* 6 per node */
    int* node_child;  /* 2 per node: >=0 internal node, <0: ~leaf */
    int* node_parent;
    int n_leaves;
    int* leaf_start; /* into leaf_prims */
    int* leaf_count;
    int* leaf_prims; /* DFS order of primitives */
    int* prim_parent;
    int root; /* >=0 internal node, <0 leaf, or 0x7fffffff when empty */
    int fast;       /* queries by the culling traversal (closest_fast / any_fast) */
    float fast_pad; /* box inflation of the culling test */
    /* image textures (loader.h:78-92, image_texture.h, rgb_image.h): uv per
     * vertex (2 floats), texture pixels as the reference's Image holds them,
     * {first float, width, height, channels} per texture, and per material
     * the texture of albedo / emission colour, roughness, metal, normal map
     * (-1: constant) and the intensity of a textured emitter */
    float* uv;
    int n_tex;
    int* tex_info;
    float* tex_px;
    int* mat_tex;
    float* mat_emit;
    /* camera (camera_perspective.h:19-39) */
    v3 cam_origin;
    m3 cam_coords;
    float tan_fovy, aspect;
    int width, height;
} or_scene;

/* Triangle::get_bounds, triangle.h:197-207 */
static void tri_bounds(const or_scene* s, int t, v3* mn, v3* mx) {
    v3 a = s->pos[s->tri[3 * t]], b = s->pos[s->tri[3 * t + 1]], c = s->pos[s->tri[3 * t + 2]];
    *mn = vminf(vminf(a, b), c);
    *mx = vmaxf(vmaxf(a, b), c);
}

/* AABB::area, aabb.h:77-82 (float products summed, doubled in double) */
static float box_area(v3 mn, v3 mx) {
    float s = fabsf(mx.x - mn.x) * (mx.y - mn.y) + fabsf(mx.z - mn.z) * (mx.y - mn.y) +
              fabsf(mx.x - mn.x) * (mx.z - mn.z);
    return (float)(2.0 * (double)s);
}

/* ---- BVH build: BVH::compute_split / build_node (bvh.h:57-202) ---- */
typedef struct {
    or_scene* s;
    v3* bmin; v3* bmax; v3* cen; /* per primitive */
    int cap_nodes, cap_leaves;
    int n_leaf_prims;
} builder;

static void b_push_node(builder* B) {
    or_scene* s = B->s;
    if (s->n_nodes >= B->cap_nodes) {
        B->cap_nodes = B->cap_nodes ? 2 * B->cap_nodes : 64;
        s->node_box = realloc(s->node_box, sizeof(float) * 6 * B->cap_nodes);
        s->node_child = realloc(s->node_child, sizeof(int) * 2 * B->cap_nodes);
        s->node_parent = realloc(s->node_parent, sizeof(int) * B->cap_nodes);
    }
}

static int b_make_leaf(builder* B, const int* prims, int n, int parent) {
    or_scene* s = B->s;
    if (s->n_leaves >= B->cap_leaves) {
        B->cap_leaves = B->cap_leaves ? 2 * B->cap_leaves : 64;
        s->leaf_start = realloc(s->leaf_start, sizeof(int) * B->cap_leaves);
        s->leaf_count = realloc(s->leaf_count, sizeof(int) * B->cap_leaves);
    }
    int id = s->n_leaves++;
    s->leaf_start[id] = B->n_leaf_prims;
    s->leaf_count[id] = n;
    for (int i = 0; i < n; i++) {
        s->leaf_prims[B->n_leaf_prims++] = prims[i];
        s->prim_parent[prims[i]] = parent;
    }
    return ~id;
}

/* compute_split for one axis; writes the left/right lists, returns cost. */
static float b_split(builder* B, int axis, const int* prims, int n, v3 cmin, v3 cmax, int* out,
                     int* n_left, int* part_of) {
    const int P = 5;
    float lo = vget(cmin, axis), hi = vget(cmax, axis);
    int counts[5] = {0, 0, 0, 0, 0};
    for (int q = 0; q < n; q++) {
        int i = prims[q];
        float c = vget(B->cen[i], axis);
        int bin = P - 1;
        for (int j = 0; j < P - 1; j++) {
            float thr = lo + (hi - lo) * (float)(j + 1) / (float)P;
            if (c < thr) { bin = j; break; }
        }
        part_of[q] = bin;
        counts[bin]++;
    }
    float cost[4];
    for (int i = 0; i < P - 1; i++) {
        v3 lmn = V(INFINITY, INFINITY, INFINITY), lmx = V(-INFINITY, -INFINITY, -INFINITY);
        v3 rmn = lmn, rmx = lmx;
        int lc = 0, rc = 0;
        /* partitions are visited bin by bin, each in insertion order */
        for (int j = 0; j < P; j++)
            for (int q = 0; q < n; q++) {
                if (part_of[q] != j) continue;
                int p = prims[q];
                if (j <= i) { lc++; lmn = vminf(lmn, B->bmin[p]); lmx = vmaxf(lmx, B->bmax[p]); }
                else { rc++; rmn = vminf(rmn, B->bmin[p]); rmx = vmaxf(rmx, B->bmax[p]); }
            }
        cost[i] = (lc == 0 || rc == 0) ? INFINITY : box_area(lmn, lmx) + box_area(rmn, rmx);
    }
    int best = 0;
    float best_cost = cost[0];
    for (int i = 1; i < P - 1; i++)
        if (cost[i] < best_cost) { best_cost = cost[i]; best = i; }
    int k = 0;
    for (int j = 0; j <= best; j++)
        for (int q = 0; q < n; q++) if (part_of[q] == j) out[k++] = prims[q];
    *n_left = k;
    for (int j = best + 1; j < P; j++)
        for (int q = 0; q < n; q++) if (part_of[q] == j) out[k++] = prims[q];
    return best_cost;
}

static int b_build(builder* B, int* prims, int n, int parent) {
    if (n < 4) return b_make_leaf(B, prims, n, parent);
    v3 bmn = V(INFINITY, INFINITY, INFINITY), bmx = V(-INFINITY, -INFINITY, -INFINITY);
    v3 cmn = bmn, cmx = bmx;
    for (int q = 0; q < n; q++) {
        int p = prims[q];
        bmn = vminf(bmn, B->bmin[p]); bmx = vmaxf(bmx, B->bmax[p]);
        cmn = vminf(cmn, B->cen[p]); cmx = vmaxf(cmx, B->cen[p]);
    }
    int* tmp = malloc(sizeof(int) * 4 * n);
    int* s0 = tmp; int* s1 = tmp + n; int* s2 = tmp + 2 * n; int* part = tmp + 3 * n;
    int l0, l1, l2;
    float c1 = b_split(B, 0, prims, n, cmn, cmx, s0, &l0, part);
    float c2 = b_split(B, 1, prims, n, cmn, cmx, s1, &l1, part);
    float c3 = b_split(B, 2, prims, n, cmn, cmx, s2, &l2, part);
    int* chosen; int nl;
    /* bvh.h:179-197 */
    if (c1 < c2) {
        if (c1 < c3) { chosen = s0; nl = l0; }
        else if (c2 < c3) { chosen = s1; nl = l1; }
        else { chosen = s2; nl = l2; }
    } else if (c2 < c3) { chosen = s1; nl = l1; }
    else { chosen = s2; nl = l2; }
    if (nl == 0 || nl == n) { /* the reference would not terminate here */
        int leaf = b_make_leaf(B, prims, n, parent);
        free(tmp);
        return leaf;
    }
    memcpy(prims, chosen, sizeof(int) * n);
    free(tmp);
    b_push_node(B);
    or_scene* s = B->s;
    int id = s->n_nodes++;
    float* bx = s->node_box + 6 * id;
    bx[0] = bmn.x; bx[1] = bmn.y; bx[2] = bmn.z; bx[3] = bmx.x; bx[4] = bmx.y; bx[5] = bmx.z;
    s->node_parent[id] = parent;
    /* the left partition is stored in member `right` and visited first */
    int a = b_build(B, prims, nl, id);
    int b = b_build(B, prims + nl, n - nl, id);
    s->node_child[2 * id] = a;
    s->node_child[2 * id + 1] = b;
    return id;
}

static void bvh_build(or_scene* s) {
    builder B;
    memset(&B, 0, sizeof(B));
    B.s = s;
    int n = s->n_tris;
    B.bmin = malloc(sizeof(v3) * (n ? n : 1));
    B.bmax = malloc(sizeof(v3) * (n ? n : 1));
    B.cen = malloc(sizeof(v3) * (n ? n : 1));
    for (int t = 0; t < n; t++) {
        tri_bounds(s, t, &B.bmin[t], &B.bmax[t]);
        B.cen[t] = vscale(vadd(B.bmin[t], B.bmax[t]), 0.5f); /* AABB::center, aabb.h:62-64 */
    }
    s->leaf_prims = malloc(sizeof(int) * (n ? n : 1));
    s->prim_parent = malloc(sizeof(int) * (n ? n : 1));
    int* prims = malloc(sizeof(int) * (n ? n : 1));
    for (int i = 0; i < n; i++) prims[i] = i;
    s->root = b_build(&B, prims, n, -1);
    free(prims);
    free(B.bmin); free(B.bmax); free(B.cen);
}

/* ---- Queries ---- */
typedef struct { v3 o, d; float max_t; } ray_t;

/* AABB::intersect_any, aabb.h:19-61, including its comparison order. */
static int box_hit(const float* bx, const ray_t* r) {
    v3 mn = V(bx[0], bx[1], bx[2]), mx = V(bx[3], bx[4], bx[5]);
    v3 dmin = vsub(mn, r->o), dmax = vsub(mx, r->o);
    float nminx = dmin.x / r->d.x, nminy = dmin.y / r->d.y, nminz = dmin.z / r->d.z;
    float nmaxx = dmax.x / r->d.x, nmaxy = dmax.y / r->d.y, nmaxz = dmax.z / r->d.z;
    float t;
    if (!(nmaxx >= nminx)) { t = nminx; nminx = nmaxx; nmaxx = t; } /* order2, math.h:699-705 */
    if (!(nmaxy >= nminy)) { t = nminy; nminy = nmaxy; nmaxy = t; }
    if (!(nmaxz >= nminz)) { t = nminz; nminz = nmaxz; nmaxz = t; }
    float tmin = nminx;
    if (tmin < nminy) tmin = nminy;
    if (tmin < nminz && nminz > nminy) tmin = nminz;
    float tmax = nmaxx;
    if (tmax > nmaxy) tmax = nmaxy;
    if (tmax > nmaxz && nmaxz < nmaxy) tmax = nmaxz;
    if (tmax < tmin) return 0;
    if (tmin > 0 && (double)tmin < (double)r->max_t + OR_EPS) return 1;
    if (tmax > 0) return 1;
    return 0;
}

typedef struct { float t, beta, gamma, alpha; } tri_hit;

/* Triangle::intersect / intersect_any up to the acceptance test,
 * triangle.h:18-80 and 117-179.  Returns 1 when the candidate is accepted. */
static int tri_test(const or_scene* s, int t, const ray_t* r, tri_hit* h) {
    v3 a = s->pos[s->tri[3 * t]], b = s->pos[s->tri[3 * t + 1]], c = s->pos[s->tri[3 * t + 2]];
    v3 v1 = vsub(b, a), v2 = vsub(c, a), v3_ = vneg(r->d), vs = vsub(r->o, a);
    float den = v1.x * v2.y * v3_.z + v2.x * v3_.y * v1.z + v3_.x * v1.y * v2.z - v3_.x * v2.y * v1.z -
                v3_.y * v2.z * v1.x - v3_.z * v2.x * v1.y;
    float inv = (float)(1.0 / (double)den);
    float tt = (v1.x * v2.y * vs.z + v2.x * vs.y * v1.z + vs.x * v1.y * v2.z - vs.x * v2.y * v1.z -
                vs.y * v2.z * v1.x - vs.z * v2.x * v1.y) * inv;
    if ((double)tt < OR_EPS || tt > r->max_t) return 0;
    float beta = (vs.x * v2.y * v3_.z + v2.x * v3_.y * vs.z + v3_.x * vs.y * v2.z - v3_.x * v2.y * vs.z -
                  v3_.y * v2.z * vs.x - v3_.z * v2.x * vs.y) * inv;
    float gamma = (v1.x * vs.y * v3_.z + vs.x * v3_.y * v1.z + v3_.x * v1.y * vs.z - v3_.x * vs.y * v1.z -
                   v3_.y * vs.z * v1.x - v3_.z * vs.x * v1.y) * inv;
    float alpha = (float)(1.0 - (double)(gamma + beta));
    if (alpha < 0 || alpha > 1 || beta < 0 || beta > 1 || gamma < 0 || gamma > 1) return 0;
    h->t = tt; h->beta = beta; h->gamma = gamma; h->alpha = alpha;
    return 1;
}

/* BVHNode::intersect (bvh.h:22-37) + SimpleGroup::intersect (simple_group.h:21-28):
 * exhaustive, member `right` (left partition) first; equal t: the later wins. */
static void closest_rec(const or_scene* s, int node, ray_t* r, int* best, tri_hit* bh) {
    if (node >= 0) {
        if (!box_hit(s->node_box + 6 * node, r)) return;
        closest_rec(s, s->node_child[2 * node], r, best, bh);
        closest_rec(s, s->node_child[2 * node + 1], r, best, bh);
    } else {
        int leaf = ~node;
        for (int k = 0; k < s->leaf_count[leaf]; k++) {
            int p = s->leaf_prims[s->leaf_start[leaf] + k];
            tri_hit h;
            if (tri_test(s, p, r, &h)) { r->max_t = h.t; *best = p; *bh = h; }
        }
    }
}

static int any_rec(const or_scene* s, int node, ray_t* r) {
    if (node >= 0) {
        if (!box_hit(s->node_box + 6 * node, r)) return 0;
        return any_rec(s, s->node_child[2 * node], r) || any_rec(s, s->node_child[2 * node + 1], r);
    }
    int leaf = ~node;
    for (int k = 0; k < s->leaf_count[leaf]; k++) {
        tri_hit h;
        if (tri_test(s, s->leaf_prims[s->leaf_start[leaf] + k], r, &h)) return 1;
    }
    return 0;
}

/* Culling traversal with the same answers (test infrastructure: it lets the
 * oracle render million-triangle scenes in seconds; the reference's
 * exhaustive recursion would take hours).  The reference's closest hit is
 * the smallest t among the triangles it tests -- those whose ancestor boxes
 * all pass box_hit -- and on equal t the one visited last, i.e. the larger
 * position in leaf_prims (leaves are numbered in the recursion's order).
 * A subtree whose entry distance (boxes inflated by fast_pad) exceeds the
 * best t so far by more than 2^-8 relative cannot hold a better candidate,
 * so skipping it, and visiting the nearer child first, changes nothing.
 * test_oracle_pins.py checks the two traversals against each other. */
#define OR_FAST_STACK 4096
static float box_entry(const float* bx, const ray_t* r, float pad) {
    float t0 = 0.0f;
    for (int k = 0; k < 3; k++) {
        float o = vget(r->o, k), d = vget(r->d, k);
        float a = (bx[k] - pad - o) / d, b = (bx[3 + k] + pad - o) / d; /* d == 0: +-inf or NaN */
        float near = fminf(a, b);                                      /* fminf drops a NaN */
        if (near > t0) t0 = near;
    }
    return t0;
}

static int closest_fast(const or_scene* s, ray_t* r, tri_hit* h) {
    int stack[OR_FAST_STACK];
    int sp = 0, best = -1, best_rank = -1;
    float best_t = INFINITY;
    const float slack = 1.0f + 1.0f / 256.0f;
    stack[sp++] = s->root;
    while (sp > 0) {
        int node = stack[--sp];
        if (node >= 0) {
            const float* bx = s->node_box + 6 * node;
            if (!box_hit(bx, r)) continue;
            if (best >= 0 && box_entry(bx, r, s->fast_pad) > best_t * slack) continue;
            int c0 = s->node_child[2 * node], c1 = s->node_child[2 * node + 1];
            float e0 = c0 >= 0 ? box_entry(s->node_box + 6 * c0, r, s->fast_pad) : 0.0f;
            float e1 = c1 >= 0 ? box_entry(s->node_box + 6 * c1, r, s->fast_pad) : 0.0f;
            if (sp + 2 > OR_FAST_STACK) { /* deeper than the stack: the exhaustive recursion */
                best = -1;
                closest_rec(s, s->root, r, &best, h);
                return best;
            }
            if (e0 <= e1) { stack[sp++] = c1; stack[sp++] = c0; }
            else { stack[sp++] = c0; stack[sp++] = c1; }
        } else {
            int leaf = ~node;
            for (int k = 0; k < s->leaf_count[leaf]; k++) {
                int rank = s->leaf_start[leaf] + k;
                int p = s->leaf_prims[rank];
                tri_hit th;
                if (!tri_test(s, p, r, &th)) continue;
                if (th.t < best_t || (th.t == best_t && rank > best_rank)) {
                    best_t = th.t; best_rank = rank; best = p; *h = th;
                }
            }
        }
    }
    if (best >= 0) r->max_t = best_t;
    return best;
}

static int any_fast(const or_scene* s, ray_t* r) {
    int stack[OR_FAST_STACK];
    int sp = 0;
    const float limit = r->max_t * (1.0f + 1.0f / 256.0f);
    stack[sp++] = s->root;
    while (sp > 0) {
        int node = stack[--sp];
        if (node >= 0) {
            const float* bx = s->node_box + 6 * node;
            if (!box_hit(bx, r)) continue;
            if (box_entry(bx, r, s->fast_pad) > limit) continue;
            if (sp + 2 > OR_FAST_STACK) return any_rec(s, s->root, r);
            stack[sp++] = s->node_child[2 * node + 1];
            stack[sp++] = s->node_child[2 * node];
        } else {
            int leaf = ~node;
            for (int k = 0; k < s->leaf_count[leaf]; k++) {
                tri_hit h;
                if (tri_test(s, s->leaf_prims[s->leaf_start[leaf] + k], r, &h)) return 1;
            }
        }
    }
    return 0;
}

static int closest(const or_scene* s, ray_t* r, tri_hit* h) {
    int best = -1;
    if (s->n_tris <= 0) return -1;
    if (s->fast) return closest_fast(s, r, h);
    closest_rec(s, s->root, r, &best, h);
    return best;
}

static int any_hit(const or_scene* s, ray_t* r) {
    if (s->n_tris <= 0) return 0;
    return s->fast ? any_fast(s, r) : any_rec(s, s->root, r);
}

/* ----------------------------------------------------------------------- */
/* Shading: Intersection + materials + BxDFs                                 */
/* ----------------------------------------------------------------------- */
typedef struct {
    v3 normal, g_normal, tangent, bitangent, hit;
    int prim;
    float u, v; /* texture coordinates (triangle.h:91-94) */
} isect;

/* ImageTexture::sample, bilinear branch (image_texture.h:24-41; the harness
 * pins the uninitialised filtering member to it), over Image::get_pixel with
 * the REPEAT border (rgb_image.h:210-250).  Vec3 images compute in float with
 * each (1.0 - x) rounded to float (Vector3<float>::operator*(float)); float
 * images sum in double (pixel * (1.0 - x) promotes) and round once. */
static int tex_wrap(int i, int n) {
    if (i >= n) return i % n;
    if (i < 0) return i % n + n;
    return i;
}
static const float* tex_px(const or_scene* s, int t, int i, int j) {
    const int* info = s->tex_info + 4 * t;
    int w = info[1], h = info[2];
    long idx = (long)tex_wrap(i, w) + (long)tex_wrap(j, h) * w;
    if (idx > (long)w * h - 1) idx = (long)w * h - 1; /* the reference reads past the image here */
    if (idx < 0) idx = 0;
    return s->tex_px + info[0] + idx * info[3];
}
static v3 tex_sample(const or_scene* s, int t, float u, float v) {
    const int* info = s->tex_info + 4 * t;
    float x = u * (float)info[1];
    float y = (float)((1.0 - (double)v) * (double)info[2]);
    x = (float)((double)x - 0.5);
    y = (float)((double)y - 0.5);
    int i = (int)floorf(x), j = (int)floorf(y);
    x = x - (float)i;
    y = y - (float)j;
    const float *p00 = tex_px(s, t, i, j), *p10 = tex_px(s, t, i + 1, j);
    const float *p01 = tex_px(s, t, i, j + 1), *p11 = tex_px(s, t, i + 1, j + 1);
    if (info[3] == 1) { /* pixel * (1.0 - x) is double, pixel * x a float product */
        double r = ((double)p00[0] * (1.0 - (double)x) + (double)(p10[0] * x)) * (1.0 - (double)y) +
                   ((double)p01[0] * (1.0 - (double)x) + (double)(p11[0] * x)) * (double)y;
        float f = (float)r;
        return V(f, f, f);
    }
    float omx = (float)(1.0 - (double)x), omy = (float)(1.0 - (double)y);
    v3 a = vadd(vscale(V(p00[0], p00[1], p00[2]), omx), vscale(V(p10[0], p10[1], p10[2]), x));
    v3 b = vadd(vscale(V(p01[0], p01[1], p01[2]), omx), vscale(V(p11[0], p11[1], p11[2]), x));
    return vadd(vscale(a, omy), vscale(b, y));
}
static int mat_tex(const or_scene* s, int m, int slot) { return s->mat_tex ? s->mat_tex[4 * m + slot] : -1; }

/* triangle.h:83-114 then Intersection::get_bxdf (intersection.h:25-33).
 * `first`: the Intersection object of PathtracerMIS::integrate is reused for
 * every bounce and its computed_normal flag is never reset, so the normal
 * mapping and re-orthogonalisation only happen at a path's first hit. */
static void fill_isect(const or_scene* s, int p, const ray_t* r, const tri_hit* h, int first, isect* it) {
    int i0 = s->tri[3 * p], i1 = s->tri[3 * p + 1], i2 = s->tri[3 * p + 2];
    v3 a = s->pos[i0], b = s->pos[i1], c = s->pos[i2];
    v3 normal = vnorm(vadd(vadd(vscale(s->nrm[i0], h->alpha), vscale(s->nrm[i1], h->beta)),
                           vscale(s->nrm[i2], h->gamma)));
    v3 bt = vnorm(vadd(vadd(vscale(s->btan[i0], h->alpha), vscale(s->btan[i1], h->beta)),
                       vscale(s->btan[i2], h->gamma)));
    it->normal = normal;
    it->g_normal = vnorm(vcross(vsub(b, a), vsub(c, a)));
    it->bitangent = bt;
    it->tangent = vnorm(vcross(bt, normal));
    it->hit = vadd(r->o, vscale(r->d, h->t));
    it->prim = p;
    it->u = it->v = 0.0f;
    if (s->uv) { /* triangle.h:91-94: uv1 * alpha + uv2 * beta + uv3 * gamma */
        it->u = s->uv[2 * i0] * h->alpha + s->uv[2 * i1] * h->beta + s->uv[2 * i2] * h->gamma;
        it->v = s->uv[2 * i0 + 1] * h->alpha + s->uv[2 * i1 + 1] * h->beta + s->uv[2 * i2 + 1] * h->gamma;
    }
    if (!first) return;
    /* get_normal_mapped: StandardMaterial maps the normal-map value through
     * Mat3(tangent, bitangent, normal) (standard_material.h:64-71), the
     * constant rgb(0.5,0.5,1) to (0,0,1); the emissive and dielectric
     * materials keep the normal. */
    int m = s->tri_mat[p], kind = s->mat_kind[m];
    if (kind == MAT_DIFFUSE || kind == MAT_GGX) {
        m3 M = mcols(it->tangent, it->bitangent, it->normal);
        v3 c = V(0.5f, 0.5f, 1.0f);
        int tn = mat_tex(s, m, 3);
        if (tn >= 0) c = tex_sample(s, tn, it->u, it->v);
        float nx = (float)((double)c.x * 2.0 - 1.0), ny = (float)((double)c.y * 2.0 - 1.0);
        it->normal = vnorm(mmul(&M, V(nx, ny, c.z)));
    }
    it->bitangent = vnorm(vcross(it->normal, it->tangent));
    it->tangent = vnorm(vcross(it->bitangent, it->normal));
}

/* BxDF::same_hemisphere, bxdf.h:42-45 */
static int same_hemisphere(const isect* it, v3 wo, v3 wi) {
    float sign = vdot(wo, it->g_normal);
    return sign * vdot(wi, it->normal) > 0.0 && sign * vdot(wi, it->g_normal) > 0.0;
}

/* math.h:647-653 */
static v3 sample_hemisphere_cos(float r1, float r2) {
    float theta = (float)((double)r1 * 2.0 * OR_PI);
    float sin_phi = sqrtf(r2);
    float cos_phi = (float)sqrt(1.0 - (double)(sin_phi * sin_phi));
    return V(cosf(theta) * sin_phi, sinf(theta) * sin_phi, cos_phi);
}

/* math.h:663-688 */
static void orthogonal(v3 v1, v3* x, v3* y, v3* z) {
    float ax = fabsf(v1.x), ay = fabsf(v1.y), az = fabsf(v1.z);
    v3 aux;
    if (ax < ay) aux = ax < az ? V(1, 0, 0) : V(0, 0, 1);
    else aux = ay < az ? V(0, 1, 0) : V(0, 0, 1);
    v3 aux2 = vcross(v1, aux);
    *x = vnorm(v1);
    *y = vnorm(vcross(aux2, v1));
    *z = vnorm(aux2);
}

/* math.h:712-742 */
static inline float cosT(v3 w) { return w.z; }
static inline float cos2T(v3 w) { return w.z * w.z; }
static inline float sinT(v3 w) { return (float)sqrt(1.0 - (double)cos2T(w)); }
static inline float cosP(v3 w) { float s = sinT(w); if ((double)s == 0.0) return 1.0f; return w.x / sinT(w); }
static inline float sinP(v3 w) { float s = sinT(w); if ((double)s == 0.0) return 1.0f; return w.y / sinT(w); }
static v3 reflect(v3 wo, v3 wh) {
    return vnorm(vadd(vneg(wo), vscale(vscale(wh, vdot(wh, wo)), (float)2.0)));
}

/* MicrofacetDistribution, microfacet_distribution.h:9-168 (isotropic use) */
static void md_sample11(float cosTheta, float U1, float U2, float* slope_x, float* slope_y) {
    if ((double)cosTheta > .9999) {
        float r = sqrtf(U1 / (1 - U1));
        float phi = (float)(6.28318530718 * (double)U2);
        *slope_x = r * cosf(phi);
        *slope_y = r * sinf(phi);
        return;
    }
    float sinTheta = sqrtf(fmaxf(0.0f, 1.0f - cosTheta * cosTheta));
    float tanTheta = sinTheta / cosTheta;
    float a = (float)(1. / (double)tanTheta);
    float G1 = (float)(2. / (double)(1 + sqrtf(1.f + 1.f / (a * a))));
    float A = 2 * U1 / G1 - 1;
    float tmp = 1.f / (A * A - 1.f);
    if ((double)tmp > 1e10) tmp = (float)1e10;
    float B = tanTheta;
    float Dv = sqrtf(fmaxf(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.0f));
    float s1 = B * tmp - Dv, s2 = B * tmp + Dv;
    *slope_x = (A < 0 || s2 > 1.f / tanTheta) ? s1 : s2;
    float S;
    if (U2 > 0.5f) { S = 1.f; U2 = 2.f * (U2 - .5f); }
    else { S = -1.f; U2 = 2.f * (.5f - U2); }
    float z = (U2 * (U2 * (U2 * 0.27385f - 0.73369f) + 0.46341f)) /
              (U2 * (U2 * (U2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
    *slope_y = S * z * sqrtf(1.f + *slope_x * *slope_x);
    if (isinf(*slope_y) || isnan(*slope_y)) *slope_y = 0.0f;
}

static v3 md_sample(float alpha, v3 wi, float U1, float U2) {
    v3 ws = vnorm(V(alpha * wi.x, alpha * wi.y, wi.z));
    float sx, sy;
    md_sample11(cosT(ws), U1, U2, &sx, &sy);
    float tmp = cosP(ws) * sx - sinP(ws) * sy;
    sy = sinP(ws) * sx + cosP(ws) * sy;
    sx = tmp;
    sx = alpha * sx;
    sy = alpha * sy;
    return vnorm(V(-sx, -sy, 1.0f));
}

static float md_d(float alpha, v3 wh) {
    float tan2 = sinT(wh) / cosT(wh);
    tan2 = tan2 * tan2;
    if (isinf(tan2)) return 0.0f;
    float cos4 = cos2T(wh) * cos2T(wh);
    float e = (cosP(wh) * cosP(wh) / (alpha * alpha) + sinP(wh) * sinP(wh) / (alpha * alpha)) * tan2;
    return (float)(1.0 / (OR_PI * alpha * alpha * cos4 * (1 + e) * (1 + e)));
}

/* note: |cos/sin| as written at microfacet_distribution.h:138 */
static float md_lambda(float alpha, v3 w) {
    float absTan = fabsf(cosT(w) / sinT(w));
    if (isinf(absTan)) return 0.0f;
    float al = sqrtf(cosP(w) * cosP(w) * alpha * alpha + sinP(w) * sinP(w) * alpha * alpha);
    float a2t2 = (al * absTan) * (al * absTan);
    return (float)((-1.0 + sqrt(1.0 + (double)a2t2)) / 2.0);
}
static float md_g(float alpha, v3 wo, v3 wi) {
    return (float)(1.0 / (1.0 + (double)md_lambda(alpha, wo) + (double)md_lambda(alpha, wi)));
}
static float md_g1(float alpha, v3 w) { return (float)(1.0 / (1.0 + (double)md_lambda(alpha, w))); }
static float md_pdf(float alpha, v3 wo, v3 wh) {
    float ad = md_d(alpha, wh), ag1 = md_g1(alpha, wo);
    float adot = fabsf(vdot(wo, wh)), aother = fabsf(cosT(wo));
    return ad * ag1 * adot / aother;
}

typedef struct { v3 wi; float pdf; int delta; } dsample;

typedef struct {
    int kind;
    v3 col;       /* albedo / emission (albedo * intensity) */
    float alpha;  /* GGX */
    int delta;    /* GGX with roughness < 0.01 */
    float ior;
} bsdf_t;

/* Material::get_bxdf at texture coordinates (u, v): StandardMaterial
 * (standard_material.h:46-61: Diffuse(albedo) when metal < 0.1, else
 * Glossy(roughness)), EmissiveMaterial (emissive_material.h:28-30: colour x
 * intensity), from constants or image textures. */
static bsdf_t make_bsdf(const or_scene* s, int prim, float u, float v) {
    int m = s->tri_mat[prim];
    const float* p = s->mat_params + 8 * m;
    bsdf_t b;
    memset(&b, 0, sizeof(b));
    b.kind = s->mat_kind[m];
    int ta = mat_tex(s, m, 0), tr = mat_tex(s, m, 1), tm = mat_tex(s, m, 2);
    if (b.kind == MAT_EMISSIVE) {
        if (ta >= 0) b.col = vscale(tex_sample(s, ta, u, v), s->mat_emit[m]);
        else b.col = vscale(V(p[0], p[1], p[2]), p[5]);
    } else {
        b.col = ta >= 0 ? tex_sample(s, ta, u, v) : V(p[0], p[1], p[2]);
        if (tm >= 0) b.kind = (double)tex_sample(s, tm, u, v).x < 0.1 ? MAT_DIFFUSE : MAT_GGX;
    }
    if (b.kind == MAT_GGX) {
        float r = tr >= 0 ? tex_sample(s, tr, u, v).x : p[3];
        float a2 = r * r;
        b.alpha = a2 > 0.01f ? a2 : 0.01f; /* std::max(r*r, 0.01f) */
        b.delta = (double)r < 0.01;
    }
    b.ior = p[4];
    return b;
}

static v3 bsdf_eval(const bsdf_t* b, v3 wo, v3 wi, const isect* it) {
    if (b->kind == MAT_DIFFUSE) /* diffuse_bxdf.h:25-27 */
        return vdivs(vscale(b->col, fabsf(vdot(it->normal, wi))), (float)OR_PI);
    if (b->kind == MAT_GGX) { /* glossy_bxdf.h:23-33 */
        m3 M = mcols(it->tangent, it->bitangent, it->normal);
        m3 Mt = mtranspose(&M);
        v3 wol = vnorm(mmul(&Mt, wo)), wil = vnorm(mmul(&Mt, wi));
        v3 wh = vnorm(vadd(wol, wil));
        float v = (float)((double)(md_g(b->alpha, wol, wil) * md_d(b->alpha, wh)) /
                          (4.0 * (double)vdot(wo, it->normal)));
        return V(v, v, v);
    }
    if (b->kind == MAT_DIELECTRIC) return V(1, 1, 1);
    return V(0, 0, 0);
}

static float bsdf_pdf(const bsdf_t* b, v3 wo, v3 wi, const isect* it) {
    if (b->kind == MAT_DIFFUSE) return (float)((double)fabsf(vdot(it->normal, wi)) / OR_PI);
    if (b->kind == MAT_GGX) { /* glossy_bxdf.h:55-72 */
        m3 M = mcols(it->tangent, it->bitangent, it->normal);
        m3 Mt = mtranspose(&M);
        v3 wol = vnorm(mmul(&Mt, wo));
        v3 wh = vnorm(mmul(&Mt, vadd(wo, wi)));
        return (float)((double)md_pdf(b->alpha, wol, wh) / (4.0 * (double)fabsf(vdot(wol, wh))));
    }
    return 1.0f;
}

/* BxDF::sample on the two uniform numbers it draws (Lambert: r1, r2 of
 * sample_hemisphere_cos; GGX: U1, U2 of MicrofacetDistribution::sample; the
 * delta GGX and the dielectric draw none). */
static dsample bsdf_sample_u(const bsdf_t* b, float r1, float r2, v3 wo, const isect* it) {
    dsample d;
    if (b->kind == MAT_DIFFUSE) { /* diffuse_bxdf.h:28-41 */
        v3 sm = sample_hemisphere_cos(r1, r2);
        float p = (float)((double)sm.z / OR_PI);
        v3 n = it->normal;
        if ((double)vdot(n, wo) < 0.0) n = vneg(n); /* correct_normal, bxdf.h:52-57 */
        v3 x, y, z;
        orthogonal(n, &x, &y, &z);
        m3 C = mcols(y, z, x);
        d.wi = mmul(&C, sm);
        d.pdf = p;
        d.delta = 0;
        return d;
    }
    if (b->kind == MAT_GGX) { /* glossy_bxdf.h:34-46 */
        if (b->delta) { d.wi = reflect(wo, it->normal); d.pdf = 1.0f; d.delta = 1; return d; }
        m3 M = mcols(it->tangent, it->bitangent, it->normal);
        m3 Mt = mtranspose(&M);
        v3 wol = vnorm(mmul(&Mt, wo));
        v3 whl = vnorm(md_sample(b->alpha, wol, r1, r2));
        v3 wh = vnorm(mmul(&M, whl));
        d.wi = reflect(wo, wh);
        d.pdf = bsdf_pdf(b, wo, d.wi, it);
        d.delta = 0;
        return d;
    }
    /* RefractionBxDF::sample, refraction_bxdf.h:26-52 */
    v3 n = it->normal;
    float n2 = (float)(1.0 / (double)b->ior);
    if ((double)vdot(n, wo) < 0.0) { n2 = (float)(1.0 / (double)n2); n = vneg(n); }
    float ci = vdot(wo, n);
    float ct2 = (float)(1.0 - (double)(n2 * n2) * (1.0 - (double)(ci * ci)));
    v3 r = vnorm(vadd(vscale(vneg(wo), n2), vscale(n, n2 * ci - sqrtf(ct2))));
    if (ct2 < 0) r = vnorm(vadd(vneg(wo), vscale(vscale(it->normal, vdot(it->normal, wo)), (float)2.0)));
    d.wi = r; d.pdf = 1.0f; d.delta = 1;
    return d;
}

static dsample bsdf_sample(const bsdf_t* b, mt19937* g, v3 wo, const isect* it) {
    float r1 = 0.0f, r2 = 0.0f;
    if (b->kind == MAT_DIFFUSE || (b->kind == MAT_GGX && !b->delta)) {
        r1 = mt_float(g);
        r2 = mt_float(g);
    }
    return bsdf_sample_u(b, r1, r2, wo, it);
}

/* Triangle::sample (triangle.h:209-269): position and interpolated normal */
static void tri_sample(const or_scene* s, int p, float r1, float r2, v3* pos, v3* normal, float* u, float* v) {
    float al = r1, be = r2;
    if ((double)(al + be) > 1.0) { al = (float)(1.0 - (double)al); be = (float)(1.0 - (double)be); }
    float ga = (float)(1.0 - (double)al - (double)be);
    int i0 = s->tri[3 * p], i1 = s->tri[3 * p + 1], i2 = s->tri[3 * p + 2];
    *pos = vadd(vadd(vscale(s->pos[i0], al), vscale(s->pos[i1], be)), vscale(s->pos[i2], ga));
    *normal = vnorm(vadd(vadd(vscale(s->nrm[i0], al), vscale(s->nrm[i1], be)), vscale(s->nrm[i2], ga)));
    *u = *v = 0.0f;
    if (s->uv) { /* triangle.h:244-249: uv1 * alpha + uv2 * beta + uv2 * gamma (the second vertex twice) */
        *u = s->uv[2 * i0] * al + s->uv[2 * i1] * be + s->uv[2 * i1] * ga;
        *v = s->uv[2 * i0 + 1] * al + s->uv[2 * i1 + 1] * be + s->uv[2 * i1 + 1] * ga;
    }
}

static float tri_area(const or_scene* s, int p) { /* triangle.h:197-207 */
    v3 a = s->pos[s->tri[3 * p]], b = s->pos[s->tri[3 * p + 1]], c = s->pos[s->tri[3 * p + 2]];
    return (float)((double)vlen(vcross(vsub(b, a), vsub(c, a))) * 0.5);
}

typedef struct { float pdf; v3 position, intensity, normal; } light_sample;

/* LightGroup::connect_eye_path (light_group.h:25-30) + ShapeLight (shape_light.h:24-44) */
static light_sample light_connect_u(const or_scene* s, float u0, float r1, float r2, const isect* from) {
    size_t n = (size_t)s->n_lights;
    int k = (int)((size_t)(int)(u0 * (float)n) % n);
    int p = s->light_tri[k];
    light_sample ls;
    v3 normal;
    float su, sv;
    tri_sample(s, p, r1, r2, &ls.position, &normal, &su, &sv);
    bsdf_t e = make_bsdf(s, p, su, sv);
    v3 dir = vnorm(vsub(from->hit, ls.position));
    ls.intensity = vscale(e.col, fabsf(vdot(normal, dir)));
    ls.pdf = (float)(1.0 / (double)tri_area(s, p));
    ls.normal = normal;
    ls.pdf = (float)((double)ls.pdf * (1.0 / (double)(float)n));
    return ls;
}

/* draws the light index, then the triangle's two numbers (triangle.h:209-215) */
static light_sample light_connect(const or_scene* s, mt19937* g, const isect* from) {
    float u0 = mt_float(g);
    float r1 = mt_float(g);
    float r2 = mt_float(g);
    return light_connect_u(s, u0, r1, r2, from);
}

static float light_pdf(const or_scene* s, int prim) { /* light_group.h:43-55 */
    float pdf = (float)(1.0 / (double)(float)s->n_lights);
    pdf *= (float)(1.0 / (double)tri_area(s, prim));
    return pdf;
}

static ray_t camera_ray(const or_scene* s, float cx, float cy) { /* camera_perspective.h:30-39 */
    v3 d;
    d.z = -1.0f;
    d.y = cy * s->tan_fovy;
    d.x = cx * s->tan_fovy * s->aspect;
    ray_t r;
    r.o = s->cam_origin;
    r.d = vnorm(mmul(&s->cam_coords, d));
    r.max_t = INFINITY;
    return r;
}

/* PathtracerMIS::integrate, pathtracerMIS.h:29-131 */
/* integrator 0: PathtracerMIS::integrate (pathtracerMIS.h:29-131);
 * 1: Pathtracer::integrate, NEE without MIS (pathtracer.h:27-102): emitters
 *    count only after the camera or a delta bounce, NEE at full weight;
 * 2: PurePt::integrate (pure_pt.h:28-71): no NEE, every emitter hit counts.
 * The random numbers are drawn in the same order as each reference method. */
static v3 integrate(const or_scene* s, float cx, float cy, mt19937* g, int max_depth, int integrator) {
    ray_t ray = camera_ray(s, cx, cy);
    v3 col = V(0, 0, 0), mul = V(1, 1, 1);
    int sampled_delta = 1;
    float p = 1.0f;
    for (int i = 0; i < max_depth; i++) {
        tri_hit h;
        int prim = closest(s, &ray, &h);
        if (prim < 0) { col = vadd(col, vmul(mul, V(0, 0, 0))); break; }
        ray.max_t = h.t;
        isect it;
        fill_isect(s, prim, &ray, &h, i == 0, &it);
        bsdf_t b = make_bsdf(s, prim, it.u, it.v);
        v3 wo = vneg(ray.d);
        if (b.kind == MAT_EMISSIVE) {
            if (sampled_delta || integrator == 2) {
                col = vadd(col, vmul(mul, b.col));
            } else if (integrator == 0) {
                float r = ray.max_t;
                float cos_theta = (float)((double)fabsf(vdot(it.normal, ray.d)) + OR_EPS);
                float p_nee = light_pdf(s, prim) * r * r / cos_theta;
                float w = p / (p + p_nee);
                col = vadd(col, vscale(vmul(mul, b.col), w));
            }
            break;
        }
        sampled_delta = 0;
        dsample smp = bsdf_sample(&b, g, wo, &it);
        v3 wi = smp.wi;
        p = smp.pdf;
        if (integrator == 2) {
            /* pure PT: no light sample */
        } else if (!smp.delta) {
            light_sample ls = light_connect(s, g, &it);
            v3 sd = vsub(ls.position, it.hit);
            float len = vlen(sd);
            sd = vdivs(sd, len);
            ray_t sh;
            sh.o = vadd(it.hit, vscale(sd, (float)OR_EPS));
            sh.d = sd;
            sh.max_t = (float)((double)len - 2.0 * OR_EPS);
            if (same_hemisphere(&it, wo, sh.d)) {
                if (!any_hit(s, &sh)) {
                    float r = len;
                    v3 ev = bsdf_eval(&b, wo, sh.d, &it);
                    v3 c = vdivs(vmul(vmul(mul, ev), ls.intensity), ls.pdf * r * r);
                    if (integrator == 0) {
                        float p_bsdf = bsdf_pdf(&b, wo, sd, &it);
                        float cos_l = (float)((double)fabsf(vdot(ls.normal, sd)) + OR_EPS);
                        float p_nee = ls.pdf * r * r / cos_l;
                        float w = p_nee / (p_bsdf + p_nee);
                        c = vscale(c, w);
                    }
                    col = vadd(col, c);
                }
            }
        } else {
            sampled_delta = 1;
        }
        if (!same_hemisphere(&it, wo, wi)) break;
        v3 ev = bsdf_eval(&b, wo, wi, &it);
        if (i > 2) {
            float rr = (float)(fabs((double)ev.x * 0.2 + (double)ev.y * 0.5 + (double)ev.z * 0.3) * 0.5 + 0.4);
            if (mt_float(g) > rr) break;
            p = p * rr;
        }
        mul = vdivs(vmul(mul, ev), p);
        ray.o = vadd(it.hit, vscale(wi, (float)OR_EPS));
        ray.d = wi;
        ray.max_t = INFINITY;
    }
    return col;
}

/* ----------------------------------------------------------------------- */
/* C API (ctypes)                                                            */
/* ----------------------------------------------------------------------- */
void* or_scene_create(int n_meshes, const int* mesh_vert_offset, const int* mesh_tri_offset,
                      const int* mesh_material, const float* vertices, const float* normals,
                      const float* tangents, const int* triangles, int n_materials, const int* mat_kind,
                      const float* mat_params, const float* camera, int width, int height) {
    or_scene* s = calloc(1, sizeof(or_scene));
    int nv = mesh_vert_offset[n_meshes], nt = mesh_tri_offset[n_meshes];
    s->n_verts = nv;
    s->n_tris = nt;
    s->pos = malloc(sizeof(v3) * (nv ? nv : 1));
    s->nrm = malloc(sizeof(v3) * (nv ? nv : 1));
    s->btan = malloc(sizeof(v3) * (nv ? nv : 1));
    for (int v = 0; v < nv; v++) {
        s->pos[v] = V(vertices[3 * v], vertices[3 * v + 1], vertices[3 * v + 2]);
        s->nrm[v] = V(normals[3 * v], normals[3 * v + 1], normals[3 * v + 2]);
        s->btan[v] = vcross(s->nrm[v], V(tangents[3 * v], tangents[3 * v + 1], tangents[3 * v + 2]));
    }
    s->tri = malloc(sizeof(int) * 3 * (nt ? nt : 1));
    memcpy(s->tri, triangles, sizeof(int) * 3 * nt);
    s->tri_mat = malloc(sizeof(int) * (nt ? nt : 1));
    for (int m = 0; m < n_meshes; m++)
        for (int f = mesh_tri_offset[m]; f < mesh_tri_offset[m + 1]; f++) s->tri_mat[f] = mesh_material[m];
    s->n_mats = n_materials;
    s->mat_kind = malloc(sizeof(int) * (n_materials ? n_materials : 1));
    memcpy(s->mat_kind, mat_kind, sizeof(int) * n_materials);
    s->mat_params = malloc(sizeof(float) * 8 * (n_materials ? n_materials : 1));
    memcpy(s->mat_params, mat_params, sizeof(float) * 8 * n_materials);
    s->tri_light = malloc(sizeof(int) * (nt ? nt : 1));
    s->light_tri = malloc(sizeof(int) * (nt ? nt : 1));
    for (int t = 0; t < nt; t++) {
        s->tri_light[t] = -1;
        if (s->mat_kind[s->tri_mat[t]] == MAT_EMISSIVE) { s->tri_light[t] = s->n_lights; s->light_tri[s->n_lights++] = t; }
    }
    v3 o = V(camera[0], camera[1], camera[2]), at = V(camera[3], camera[4], camera[5]);
    v3 up = V(camera[6], camera[7], camera[8]);
    v3 fwd = vnorm(vsub(at, o));
    v3 z = vnorm(vneg(fwd)), x = vnorm(vcross(up, z)), y = vnorm(vcross(z, x));
    s->cam_origin = o;
    s->cam_coords = mcols(x, y, z);
    s->tan_fovy = camera[9];
    s->aspect = (float)width / (float)height;
    s->width = width;
    s->height = height;
    s->root = 0x7fffffff;
    if (nt > 0) bvh_build(s);
    float ext = 0.0f;
    for (int v = 0; v < nv; v++) {
        float m = fmaxf(fabsf(s->pos[v].x), fmaxf(fabsf(s->pos[v].y), fabsf(s->pos[v].z)));
        if (m > ext) ext = m;
    }
    s->fast_pad = 1e-5f * (2.0f * ext + 1.0f);
    return s;
}

/* Switches the scene's queries between the reference's exhaustive recursion
 * (0, the default) and the culling traversal with the same answers (1). */
void or_scene_set_fast(void* h, int fast) { ((or_scene*)h)->fast = fast; }

/* Image textures of a scene read from the reference's files: uv (2 per
 * vertex), n_tex textures ({first float, width, height, channels} each,
 * pixels as the reference's Image<Vec3> / Image<float> holds them, n_px
 * floats in all), per material four texture indices (albedo or emission
 * colour, roughness, metal, normal map; -1: constant) and the intensity of
 * a textured emitter. */
void or_scene_set_textures(void* h, const float* uv, int n_tex, const int* tex_info, const float* tex_px, long n_px,
                           const int* mat_tex, const float* mat_emit) {
    or_scene* s = (or_scene*)h;
    s->uv = malloc(sizeof(float) * 2 * (s->n_verts ? s->n_verts : 1));
    memcpy(s->uv, uv, sizeof(float) * 2 * s->n_verts);
    s->n_tex = n_tex;
    s->tex_info = malloc(sizeof(int) * 4 * (n_tex ? n_tex : 1));
    memcpy(s->tex_info, tex_info, sizeof(int) * 4 * n_tex);
    s->tex_px = malloc(sizeof(float) * (n_px ? n_px : 1));
    memcpy(s->tex_px, tex_px, sizeof(float) * n_px);
    s->mat_tex = malloc(sizeof(int) * 4 * (s->n_mats ? s->n_mats : 1));
    memcpy(s->mat_tex, mat_tex, sizeof(int) * 4 * s->n_mats);
    s->mat_emit = malloc(sizeof(float) * (s->n_mats ? s->n_mats : 1));
    memcpy(s->mat_emit, mat_emit, sizeof(float) * s->n_mats);
}

void or_scene_destroy(void* h) {
    or_scene* s = h;
    if (!s) return;
    free(s->pos); free(s->nrm); free(s->btan); free(s->tri); free(s->tri_mat);
    free(s->mat_kind); free(s->mat_params); free(s->tri_light); free(s->light_tri);
    free(s->uv); free(s->tex_info); free(s->tex_px); free(s->mat_tex); free(s->mat_emit);
    free(s->node_box); free(s->node_child); free(s->node_parent);
    free(s->leaf_start); free(s->leaf_count); free(s->leaf_prims); free(s->prim_parent);
    free(s);
}

/* Same layout as ref_bvh_dump in ref_harness.cpp. */
int or_bvh_dump(void* h, int* leaf_order, float* node_boxes, int* node_parent, int* prim_parent,
                int max_nodes) {
    or_scene* s = h;
    for (int i = 0; i < s->n_tris; i++) { leaf_order[i] = s->leaf_prims[i]; prim_parent[i] = s->prim_parent[i]; }
    for (int i = 0; i < s->n_nodes && i < max_nodes; i++) {
        memcpy(node_boxes + 6 * i, s->node_box + 6 * i, sizeof(float) * 6);
        node_parent[i] = s->node_parent[i];
    }
    return s->n_nodes;
}

void or_trace_closest(void* h, const float* rays, int n, int* out_index, float* out_t) {
    const or_scene* s = h;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        const float* q = rays + 7 * i;
        ray_t r = {V(q[0], q[1], q[2]), V(q[3], q[4], q[5]), q[6]};
        tri_hit hh;
        int p = closest(s, &r, &hh);
        out_index[i] = p;
        out_t[i] = r.max_t;
    }
}

void or_trace_any(void* h, const float* rays, int n, unsigned char* out_hit) {
    const or_scene* s = h;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        const float* q = rays + 7 * i;
        ray_t r = {V(q[0], q[1], q[2]), V(q[3], q[4], q[5]), q[6]};
        out_hit[i] = (unsigned char)any_hit(s, &r);
    }
}

/* PathtracerMIS::render (pathtracerMIS.h:135-167): column i uses
 * RandomSampler(i + seed_offset); spp_axis^2 stratified samples per pixel.
 * When x0/x1 restrict the columns, only those columns are written. */
static void render_cols(void* h, int spp_axis, int max_depth, int seed_offset, int x0, int x1, int integrator,
                        float* rgb_out) {
    const or_scene* s = h;
    int W = s->width, H = s->height;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = x0; i < x1; i++) {
        mt19937 g;
        mt_seed(&g, (uint32_t)(i + seed_offset));
        for (int j = 0; j < H; j++) {
            v3 acc = V(0, 0, 0);
            for (int k = 0; k < spp_axis; k++)
                for (int l = 0; l < spp_axis; l++) {
                    float r1 = mt_float(&g), r2 = mt_float(&g);
                    float cx = (float)((double)(((float)i + (float)((float)k + r1) / (float)spp_axis) / (float)W) * 2.0 - 1.0);
                    float cy = (float)-((double)(((float)j + (float)((float)l + r2) / (float)spp_axis) / (float)H) * 2.0 - 1.0);
                    acc = vadd(acc, integrate(s, cx, cy, &g, max_depth, integrator));
                }
            acc = vdivs(acc, (float)(spp_axis * spp_axis));
            float* o = rgb_out + 3 * (i + j * W);
            o[0] = acc.x; o[1] = acc.y; o[2] = acc.z;
        }
    }
}

void or_render_mis_cols(void* h, int spp_axis, int max_depth, int seed_offset, int x0, int x1,
                        float* rgb_out) {
    render_cols(h, spp_axis, max_depth, seed_offset, x0, x1, 0, rgb_out);
}

void or_render_mis(void* h, int spp_axis, int max_depth, int seed_offset, float* rgb_out) {
    render_cols(h, spp_axis, max_depth, seed_offset, 0, ((or_scene*)h)->width, 0, rgb_out);
}

/* Pathtracer::render (integrator 1) / PurePt::render (integrator 2): the
 * same column seeding and stratification as PathtracerMIS::render. */
void or_render_variant(void* h, int integrator, int spp_axis, int max_depth, int seed_offset, float* rgb_out) {
    render_cols(h, spp_axis, max_depth, seed_offset, 0, ((or_scene*)h)->width, integrator, rgb_out);
}

/* ---- single-vertex BSDF / light primitives for kernel unit tests ----- */
/* Shading frame from a normal and a tangent as triangle.h + get_bxdf build it
 * for a flat triangle: out = {normal, g_normal, tangent, bitangent} */
static void frame_from(const float* n, const float* t, int kind, isect* it) {
    v3 N = vnorm(V(n[0], n[1], n[2]));
    v3 Tn = V(t[0], t[1], t[2]);
    v3 bt = vnorm(vcross(N, Tn));
    it->normal = N;
    it->g_normal = N;
    it->bitangent = bt;
    it->tangent = vnorm(vcross(bt, N));
    it->hit = V(0, 0, 0);
    if (kind == MAT_DIFFUSE || kind == MAT_GGX) {
        m3 M = mcols(it->tangent, it->bitangent, it->normal);
        it->normal = vnorm(mmul(&M, V(0.0f, 0.0f, 1.0f)));
    }
    it->bitangent = vnorm(vcross(it->normal, it->tangent));
    it->tangent = vnorm(vcross(it->bitangent, it->normal));
}

/* Evaluates eval(wo,wi) (3 floats), pdf(wo,wi) and non_zero for n cases.
 * params: kind, r, g, b, roughness, ior per case (6 floats; kind as float). */
void or_bsdf_eval(int n, const float* params, const float* normal, const float* tangent, const float* wo,
                  const float* wi, float* out_eval, float* out_pdf, int* out_nonzero) {
    for (int i = 0; i < n; i++) {
        const float* pp = params + 6 * i;
        int kind = (int)pp[0];
        isect it;
        frame_from(normal + 3 * i, tangent + 3 * i, kind, &it);
        float mp[8] = {pp[1], pp[2], pp[3], pp[4], pp[5], 1.0f, 0, 0};
        or_scene fake;
        memset(&fake, 0, sizeof(fake));
        int tm = 0;
        fake.tri_mat = &tm;
        fake.mat_kind = &kind;
        fake.mat_params = mp;
        bsdf_t b = make_bsdf(&fake, 0, 0.0f, 0.0f);
        v3 o = V(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), w = V(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        v3 e = bsdf_eval(&b, o, w, &it);
        out_eval[3 * i] = e.x; out_eval[3 * i + 1] = e.y; out_eval[3 * i + 2] = e.z;
        out_pdf[i] = (kind == MAT_DIELECTRIC) ? 1.0f : bsdf_pdf(&b, o, w, &it);
        out_nonzero[i] = same_hemisphere(&it, o, w);
    }
}

/* BxDF::sample for n cases on given uniform numbers u (2 per case): out_wi
 * (3 floats), out_pdf and out_delta.  Same case layout as or_bsdf_eval. */
void or_bsdf_sample(int n, const float* params, const float* normal, const float* tangent, const float* wo,
                    const float* u, float* out_wi, float* out_pdf, int* out_delta) {
    for (int i = 0; i < n; i++) {
        const float* pp = params + 6 * i;
        int kind = (int)pp[0];
        isect it;
        frame_from(normal + 3 * i, tangent + 3 * i, kind, &it);
        float mp[8] = {pp[1], pp[2], pp[3], pp[4], pp[5], 1.0f, 0, 0};
        or_scene fake;
        memset(&fake, 0, sizeof(fake));
        int tm = 0;
        fake.tri_mat = &tm;
        fake.mat_kind = &kind;
        fake.mat_params = mp;
        bsdf_t b = make_bsdf(&fake, 0, 0.0f, 0.0f);
        v3 o = V(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        dsample d = bsdf_sample_u(&b, u[2 * i], u[2 * i + 1], o, &it);
        out_wi[3 * i] = d.wi.x; out_wi[3 * i + 1] = d.wi.y; out_wi[3 * i + 2] = d.wi.z;
        out_pdf[i] = d.pdf;
        out_delta[i] = d.delta;
    }
}

/* LightGroup::connect_eye_path from n points on the scene's lights: in = 6
 * floats per case (from xyz, u0, u1, u2), out = 10 floats (position, normal,
 * intensity = Le |n_l . w|, pdf). */
void or_light_sample(void* h, int n, const float* in, float* out) {
    const or_scene* s = (const or_scene*)h;
    for (int i = 0; i < n; i++) {
        const float* c = in + 6 * i;
        isect it;
        memset(&it, 0, sizeof(it));
        it.hit = V(c[0], c[1], c[2]);
        light_sample ls = light_connect_u(s, c[3], c[4], c[5], &it);
        float* o = out + 10 * i;
        o[0] = ls.position.x; o[1] = ls.position.y; o[2] = ls.position.z;
        o[3] = ls.normal.x; o[4] = ls.normal.y; o[5] = ls.normal.z;
        o[6] = ls.intensity.x; o[7] = ls.intensity.y; o[8] = ls.intensity.z;
        o[9] = ls.pdf;
    }
}
