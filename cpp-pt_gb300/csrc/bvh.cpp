// Host BVH builders (see bvh.h).  Compiled with -ffp-contract=off: the
// reference-topology build must round every float step exactly as the
// reference's x86-64 build does.
#include "bvh.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <thread>

namespace cpppt_gb300 {
namespace {

constexpr float kInf = std::numeric_limits<float>::infinity();

struct V3 {
    float x, y, z;
    float operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};
inline V3 vmin(V3 a, V3 b) { return {a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z}; }
inline V3 vmax(V3 a, V3 b) { return {a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z}; }

struct AB {
    V3 lo{kInf, kInf, kInf}, hi{-kInf, -kInf, -kInf};
    void unite(const AB& o) { lo = vmin(lo, o.lo); hi = vmax(hi, o.hi); }
    void unite(V3 p) { lo = vmin(lo, p); hi = vmax(hi, p); }
    // AABB::area (aabb.h:77-82): float products and sums, doubled in double
    float ref_area() const {
        float s = std::fabs(hi.x - lo.x) * (hi.y - lo.y) + std::fabs(hi.z - lo.z) * (hi.y - lo.y) +
                  std::fabs(hi.x - lo.x) * (hi.z - lo.z);
        return (float)(2.0 * (double)s);
    }
    float sah_area() const {
        float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
        return dx * dy + dy * dz + dz * dx;
    }
};

void tri_box(const float* v, AB* b) {
    V3 a{v[0], v[1], v[2]}, bb{v[3], v[4], v[5]}, c{v[6], v[7], v[8]};
    // Triangle::get_bounds (triangle.h:197-207)
    b->lo = vmin(vmin(a, bb), c);
    b->hi = vmax(vmax(a, bb), c);
}

// ---------------------------------------------------------------------------
// Reference topology (bvh.h:57-216).
// ---------------------------------------------------------------------------
// A subtree of the reference topology built on its own: node ids are local
// (pre-order from 0); -1 as a parent means the subtree's parent outside it.
struct RefFrag {
    std::vector<Box3> node_box;
    std::vector<int32_t> node_parent;
    std::vector<int32_t> leaf_order;   // primitives in DFS order
    std::vector<int32_t> leaf_parent;  // per entry of leaf_order
};

// Appends fragment c as the next child subtree of node `id` of f (pre-order
// keeps: the parent, then its left subtree, then its right subtree).
void append_frag(RefFrag& f, const RefFrag& c, int32_t id) {
    const int32_t off = (int32_t)f.node_box.size();
    f.node_box.insert(f.node_box.end(), c.node_box.begin(), c.node_box.end());
    for (int32_t p : c.node_parent) f.node_parent.push_back(p < 0 ? id : p + off);
    f.leaf_order.insert(f.leaf_order.end(), c.leaf_order.begin(), c.leaf_order.end());
    for (int32_t p : c.leaf_parent) f.leaf_parent.push_back(p < 0 ? id : p + off);
}

constexpr int kRefParallelMin = 16384;   // subtrees below this size are built by the thread that reaches them
constexpr int kRefChunkMin = 1 << 18;     // nodes of at least this many primitives bin and partition in chunks

// f(chunk, begin, end) over [0, n) in T contiguous chunks, chunk 0 on the caller.
template <class F>
void par_chunks(int T, int n, F f) {
    std::vector<std::thread> th;
    for (int c = 1; c < T; c++) th.emplace_back(f, c, (int)((long long)n * c / T), (int)((long long)n * (c + 1) / T));
    f(0, 0, (int)((long long)n / T));
    for (std::thread& t : th) t.join();
}

// A primitive as the reference-topology build reads it: bounds, centroid,
// insertion index (moved as a whole by each partition).
struct PrimRec {
    AB b;
    V3 c;
    int32_t id;
};

struct RefBuilder {
    std::vector<PrimRec> tmp;
    std::vector<uint8_t> bin_of;
    int threads = 1;  // for the chunked passes of large nodes

    void leaf(const PrimRec* prims, int n, int parent, RefFrag& f) {
        for (int i = 0; i < n; i++) {
            f.leaf_order.push_back(prims[i].id);
            f.leaf_parent.push_back(parent);
        }
    }

    // bvh.h:151-216 for prims[0..n) under `parent` (a local id of f, or -1);
    // the partition is written back into prims (records move with it, so
    // every pass reads them in sequence).  spawn: levels on which the
    // left subtree may go to a new thread.
    void build(PrimRec* prims, int n, int parent, RefFrag& f, int spawn) {
        if (n < 4) {  // bvh.h:152-158: SimpleGroup of < 4 primitives
            leaf(prims, n, parent, f);
            return;
        }
        // large nodes: passes over the primitives in T chunks; boxes are
        // united with min / max and counts added, so the result does not
        // depend on the chunking
        const int T = (n >= kRefChunkMin && threads > 1) ? threads : 1;
        AB bounds, cb;
        {
            std::vector<AB> pb(T), pcb(T);
            par_chunks(T, n, [&](int c, int b, int e) {
                for (int i = b; i < e; i++) {
                    pb[c].unite(prims[i].b);
                    pcb[c].unite(prims[i].c);
                }
            });
            for (int c = 0; c < T; c++) {
                bounds.unite(pb[c]);
                cb.unite(pcb[c]);
            }
        }
        // compute_split for x, y, z (bvh.h:57-149): 5 equal-width bins over
        // the centroid bounds, a primitive joins the first bin j with
        // center < min + (max - min) * (j + 1) / 5
        const int P = 5;
        float cost[3];
        int best_split[3];
        float thr_axis[3][4];
        for (int axis = 0; axis < 3; axis++) {
            float lo = cb.lo[axis], hi = cb.hi[axis];
            for (int j = 0; j < P - 1; j++) thr_axis[axis][j] = lo + (hi - lo) * float(j + 1) / float(P);
        }
        std::vector<AB> pbin(T * 15);
        std::vector<int> pcnt(T * 15, 0);
        par_chunks(T, n, [&](int ch, int b0, int e0) {
            AB* bb = pbin.data() + 15 * ch;
            int* cc = pcnt.data() + 15 * ch;
            for (int i = b0; i < e0; i++) {
                const AB& pbx = prims[i].b;
                const V3& pc = prims[i].c;
                for (int axis = 0; axis < 3; axis++) {
                    const float* thr = thr_axis[axis];
                    float c = pc[axis];
                    int b = P - 1;
                    for (int j = 0; j < P - 1; j++)
                        if (c < thr[j]) { b = j; break; }
                    cc[5 * axis + b]++;
                    bb[5 * axis + b].unite(pbx);
                }
            }
        });
        for (int axis = 0; axis < 3; axis++) {
            AB bin_box[5];
            int cnt[5] = {0, 0, 0, 0, 0};
            for (int ch = 0; ch < T; ch++)
                for (int b = 0; b < P; b++) {
                    cnt[b] += pcnt[15 * ch + 5 * axis + b];
                    bin_box[b].unite(pbin[15 * ch + 5 * axis + b]);
                }
            float pc[4];
            for (int i = 0; i < P - 1; i++) {
                AB l, r;
                int lc = 0, rc = 0;
                for (int j = 0; j < P; j++) {
                    if (j <= i) { lc += cnt[j]; if (cnt[j]) l.unite(bin_box[j]); }
                    else { rc += cnt[j]; if (cnt[j]) r.unite(bin_box[j]); }
                }
                pc[i] = (lc == 0 || rc == 0) ? kInf : l.ref_area() + r.ref_area();
            }
            int m = 0;
            float mc = pc[0];
            for (int i = 1; i < P - 1; i++)
                if (pc[i] < mc) { mc = pc[i]; m = i; }
            cost[axis] = mc;
            best_split[axis] = m;
        }
        // bvh.h:179-197
        float c1 = cost[0], c2 = cost[1], c3 = cost[2];
        int axis;
        if (c1 < c2) axis = (c1 < c3) ? 0 : (c2 < c3 ? 1 : 2);
        else axis = (c2 < c3) ? 1 : 2;
        const int split = best_split[axis];
        // stable partition: bins 0..split, then split+1..4, each in input
        // order (one counting pass, one scatter)
        const float* thr = thr_axis[axis];
        if ((int)tmp.size() < n) tmp.resize(n);
        if ((int)bin_of.size() < n) bin_of.resize(n);
        std::vector<int> ccnt(T * 5, 0);
        par_chunks(T, n, [&](int ch, int b0, int e0) {
            int* cc = ccnt.data() + 5 * ch;
            for (int i = b0; i < e0; i++) {
                float c = prims[i].c[axis];
                int b = P - 1;
                for (int j = 0; j < P - 1; j++)
                    if (c < thr[j]) { b = j; break; }
                bin_of[i] = (uint8_t)b;
                cc[b]++;
            }
        });
        // chunk ch's bin b starts after all of bin b's earlier chunks
        std::vector<int> cstart(T * 5);
        int nl = 0;
        for (int b = 0, k = 0; b < P; b++) {
            for (int ch = 0; ch < T; ch++) {
                cstart[5 * ch + b] = k;
                k += ccnt[5 * ch + b];
            }
            if (b == split) nl = k;
        }
        if (nl == 0 || nl == n) {
            // The reference recurses without end here (bvh.h:200, TODO);
            // emit one leaf holding every primitive instead.
            leaf(prims, n, parent, f);
            return;
        }
        par_chunks(T, n, [&](int ch, int b0, int e0) {
            int* st = cstart.data() + 5 * ch;
            for (int i = b0; i < e0; i++) tmp[st[bin_of[i]]++] = prims[i];
        });
        par_chunks(T, n, [&](int, int b0, int e0) {
            std::memcpy(prims + b0, tmp.data() + b0, sizeof(PrimRec) * (e0 - b0));
        });
        const int32_t id = (int32_t)f.node_box.size();
        Box3 bx;
        bx.lo[0] = bounds.lo.x; bx.lo[1] = bounds.lo.y; bx.lo[2] = bounds.lo.z;
        bx.hi[0] = bounds.hi.x; bx.hi[1] = bounds.hi.y; bx.hi[2] = bounds.hi.z;
        f.node_box.push_back(bx);
        f.node_parent.push_back(parent);
        if (spawn > 0 && nl >= kRefParallelMin && n - nl >= kRefParallelMin) {
            // the two subtrees are independent: the left one on a new thread,
            // each into its own fragment, stitched in pre-order afterwards
            RefFrag lf, rf;
            std::thread th([&] {
                RefBuilder lb{{}, {}, std::max(1, threads / 2)};
                lb.build(prims, nl, -1, lf, spawn - 1);
            });
            threads = std::max(1, threads - threads / 2);
            build(prims + nl, n - nl, -1, rf, spawn - 1);
            th.join();
            append_frag(f, lf, id);
            append_frag(f, rf, id);
            return;
        }
        build(prims, nl, id, f, spawn);
        build(prims + nl, n - nl, id, f, spawn);
    }
};

}  // namespace

RefTopology build_ref_topology(const float* tri_v, int n, int n_threads) {
    RefTopology t;
    t.rank.assign(n, 0);
    t.prim_parent.assign(n, -1);
    t.leaf_order.reserve(n);
    std::vector<AB> box(n);
    std::vector<V3> cen(n);
    for (int i = 0; i < n; i++) {
        tri_box(tri_v + 9 * (size_t)i, &box[i]);
        // AABB::center (aabb.h:62-64): (min + max) * 0.5
        cen[i] = {(box[i].lo.x + box[i].hi.x) * 0.5f, (box[i].lo.y + box[i].hi.y) * 0.5f,
                  (box[i].lo.z + box[i].hi.z) * 0.5f};
    }
    std::vector<PrimRec> prims(n);
    for (int i = 0; i < n; i++) prims[i] = PrimRec{box[i], cen[i], i};
    if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
    int spawn = 0;
    while ((1 << spawn) < 2 * n_threads && spawn < 12) spawn++;
    if (n_threads == 1) spawn = 0;
    RefFrag f;
    f.leaf_order.reserve(n);
    f.leaf_parent.reserve(n);
    RefBuilder b{{}, {}, n_threads};
    if (n > 0) b.build(prims.data(), n, -1, f, spawn);
    t.leaf_order = std::move(f.leaf_order);
    for (int r = 0; r < n; r++) t.prim_parent[t.leaf_order[r]] = f.leaf_parent[r];
    t.node_box = std::move(f.node_box);
    t.node_parent = std::move(f.node_parent);
    for (int r = 0; r < n; r++) t.rank[t.leaf_order[r]] = r;
    return t;
}

// ---------------------------------------------------------------------------
// Binned SAH BVH2, collapsed to the compressed 4-wide layout.
// ---------------------------------------------------------------------------
namespace {

struct Node2 {
    AB box;
    int32_t left = -1, right = -1;  // children (Node2 indices), -1 for a leaf
    int32_t start = 0, count = 0;   // leaf range in the primitive order
};

struct SahBuilder {
    const std::vector<AB>& box;
    const std::vector<V3>& cen;
    std::vector<Node2>& nodes;
    std::atomic<int32_t>& next;
    int32_t* order;
    int max_leaf;

    static constexpr int kBins = 32;

    int32_t alloc() { return next.fetch_add(1); }

    void build(int32_t id, int start, int count, int depth, int threads) {
        Node2& nd = nodes[id];
        AB bb, cb;
        for (int i = start; i < start + count; i++) {
            bb.unite(box[order[i]]);
            cb.unite(cen[order[i]]);
        }
        nd.box = bb;
        if (count <= 1) { nd.start = start; nd.count = count; return; }
        int best_axis = -1, best_bin = -1;
        float best_cost = kInf;
        int mid = -1;
        if (depth < 56) {
            for (int axis = 0; axis < 3; axis++) {
                float lo = cb.lo[axis], hi = cb.hi[axis];
                if (!(hi > lo)) continue;
                float scale = kBins / (hi - lo);
                AB bins[kBins];
                int cnt[kBins] = {};
                for (int i = start; i < start + count; i++) {
                    int b = (int)((cen[order[i]][axis] - lo) * scale);
                    b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
                    cnt[b]++;
                    bins[b].unite(box[order[i]]);
                }
                float right_area[kBins];
                int right_cnt[kBins];
                AB acc;
                int c = 0;
                for (int b = kBins - 1; b > 0; b--) {
                    if (cnt[b]) acc.unite(bins[b]);
                    c += cnt[b];
                    right_area[b] = c ? acc.sah_area() : 0.0f;
                    right_cnt[b] = c;
                }
                AB lacc;
                int lc = 0;
                for (int b = 0; b < kBins - 1; b++) {
                    if (cnt[b]) lacc.unite(bins[b]);
                    lc += cnt[b];
                    int rc = right_cnt[b + 1];
                    if (lc == 0 || rc == 0) continue;
                    float cost = lacc.sah_area() * lc + right_area[b + 1] * rc;
                    if (cost < best_cost) { best_cost = cost; best_axis = axis; best_bin = b; }
                }
            }
        }
        float leaf_cost = bb.sah_area() * count;
        float trav = bb.sah_area() * 1.0f;  // traversal cost relative to one triangle test
        bool make_leaf = count <= max_leaf && (best_axis < 0 || best_cost + trav >= leaf_cost);
        if (make_leaf) { nd.start = start; nd.count = count; return; }
        // Both sides keep their order (a stable partition), so every node's
        // primitives stay sorted by insertion index and the tree depends
        // only on which primitives each node holds: the device build
        // (gpu_sah.cu) reproduces it node for node.
        if (best_axis >= 0) {
            float lo = cb.lo[best_axis], hi = cb.hi[best_axis];
            float scale = kBins / (hi - lo);
            int32_t* p = std::stable_partition(order + start, order + start + count, [&](int32_t t) {
                int b = (int)((cen[t][best_axis] - lo) * scale);
                b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
                return b <= best_bin;
            });
            mid = (int)(p - order);
        }
        if (mid <= start || mid >= start + count) {
            // no SAH split (coincident centroids or the depth limit): halve in
            // insertion order
            mid = start + count / 2;
        }
        int32_t l = alloc(), r = alloc();
        nd.left = l;
        nd.right = r;
        int nl = mid - start, nr = start + count - mid;
        if (threads > 1 && count > 65536) {
            std::thread th([&] { build(l, start, nl, depth + 1, threads / 2); });
            build(r, mid, nr, depth + 1, threads - threads / 2);
            th.join();
        } else {
            build(l, start, nl, depth + 1, 1);
            build(r, mid, nr, depth + 1, 1);
        }
    }
};

uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

}  // namespace

WideBVH build_wide_bvh(const float* tri_v, int n, int max_leaf, int n_threads) {
    if (max_leaf < 1 || max_leaf > 16) throw std::invalid_argument("max_leaf must be in [1,16]");
    WideBVH out;
    out.max_leaf = max_leaf;
    std::vector<AB> box(n > 0 ? n : 1);
    std::vector<V3> cen(n > 0 ? n : 1);
    AB scene;
    for (int i = 0; i < n; i++) {
        tri_box(tri_v + 9 * (size_t)i, &box[i]);
        scene.unite(box[i]);
    }
    // Boxes are inflated by delta, far above the rounding error of the
    // device slab test for rays starting inside or near the scene.
    float ext = 0.0f, mag = 0.0f;
    if (n > 0) {
        for (int k = 0; k < 3; k++) {
            ext = std::max(ext, scene.hi[k] - scene.lo[k]);
            mag = std::max(mag, std::max(std::fabs(scene.hi[k]), std::fabs(scene.lo[k])));
        }
    }
    float delta = (ext + mag + 1e-3f) * (1.0f / 262144.0f);
    out.inflate = delta;
    for (int i = 0; i < n; i++) {
        box[i].lo = {box[i].lo.x - delta, box[i].lo.y - delta, box[i].lo.z - delta};
        box[i].hi = {box[i].hi.x + delta, box[i].hi.y + delta, box[i].hi.z + delta};
        cen[i] = {0.5f * (box[i].lo.x + box[i].hi.x), 0.5f * (box[i].lo.y + box[i].hi.y),
                  0.5f * (box[i].lo.z + box[i].hi.z)};
    }
    out.tri_order.resize(n);
    for (int i = 0; i < n; i++) out.tri_order[i] = i;

    std::vector<Node2> nodes(n > 0 ? 2 * (size_t)n : 1);
    std::atomic<int32_t> next{1};
    if (n_threads <= 0) n_threads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    SahBuilder sb{box, cen, nodes, next, out.tri_order.data(), max_leaf};
    if (n > 0) sb.build(0, 0, n, 0, n_threads);
    else { nodes[0].count = 0; }

    // Collapse into 4-wide nodes, breadth first.
    struct Item { int32_t n2; int depth; };
    std::vector<Item> queue;
    queue.push_back({0, 1});
    out.nodes.reserve(n / 2 + 1);
    for (size_t qi = 0; qi < queue.size(); qi++) {
        int32_t n2 = queue[qi].n2;
        int depth = queue[qi].depth;
        out.max_depth = std::max(out.max_depth, depth);
        // gather up to 4 children
        int32_t ch[4];
        int nc = 0;
        if (nodes[n2].left < 0) {
            ch[nc++] = n2;  // a root that is a leaf
        } else {
            ch[nc++] = nodes[n2].left;
            ch[nc++] = nodes[n2].right;
            while (nc < 4) {
                int pick = -1;
                float best = -1.0f;
                for (int i = 0; i < nc; i++)
                    if (nodes[ch[i]].left >= 0 && nodes[ch[i]].box.sah_area() > best) {
                        best = nodes[ch[i]].box.sah_area();
                        pick = i;
                    }
                if (pick < 0) break;
                int32_t c = ch[pick];
                ch[pick] = nodes[c].left;
                ch[nc++] = nodes[c].right;
            }
        }
        WideNode wn;
        std::memset(&wn, 0, sizeof(wn));
        AB nb;
        for (int i = 0; i < nc; i++) nb.unite(nodes[ch[i]].box);
        if (nc == 0 || n == 0) nb.lo = nb.hi = {0, 0, 0};
        float p[3] = {nb.lo.x, nb.lo.y, nb.lo.z};
        double s[3];
        uint32_t ebits[3];
        for (int k = 0; k < 3; k++) {
            double E = (double)nb.hi[k] - (double)p[k];
            int e;
            std::frexp(std::max(E / 254.0, 1e-30), &e);  // E/254 < 2^e
            if (e < -126) e = -126;
            if (e > 127) throw std::runtime_error("scene coordinates out of range");
            s[k] = std::ldexp(1.0, e);
            ebits[k] = (uint32_t)(e + 127);
            wn.w[k] = fbits(p[k]);
        }
        wn.w[3] = ebits[0] | (ebits[1] << 8) | (ebits[2] << 16);
        uint8_t qlo[3][4], qhi[3][4];
        for (int k = 0; k < 3; k++)
            for (int i = 0; i < 4; i++) { qlo[k][i] = 255; qhi[k][i] = 0; }
        uint32_t refs[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
        for (int i = 0; i < nc; i++) {
            const Node2& c = nodes[ch[i]];
            for (int k = 0; k < 3; k++) {
                double lo = std::floor(((double)c.box.lo[k] - p[k]) / s[k]);
                double hi = std::ceil(((double)c.box.hi[k] - p[k]) / s[k]);
                while (lo > 0 && (double)p[k] + lo * s[k] > (double)c.box.lo[k]) lo -= 1;
                while (hi < 255 && (double)p[k] + hi * s[k] < (double)c.box.hi[k]) hi += 1;
                lo = std::max(0.0, std::min(255.0, lo));
                hi = std::max(0.0, std::min(255.0, hi));
                qlo[k][i] = (uint8_t)lo;
                qhi[k][i] = (uint8_t)hi;
            }
            if (c.left < 0) {
                if (c.count == 0) { qlo[0][i] = 255; qhi[0][i] = 0; continue; }
                if (c.count > 16) throw std::runtime_error("leaf too large");
                refs[i] = make_leaf_ref((uint32_t)c.start, (uint32_t)c.count);
            } else {
                refs[i] = (uint32_t)queue.size();  // breadth-first: queue position = node index
                queue.push_back({ch[i], depth + 1});
            }
        }
        auto pack = [](const uint8_t* b) {
            return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
        };
        wn.w[4] = pack(qlo[0]);
        wn.w[5] = pack(qlo[1]);
        wn.w[6] = pack(qlo[2]);
        wn.w[7] = pack(qhi[0]);
        wn.w[8] = pack(qhi[1]);
        wn.w[9] = pack(qhi[2]);
        for (int i = 0; i < 4; i++) wn.w[10 + i] = refs[i];
        out.nodes.push_back(wn);
    }
    return out;
}

}  // namespace cpppt_gb300
