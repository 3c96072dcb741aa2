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
struct RefBuilder {
    const std::vector<AB>& box;
    const std::vector<V3>& cen;
    RefTopology& out;
    std::vector<int32_t> tmp;
    std::vector<uint8_t> bin_of;

    // returns the internal-node id, or -1 when a leaf was emitted
    void build(int32_t* prims, int n, int parent) {
        if (n < 4) {  // bvh.h:152-158: SimpleGroup of < 4 primitives
            for (int i = 0; i < n; i++) {
                out.prim_parent[prims[i]] = parent;
                out.leaf_order.push_back(prims[i]);
            }
            return;
        }
        AB bounds, cb;
        for (int i = 0; i < n; i++) {
            bounds.unite(box[prims[i]]);
            cb.unite(cen[prims[i]]);
        }
        // compute_split for x, y, z
        float cost[3];
        int best_split[3];
        for (int axis = 0; axis < 3; axis++) {
            const int P = 5;
            float lo = cb.lo[axis], hi = cb.hi[axis];
            float thr[4];
            for (int j = 0; j < P - 1; j++) thr[j] = lo + (hi - lo) * float(j + 1) / float(P);
            AB bin_box[5];
            int cnt[5] = {0, 0, 0, 0, 0};
            for (int i = 0; i < n; i++) {
                float c = cen[prims[i]][axis];
                int b = P - 1;
                for (int j = 0; j < P - 1; j++)
                    if (c < thr[j]) { b = j; break; }
                cnt[b]++;
                bin_box[b].unite(box[prims[i]]);
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
        int split = best_split[axis];
        // stable partition: bins 0..split, then split+1..4, each in input order
        {
            const int P = 5;
            float lo = cb.lo[axis], hi = cb.hi[axis];
            float thr[4];
            for (int j = 0; j < P - 1; j++) thr[j] = lo + (hi - lo) * float(j + 1) / float(P);
            if ((int)tmp.size() < n) tmp.resize(n);
            int nl = 0;
            for (int i = 0; i < n; i++) {
                float c = cen[prims[i]][axis];
                int b = P - 1;
                for (int j = 0; j < P - 1; j++)
                    if (c < thr[j]) { b = j; break; }
                bin_of[i] = (uint8_t)b;
            }
            int k = 0;
            for (int b = 0; b < P; b++) {
                for (int i = 0; i < n; i++)
                    if (bin_of[i] == b) tmp[k++] = prims[i];
                if (b == split) nl = k;
            }
            if (nl == 0 || nl == n) {
                // The reference recurses without end here (bvh.h:200, TODO);
                // emit one leaf holding every primitive instead.
                for (int i = 0; i < n; i++) {
                    out.prim_parent[prims[i]] = parent;
                    out.leaf_order.push_back(prims[i]);
                }
                return;
            }
            std::memcpy(prims, tmp.data(), sizeof(int32_t) * n);
            int id = (int)out.node_box.size();
            Box3 bx;
            bx.lo[0] = bounds.lo.x; bx.lo[1] = bounds.lo.y; bx.lo[2] = bounds.lo.z;
            bx.hi[0] = bounds.hi.x; bx.hi[1] = bounds.hi.y; bx.hi[2] = bounds.hi.z;
            out.node_box.push_back(bx);
            out.node_parent.push_back(parent);
            build(prims, nl, id);
            build(prims + nl, n - nl, id);
        }
    }
};

}  // namespace

RefTopology build_ref_topology(const float* tri_v, int n) {
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
    std::vector<int32_t> prims(n);
    for (int i = 0; i < n; i++) prims[i] = i;
    RefBuilder b{box, cen, t, {}, {}};
    b.bin_of.resize(n > 0 ? n : 1);
    if (n > 0) b.build(prims.data(), n, -1);
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
        if (best_axis >= 0) {
            float lo = cb.lo[best_axis], hi = cb.hi[best_axis];
            float scale = kBins / (hi - lo);
            int32_t* p = std::partition(order + start, order + start + count, [&](int32_t t) {
                int b = (int)((cen[t][best_axis] - lo) * scale);
                b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
                return b <= best_bin;
            });
            mid = (int)(p - order);
        }
        if (mid <= start || mid >= start + count) {
            // no useful SAH split (coincident centroids or depth limit): median split
            int axis = 0;
            float ext = -1.0f;
            for (int k = 0; k < 3; k++)
                if (cb.hi[k] - cb.lo[k] > ext) { ext = cb.hi[k] - cb.lo[k]; axis = k; }
            mid = start + count / 2;
            std::nth_element(order + start, order + mid, order + start + count,
                             [&](int32_t a, int32_t b) { return cen[a][axis] < cen[b][axis]; });
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
