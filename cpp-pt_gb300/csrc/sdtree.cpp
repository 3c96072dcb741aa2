// Host side of the SD-tree (see sdtree.h).  Compiled with -ffp-contract=off
// like bvh.cpp; the float/double steps follow src/algorithms/sdtree.h.
#include "sdtree.h"

#include <cmath>
#include <unordered_map>
#include <utility>

namespace cpppt_gb300 {
namespace {
const float kPiF = (float)3.14159265358979323846;
const double kPiD = 3.14159265358979323846;
}  // namespace

std::unique_ptr<DNodeH> DNodeH::clone() const {
    auto n = std::make_unique<DNodeH>();
    n->leaf = leaf;
    n->value = value;
    if (!leaf)
        for (int i = 0; i < 4; i++) n->child[i] = child[i]->clone();
    return n;
}

DTreeH::DTreeH() : root(std::make_unique<DNodeH>()) {
    // DTree() (sdtree.h:117-119): one leaf covering (phi, cos) in [-pi,pi] x [-1,1]
    leaves.push_back({-kPiF, -1.0f, (float)(2.0 * kPiD), 2.0f});
}

std::unique_ptr<DTreeH> DTreeH::clone() const {
    auto d = std::make_unique<DTreeH>();
    d->root = root->clone();
    d->count = count;
    d->radiance = radiance;
    d->leaves = leaves;
    return d;
}

// DTree::get_radiance_and_prune (sdtree.h:97-113)
static float radiance_and_prune(DNodeH* n, float threshold) {
    if (n->leaf) return n->value;
    float rad = 0.0f;
    for (int i = 0; i < 4; i++) rad += radiance_and_prune(n->child[i].get(), threshold);
    if (rad < threshold) {
        for (int i = 0; i < 4; i++) n->child[i].reset();
        n->leaf = true;
        n->value = rad;
    }
    return rad;
}

// DTree::adapt_and_build_leaves (sdtree.h:172-233)
void DTreeH::adapt_and_build_leaves() {
    if ((double)radiance == 0.0) return;
    const float threshold = (float)((double)radiance * 0.01);
    leaves.clear();
    std::vector<DNodeH*> stack{root.get()};
    std::vector<DLeafRegion> lstack{{-kPiF, -1.0f, (float)(2.0 * kPiD), 2.0f}};
    radiance_and_prune(root.get(), threshold);
    while (!stack.empty()) {
        DNodeH* dn = stack.back();
        stack.pop_back();
        DLeafRegion l = lstack.back();
        lstack.pop_back();
        if (dn->leaf) {
            const float ratio = dn->value / threshold;
            if ((double)ratio > 1.0) {
                const float q = (float)((double)dn->value * 0.25);
                dn->leaf = false;
                for (int i = 0; i < 4; i++) {
                    dn->child[i] = std::make_unique<DNodeH>();
                    dn->child[i]->value = q;
                }
            } else {
                dn->value = 0.0f;
                leaves.push_back(l);
                continue;
            }
        }
        for (int i = 0; i < 4; i++) {
            stack.push_back(dn->child[i].get());
            DLeafRegion c;
            c.bx = (float)((double)l.bx + (double)l.sx * 0.5 * (double)(i % 2));
            c.by = (float)((double)l.by + (double)l.sy * 0.5 * (double)(i / 2));
            c.sx = l.sx * 0.5f;
            c.sy = l.sy * 0.5f;
            lstack.push_back(c);
        }
    }
    count = 0;
    radiance = 0.0f;
}

SDTreeHost::SDTreeHost(const float lo[3], const float hi[3]) : root_(std::make_unique<SNodeH>()) {
    for (int k = 0; k < 3; k++) { lo_[k] = lo[k]; hi_[k] = hi[k]; }
    root_->dtree = std::make_unique<DTreeH>();
}

int SDTreeHost::n_spatial_leaves() const {
    int n = 0;
    std::vector<const SNodeH*> st{root_.get()};
    while (!st.empty()) {
        const SNodeH* s = st.back();
        st.pop_back();
        if (s->dtree) n++;
        else { st.push_back(s->child[0].get()); st.push_back(s->child[1].get()); }
    }
    return n;
}

// SDTree::subdivide (sdtree.h:459-512) with c = 12000
void SDTreeHost::update() {
    const int threshold = c_ * (int)std::pow(2.0, (double)iteration_ * 0.5);
    std::vector<std::pair<SNodeH*, int>> stack{{root_.get(), 0}};
    while (!stack.empty()) {
        SNodeH* n = stack.back().first;
        int sub = stack.back().second;
        stack.pop_back();
        if (n->dtree) {
            if (n->dtree->count > threshold || sub) {
                int to_sub = sub;
                if (sub == 0) {
                    const float ratio = (float)n->dtree->count / (float)threshold;
                    to_sub = (int)std::log2(ratio) + 1;
                    n->dtree->adapt_and_build_leaves();
                }
                n->child[0] = std::make_unique<SNodeH>();
                n->child[1] = std::make_unique<SNodeH>();
                n->child[0]->dtree = n->dtree->clone();
                n->child[1]->dtree = n->dtree->clone();
                n->dtree.reset();
                stack.push_back({n->child[0].get(), to_sub - 1});
                stack.push_back({n->child[1].get(), to_sub - 1});
            } else {
                n->dtree->adapt_and_build_leaves();
            }
        } else {
            stack.push_back({n->child[0].get(), 0});
            stack.push_back({n->child[1].get(), 0});
        }
    }
    iteration_++;
}

namespace {
// Visits spatial leaves and quadtree leaves in the order flatten() numbers them.
template <class SLeaf, class DLeaf>
void walk(const SNodeH* root, SLeaf on_sleaf, DLeaf on_dleaf) {
    std::vector<const SNodeH*> st{root};
    while (!st.empty()) {
        const SNodeH* s = st.back();
        st.pop_back();
        if (s->dtree) {
            on_sleaf(s);
            std::vector<const DNodeH*> ds{s->dtree->root.get()};
            while (!ds.empty()) {
                const DNodeH* d = ds.back();
                ds.pop_back();
                if (d->leaf) on_dleaf(s, d);
                else
                    for (int i = 3; i >= 0; i--) ds.push_back(d->child[i].get());
            }
        } else {
            st.push_back(s->child[1].get());
            st.push_back(s->child[0].get());
        }
    }
}
}  // namespace

void SDTreeHost::accumulate(const float* slot_values, const int32_t* counts, const float* radiance) {
    int slot = 0, dtree = 0;
    walk(
        root_.get(),
        [&](const SNodeH* s) {
            DTreeH* d = s->dtree.get();
            d->count += counts[dtree];
            d->radiance += radiance[dtree];
            dtree++;
        },
        [&](const SNodeH*, const DNodeH* d) { const_cast<DNodeH*>(d)->value += slot_values[slot++]; });
}

SDTreeFlat SDTreeHost::flatten() const {
    SDTreeFlat f;
    for (int k = 0; k < 3; k++) { f.lo[k] = lo_[k]; f.hi[k] = hi_[k]; }
    // spatial nodes breadth first
    std::vector<const SNodeH*> q{root_.get()};
    std::vector<const DTreeH*> dtrees;
    f.snode.resize(2);
    for (size_t i = 0; i < q.size(); i++) {
        const SNodeH* s = q[i];
        if (s->dtree) {
            f.snode[2 * i] = -1 - (int32_t)dtrees.size();
            f.snode[2 * i + 1] = -1;
            dtrees.push_back(s->dtree.get());
        } else {
            f.snode[2 * i] = (int32_t)q.size();
            f.snode[2 * i + 1] = (int32_t)q.size() + 1;
            q.push_back(s->child[0].get());
            q.push_back(s->child[1].get());
            f.snode.resize(2 * q.size());
        }
    }
    // value slots must follow the walk() order used by accumulate(): number
    // the quadtree leaves in that order first
    std::unordered_map<const DNodeH*, int> slot_of;
    {
        int slot = 0;
        walk(root_.get(), [](const SNodeH*) {}, [&](const SNodeH*, const DNodeH* d) { slot_of[d] = slot++; });
        f.n_value_slots = slot;
    }
    auto find_slot = [&](const DNodeH* d) { return slot_of.at(d); };
    // dtrees in walk order (spatial leaves, depth first, child 0 first)
    std::vector<const DTreeH*> order;
    walk(root_.get(), [&](const SNodeH* s) { order.push_back(s->dtree.get()); }, [](const SNodeH*, const DNodeH*) {});
    // map breadth-first dtree ids to walk order ids
    std::unordered_map<const DTreeH*, int32_t> pos;
    for (size_t j = 0; j < order.size(); j++) pos[order[j]] = (int32_t)j;
    std::vector<int32_t> remap(dtrees.size());
    for (size_t i = 0; i < dtrees.size(); i++) remap[i] = pos.at(dtrees[i]);
    for (size_t i = 0; i < f.snode.size(); i += 2)
        if (f.snode[i] < 0) f.snode[i] = -1 - remap[-1 - f.snode[i]];
    f.dtree_root.resize(order.size());
    f.dtree_leaf_off.resize(order.size());
    f.dtree_leaf_cnt.resize(order.size());
    for (size_t t = 0; t < order.size(); t++) {
        const DTreeH* d = order[t];
        f.dtree_root[t] = (int32_t)f.dnode.size();
        std::vector<const DNodeH*> bq{d->root.get()};
        f.dnode.push_back(0);
        for (size_t i = 0; i < bq.size(); i++) {
            const DNodeH* n = bq[i];
            const size_t me = f.dtree_root[t] + i;
            if (n->leaf) {
                f.dnode[me] = -1 - find_slot(n);
            } else {
                f.dnode[me] = f.dtree_root[t] + (int32_t)bq.size();
                for (int c = 0; c < 4; c++) {
                    bq.push_back(n->child[c].get());
                    f.dnode.push_back(0);
                }
            }
        }
        f.dtree_leaf_off[t] = (int32_t)(f.leaves.size() / 4);
        f.dtree_leaf_cnt[t] = (int32_t)d->leaves.size();
        for (const DLeafRegion& l : d->leaves) {
            f.leaves.push_back(l.bx);
            f.leaves.push_back(l.by);
            f.leaves.push_back(l.sx);
            f.leaves.push_back(l.sy);
        }
    }
    return f;
}

DTreeH* SDTreeHost::find(const float pos[3]) const {
    float lo[3] = {lo_[0], lo_[1], lo_[2]}, hi[3] = {hi_[0], hi_[1], hi_[2]};
    const SNodeH* n = root_.get();
    for (int depth = 0;; depth++) {
        if (n->dtree) return n->dtree.get();
        const int k = depth % 3;
        const float mid = (float)((double)(lo[k] + hi[k]) * 0.5);
        if (pos[k] > mid) { lo[k] = mid; n = n->child[1].get(); }
        else { hi[k] = mid; n = n->child[0].get(); }
    }
}

// quadtree leaf containing (x, y) and the size of its cell (sdtree.h:277-352)
static DNodeH* dleaf(DNodeH* root, float x, float y, float* wx, float* wy) {
    float lx = -kPiF, ly = -1.0f, hx = kPiF, hy = 1.0f;
    DNodeH* n = root;
    while (!n->leaf) {
        const float mx = (lx + hx) * 0.5f, my = (ly + hy) * 0.5f;
        int c;
        if (x < mx) {
            if (y < my) { c = 0; hx = mx; hy = my; }
            else { c = 2; hx = mx; ly = my; }
        } else {
            if (y < my) { c = 1; lx = mx; hy = my; }
            else { c = 3; lx = mx; ly = my; }
        }
        n = n->child[c].get();
    }
    *wx = hx - lx;
    *wy = hy - ly;
    return n;
}

void SDTreeHost::splat(float radiance, const float pos[3], const float dir[3]) {
    DTreeH* d = find(pos);
    float wx, wy;
    DNodeH* l = dleaf(d->root.get(), std::atan2(dir[1], dir[0]), dir[2], &wx, &wy);
    l->value += radiance;
    d->count += 1;
    d->radiance += radiance;
}

float SDTreeHost::pdf(const float pos[3], const float dir[3]) const {
    DTreeH* d = find(pos);
    float wx, wy;
    dleaf(d->root.get(), std::atan2(dir[1], dir[0]), dir[2], &wx, &wy);
    return (float)((1.0 / (double)d->leaves.size()) * (1.0 / (double)(wx * wy)));
}

void SDTreeHost::dump(std::vector<DLeafRegion>* leaves, std::vector<int>* leaf_counts, std::vector<int>* counts,
                      std::vector<float>* flux) const {
    walk(
        root_.get(),
        [&](const SNodeH* s) {
            const DTreeH* d = s->dtree.get();
            leaves->insert(leaves->end(), d->leaves.begin(), d->leaves.end());
            leaf_counts->push_back((int)d->leaves.size());
            counts->push_back(d->count);
            flux->push_back(d->radiance);
        },
        [](const SNodeH*, const DNodeH*) {});
}

}  // namespace cpppt_gb300
