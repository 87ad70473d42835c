// Host-side SAH BVH build.
//
// The split rules are the reference's (include/bvh.h:110-205): centroids are
// binned into 16 bins along the longest centroid axis, the split with the
// lowest A_left N_left + A_right N_right wins, a node of at most 4 primitives
// stays a leaf when that is cheaper than 0.125 + best_cost / A, and below
// depth 64 (or when centroids coincide) lists are split in the middle. The
// result is the same depth-first array (left child next, right child index in
// `offset`). Unlike the reference, which nests one BVH per mesh and per
// instance, this builds one tree over every primitive of the scene, so the
// device walks a single level.
#include "bvh_build.h"

#include <algorithm>

namespace mypbr_host {

namespace {

constexpr int kBins = 16;
constexpr int kMaxLeaf = 4;
constexpr int kMaxSahDepth = 64;

struct Builder {
    std::vector<BuildItem>& items;
    std::vector<mypbr_bvh_node>& nodes;

    int leaf(int index, size_t begin, size_t count, int axis, int depth) {
        if (count > size_t(kMaxLeaf)) {
            size_t mid = begin + count / 2;
            nodes[index].axis = axis;
            build(begin, mid, depth + 1);
            int right = build(mid, begin + count, depth + 1);
            nodes[index].offset = right;
            return index;
        }
        nodes[index].offset = int(begin);
        nodes[index].count = int(count);
        return index;
    }

    int build(size_t begin, size_t end, int depth) {
        int index = int(nodes.size());
        nodes.push_back(mypbr_bvh_node{});
        Box bounds, cbounds;
        for (size_t k = begin; k < end; k++) {
            bounds.grow(items[k].box);
            // A point box is padded to 1e-4 per side, as the reference's centroid
            // bounds are (bvh.h:263), so their extent is never exactly zero
            cbounds.grow(Box::from_points(items[k].centroid, items[k].centroid));
        }
        for (int a = 0; a < 3; a++) {
            nodes[index].bmin[a] = bounds.lo[a];
            nodes[index].bmax[a] = bounds.hi[a];
        }
        size_t count = end - begin;
        int axis = cbounds.longest_axis();
        double lo = cbounds.lo[axis], extent = cbounds.size(axis);
        if (count == 1 || extent <= 0 || depth >= kMaxSahDepth)
            return leaf(index, begin, count, axis, depth);

        auto bin_of = [&](const V3& c) {
            int b = int(kBins * (c[axis] - lo) / extent);
            return std::min(b, kBins - 1);
        };
        Box bin_box[kBins];
        int bin_count[kBins] = {};
        for (size_t k = begin; k < end; k++) {
            int b = bin_of(items[k].centroid);
            bin_box[b].grow(items[k].box);
            bin_count[b]++;
        }
        // Prefix sweeps: left boxes/counts after bins [0, s], right before (s, 15]
        Box left_box[kBins], right_box[kBins];
        int left_n[kBins], right_n[kBins];
        Box acc;
        int n = 0;
        for (int s = 0; s < kBins; s++) {
            acc.grow(bin_box[s]);
            n += bin_count[s];
            left_box[s] = acc;
            left_n[s] = n;
        }
        acc = Box();
        n = 0;
        for (int s = kBins - 1; s >= 0; s--) {
            acc.grow(bin_box[s]);
            n += bin_count[s];
            right_box[s] = acc;
            right_n[s] = n;
        }
        double best_cost = kInf;
        int best_split = -1;
        for (int s = 0; s < kBins - 1; s++) {
            int nl = left_n[s], nr = right_n[s + 1];
            if (nl == 0 || nr == 0)
                continue;
            double cost = left_box[s].surface_area() * nl + right_box[s + 1].surface_area() * nr;
            if (cost < best_cost) {
                best_cost = cost;
                best_split = s;
            }
        }
        double leaf_cost = double(count);
        double split_cost = 0.125 + best_cost / bounds.surface_area();
        if (best_split < 0 || (count <= size_t(kMaxLeaf) && leaf_cost <= split_cost))
            return leaf(index, begin, count, axis, depth);

        auto mid_it = std::partition(items.begin() + begin, items.begin() + end,
                                     [&](const BuildItem& it) { return bin_of(it.centroid) <= best_split; });
        size_t mid = size_t(mid_it - items.begin());
        nodes[index].axis = axis;
        build(begin, mid, depth + 1);
        int right = build(mid, end, depth + 1);
        nodes[index].offset = right;
        return index;
    }
};

}  // namespace

void build_bvh(std::vector<BuildItem> items, std::vector<mypbr_bvh_node>& nodes, std::vector<mypbr_prim_ref>& prims) {
    nodes.clear();
    prims.clear();
    if (items.empty()) {
        mypbr_bvh_node empty{};
        for (int a = 0; a < 3; a++) {
            empty.bmin[a] = kInf;
            empty.bmax[a] = -kInf;
        }
        nodes.push_back(empty);
        return;
    }
    nodes.reserve(2 * items.size());
    Builder b{items, nodes};
    b.build(0, items.size(), 0);
    prims.reserve(items.size());
    for (const auto& it : items)
        prims.push_back(it.ref);
}

}  // namespace mypbr_host
