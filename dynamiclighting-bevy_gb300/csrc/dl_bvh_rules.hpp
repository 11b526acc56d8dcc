// The occluder BVH's build rules, shared by the host builder (dl_host.cpp) and the device builder
// (dl_bvh.cu), which make the same tree: binned SAH over the primitives' centroids, kBvhBins bins
// per axis, leaves of at most kBvhMaxLeaf triangles when a split does not pay, depth capped at
// kBvhMaxDepth. Every decision comes from exact quantities (min/max bounds, integer counts) and
// from the binary32 arithmetic below, evaluated in one order on both sides.
#pragma once

#include <cstdint>

#include "dl_math.cuh"

namespace dl {

// A sweep (16 or 32 bins, leaves of 2 to 7, node costs 0.3 to 2) left the outdoor bake within
// 1 % of these, larger leaves slower.
constexpr int kBvhBins = 16;
constexpr uint32_t kBvhMaxLeaf = 4;   // at most 7 (the leaf reference's count field)
constexpr float kBvhNodeCost = 0.3f;  // SAH cost of a node visit, triangle tests costing 1
constexpr uint32_t kBvhMaxDepth = 60;

// std::min / std::max, written out so that host and device pick the same operand.
DL_HD float bvh_min(float a, float b) { return b < a ? b : a; }
DL_HD float bvh_max(float a, float b) { return a < b ? b : a; }

DL_HD float bvh_half_area(const float lo[3], const float hi[3]) {
    float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
    if (e0 < 0 || e1 < 0 || e2 < 0) return 0.0f;
    return e0 * e1 + e1 * e2 + e2 * e0;
}

// The bin of centroid coordinate c for centroid bounds starting at clo, k = kBvhBins / extent.
DL_HD int bvh_bin(float c, float clo, float k) {
    int b = (int)((c - clo) * k);
    return b < kBvhBins - 1 ? b : kBvhBins - 1;
}

// Boxes, counts and centroid-axis use of one node's bins.
struct BvhBins {
    float bl[3][kBvhBins][3], bh[3][kBvhBins][3];
    uint32_t bc[3][kBvhBins];
};

// The SAH sweep over the bins of the used axes: the cheapest split (lowest axis, then lowest bin
// on ties) as `axis` (-1: none) and `bin` (left = bins <= bin), with its cost.
DL_HD void bvh_best_split(const BvhBins &b, const bool use[3], float &best_cost, int &axis, int &bin) {
    best_cost = INFINITY;
    axis = -1;
    bin = 0;
    for (int a = 0; a < 3; ++a) {
        if (!use[a]) continue;
        float rarea[kBvhBins];
        uint32_t rcount[kBvhBins];
        float rl[3] = {INFINITY, INFINITY, INFINITY}, rh[3] = {-INFINITY, -INFINITY, -INFINITY};
        uint32_t rc = 0;
        for (int k = kBvhBins - 1; k > 0; --k) {
            rc += b.bc[a][k];
            for (int j = 0; j < 3; ++j) {
                rl[j] = bvh_min(rl[j], b.bl[a][k][j]);
                rh[j] = bvh_max(rh[j], b.bh[a][k][j]);
            }
            rarea[k] = bvh_half_area(rl, rh);
            rcount[k] = rc;
        }
        float ll[3] = {INFINITY, INFINITY, INFINITY}, lh[3] = {-INFINITY, -INFINITY, -INFINITY};
        uint32_t lc = 0;
        for (int k = 0; k < kBvhBins - 1; ++k) {
            lc += b.bc[a][k];
            for (int j = 0; j < 3; ++j) {
                ll[j] = bvh_min(ll[j], b.bl[a][k][j]);
                lh[j] = bvh_max(lh[j], b.bh[a][k][j]);
            }
            if (!lc || !rcount[k + 1]) continue;
            float c = bvh_half_area(ll, lh) * (float)lc + rarea[k + 1] * (float)rcount[k + 1];
            if (c < best_cost) {
                best_cost = c;
                axis = a;
                bin = k;
            }
        }
    }
}

// How a node with `count` primitives at `depth` (the root is 1) is split.
enum BvhSplit : int { kBvhLeaf = 0, kBvhByBin = 1, kBvhByIndex = 2 };
// The decision before binning: leaves of at most 2 primitives (7 at the depth cap).
DL_HD bool bvh_leaf_before_bins(uint32_t count, uint32_t depth) {
    return count <= 2 || (depth >= kBvhMaxDepth && count <= 7);
}
// The decision after the sweep, from the node's box (lo, hi) and the best split.
DL_HD BvhSplit bvh_decide(uint32_t count, uint32_t depth, const float lo[3], const float hi[3], float best_cost,
                          int axis) {
    float parent_area = bvh_half_area(lo, hi);
    float leaf_cost = (float)count;
    float split_cost = kBvhNodeCost + (parent_area > 0.0f ? best_cost / parent_area : (float)count);
    if (axis < 0 || depth >= kBvhMaxDepth) return count <= kBvhMaxLeaf ? kBvhLeaf : kBvhByIndex;
    if (count <= kBvhMaxLeaf && leaf_cost <= split_cost) return kBvhLeaf;
    return kBvhByBin;
}

// Boxes are padded so that culling stays conservative with respect to the triangle test's own
// rounding: an absolute margin scaled by the coordinate magnitude.
DL_HD void bvh_pad_box(float lo[3], float hi[3]) {
    for (int a = 0; a < 3; ++a) {
        float m = bvh_max(fabsf(lo[a]), fabsf(hi[a]));
        float pad = 1e-5f * bvh_max(1.0f, m);
        lo[a] -= pad;
        hi[a] += pad;
    }
}

}  // namespace dl
