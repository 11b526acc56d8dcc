// The occluder BVH built on the device: the host builder's binned-SAH tree (build_bvh in
// dl_host.cpp), from triangles already resident in device memory. The reference builds its
// occluder BVH once per bake on the CPU (src/bake/occluder.rs:63-114); here the build takes a few
// milliseconds and no host copy of the scene.
//
// Both builders evaluate the same rules (dl_bvh_rules.hpp) on the same exact quantities: bounds
// are minima and maxima, bins are counts and bounds, and their partitions are stable, so the
// device tree equals the host tree node for node and triangle for triangle.
//
//   large nodes (more than kSmall primitives), one level of them at a time:
//     bounds     blocks of kChunk positions reduce box and centroid bounds per node (atomics on
//                order-preserving integer images of the floats)
//     bins       the same blocks bin centroids per axis in shared memory, then merge per node
//     split      a thread per node: SAH sweep, decision, children (large ones to the next level,
//                the others to the small list)
//     partition  per-block left counts, per-node block offsets, stable scatter, copy back
//   small nodes: a warp builds a whole subtree depth first (bounds by warp reductions, bins by
//     shared-memory atomics, stable partition by ballots)
//   layout: subtree sizes bottom-up and depth-first positions top-down, level by level; nodes
//     written at their positions with padded child boxes; triangles in leaf order.
#include "dl_bvh.hpp"

#include <algorithm>
#include <vector>

#include "dl_bvh_rules.hpp"

namespace dl {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kChunk = 4096;     // positions per block in the large-node kernels
constexpr uint32_t kSmall = 512;      // nodes up to this size are built whole by one warp
constexpr int kWarpStack = 96;        // pending nodes of a warp's subtree (depth + 1 at most)
constexpr int kBinWords = 3 * kBvhBins * 7;  // per (axis, bin): count, lo xyz, hi xyz

#define BK(x)                                                                 \
    do {                                                                      \
        cudaError_t e__ = (x);                                                \
        if (e__ != cudaSuccess) throw DeviceBvhError{e__, #x};                \
    } while (0)
#define BLAUNCHED(name)                                                       \
    do {                                                                      \
        cudaError_t e__ = cudaGetLastError();                                 \
        if (e__ != cudaSuccess) throw DeviceBvhError{e__, name};              \
    } while (0)

// An order-preserving map of finite floats to ints (atomicMin/atomicMax on the images order the
// floats); it is its own inverse.
__device__ __forceinline__ int ford(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float funord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

struct Task {
    uint32_t node, first, count, depth;
};

// A node while the tree is built: its box, children (TNode ids) and primitive range.
struct TNode {
    float lo[3], hi[3];
    int32_t kid[2];
    uint32_t first, count, depth, inner;
};

struct Split {
    int how, axis, bin;
    uint32_t left;
};

struct State {
    float4 *plo, *phi, *pc;        // per occluder: box and centroid
    uint32_t *idx, *tmp;           // position -> occluder
    TNode *nodes;
    uint32_t *node_count, *max_depth, *error;
    Task *small;
    uint32_t *small_count;
};

// ---- primitives ----------------------------------------------------------------------------

__global__ void k_prims(DeviceBvhInput in, State st) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= in.occluders) return;
    uint32_t m = in.occ_mesh[i];
    const uint32_t *c = in.indices + in.mesh_index_base[m] + (size_t)in.occ_tri[i] * 3;
    uint32_t vb = in.mesh_vertex_base[m];
    float x[3][3];
    for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) x[k][a] = in.positions[(size_t)(vb + c[k]) * 3 + a];
    float lo[3], hi[3], ce[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = bvh_min(x[0][a], bvh_min(x[1][a], x[2][a]));
        hi[a] = bvh_max(x[0][a], bvh_max(x[1][a], x[2][a]));
        ce[a] = (lo[a] + hi[a]) * 0.5f;
    }
    st.plo[i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    st.phi[i] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    st.pc[i] = make_float4(ce[0], ce[1], ce[2], 0.0f);
    st.idx[i] = i;
}

__device__ __forceinline__ float comp(const float4 &v, int a) { return a == 0 ? v.x : a == 1 ? v.y : v.z; }

// ---- large nodes ---------------------------------------------------------------------------

struct Level {
    const Task *tasks;
    uint32_t task_count;
    const uint32_t *blk_task, *blk_start;  // per block: task, first position
    const uint32_t *task_blk;              // per task: first block (task_count + 1 entries)
    int *bounds;                           // per task: lo, hi, clo, chi as ford images (12)
    int *bins;                             // per task: kBinWords
    Split *split;                          // per task
    uint32_t *blk_left;                    // per block: lefts, then their exclusive offset
    Task *next;
    uint32_t *next_count;
};

__global__ void k_level_init(Level lv) {
    uint32_t t = blockIdx.x;
    if (t >= lv.task_count) return;
    for (int j = threadIdx.x; j < 12; j += blockDim.x) {
        bool low = j < 3 || (j >= 6 && j < 9);
        lv.bounds[t * 12 + j] = ford(low ? INFINITY : -INFINITY);
    }
    for (int j = threadIdx.x; j < kBinWords; j += blockDim.x) {
        int w = j % 7;
        lv.bins[(size_t)t * kBinWords + j] = w == 0 ? 0 : ford(w <= 3 ? INFINITY : -INFINITY);
    }
}

__device__ __forceinline__ void block_range(const Level &lv, uint32_t &t, uint32_t &b, uint32_t &e) {
    t = lv.blk_task[blockIdx.x];
    b = lv.blk_start[blockIdx.x];
    const Task &k = lv.tasks[t];
    e = min(b + kChunk, k.first + k.count);
}

__global__ void __launch_bounds__(kThreads) k_level_bounds(State st, Level lv) {
    uint32_t t, b, e;
    block_range(lv, t, b, e);
    int v[12];
    for (int a = 0; a < 3; ++a) {
        v[a] = v[6 + a] = ford(INFINITY);
        v[3 + a] = v[9 + a] = ford(-INFINITY);
    }
    for (uint32_t p = b + threadIdx.x; p < e; p += blockDim.x) {
        uint32_t i = st.idx[p];
        float4 lo = st.plo[i], hi = st.phi[i], c = st.pc[i];
        for (int a = 0; a < 3; ++a) {
            v[a] = min(v[a], ford(comp(lo, a)));
            v[3 + a] = max(v[3 + a], ford(comp(hi, a)));
            v[6 + a] = min(v[6 + a], ford(comp(c, a)));
            v[9 + a] = max(v[9 + a], ford(comp(c, a)));
        }
    }
    __shared__ int part[kThreads / 32][12];
    uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (int j = 0; j < 12; ++j) {
        bool low = j < 3 || (j >= 6 && j < 9);
        int r = low ? __reduce_min_sync(0xFFFFFFFFu, v[j]) : __reduce_max_sync(0xFFFFFFFFu, v[j]);
        if (lane == 0) part[warp][j] = r;
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        int j = threadIdx.x;
        bool low = j < 3 || (j >= 6 && j < 9);
        int r = part[0][j];
        for (int w = 1; w < kThreads / 32; ++w) r = low ? min(r, part[w][j]) : max(r, part[w][j]);
        if (low) atomicMin(&lv.bounds[t * 12 + j], r);
        else atomicMax(&lv.bounds[t * 12 + j], r);
    }
}

// The centroid bounds of a node from its bounds images: clo, per-axis scale and use.
__device__ __forceinline__ void bin_setup(const int *bd, float clo[3], float kk[3], bool use[3]) {
    for (int a = 0; a < 3; ++a) {
        clo[a] = funord(bd[6 + a]);
        float ext = funord(bd[9 + a]) - clo[a];
        use[a] = ext > 0.0f;
        kk[a] = use[a] ? (float)kBvhBins / ext : 0.0f;
    }
}

// Adds primitive i to the bins `sb` (kBinWords ford images and counts, shared memory).
__device__ __forceinline__ void bin_add(const State &st, uint32_t i, const float clo[3], const float kk[3],
                                        const bool use[3], int *sb) {
    float4 lo = st.plo[i], hi = st.phi[i], c = st.pc[i];
    for (int a = 0; a < 3; ++a) {
        if (!use[a]) continue;
        int k = bvh_bin(comp(c, a), clo[a], kk[a]);
        int *w = sb + (a * kBvhBins + k) * 7;
        atomicAdd(w, 1);
        for (int j = 0; j < 3; ++j) {
            atomicMin(w + 1 + j, ford(comp(lo, j)));
            atomicMax(w + 4 + j, ford(comp(hi, j)));
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_level_bins(State st, Level lv) {
    uint32_t t, b, e;
    block_range(lv, t, b, e);
    __shared__ int sb[kBinWords];
    for (int j = threadIdx.x; j < kBinWords; j += blockDim.x) {
        int w = j % 7;
        sb[j] = w == 0 ? 0 : ford(w <= 3 ? INFINITY : -INFINITY);
    }
    float clo[3], kk[3];
    bool use[3];
    bin_setup(lv.bounds + t * 12, clo, kk, use);
    __syncthreads();
    for (uint32_t p = b + threadIdx.x; p < e; p += blockDim.x) bin_add(st, st.idx[p], clo, kk, use, sb);
    __syncthreads();
    int *g = lv.bins + (size_t)t * kBinWords;
    for (int j = threadIdx.x; j < kBinWords; j += blockDim.x) {
        int w = j % 7;
        if (w == 0) {
            if (sb[j]) atomicAdd(g + j, sb[j]);
        } else if (w <= 3) {
            atomicMin(g + j, sb[j]);
        } else {
            atomicMax(g + j, sb[j]);
        }
    }
}

// Reads bins images into a BvhBins (floats and counts).
__device__ void bins_decode(const int *w, BvhBins &out) {
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < kBvhBins; ++k) {
            const int *q = w + (a * kBvhBins + k) * 7;
            out.bc[a][k] = (uint32_t)q[0];
            for (int j = 0; j < 3; ++j) {
                out.bl[a][k][j] = funord(q[1 + j]);
                out.bh[a][k][j] = funord(q[4 + j]);
            }
        }
}

// The decision for node `id` (range first/count at depth) with box lo/hi; `binned` false for a
// leaf before binning, else the best split (cost, axis, bin) and the items left of it. Fills the
// TNode and, for a split, allocates both children.
__device__ Split decide_node(const State &st, uint32_t id, uint32_t first, uint32_t count, uint32_t depth,
                             const float lo[3], const float hi[3], bool binned, float cost, int axis, int bin,
                             uint32_t left) {
    TNode &n = st.nodes[id];
    for (int a = 0; a < 3; ++a) {
        n.lo[a] = lo[a];
        n.hi[a] = hi[a];
    }
    n.first = first;
    n.count = count;
    n.depth = depth;
    n.inner = 0;
    n.kid[0] = n.kid[1] = -1;
    atomicMax(st.max_depth, depth);
    Split s{kBvhLeaf, axis, bin, 0};
    if (!binned) return s;
    s.how = bvh_decide(count, depth, lo, hi, cost, axis);
    if (s.how == kBvhLeaf) return s;
    if (s.how == kBvhByBin) {
        s.left = left;
        if (left == 0 || left == count) s.how = kBvhByIndex;  // the partition leaves every item in place
    }
    if (s.how == kBvhByIndex) s.left = count / 2;
    uint32_t k0 = atomicAdd(st.node_count, 2u);
    n.inner = 1;
    n.kid[0] = (int32_t)k0;
    n.kid[1] = (int32_t)(k0 + 1);
    return s;
}

__global__ void k_level_split(State st, Level lv) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lv.task_count) return;
    const Task k = lv.tasks[t];
    const int *bd = lv.bounds + t * 12;
    float lo[3], hi[3], clo[3], kk[3];
    bool use[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = funord(bd[a]);
        hi[a] = funord(bd[3 + a]);
    }
    bin_setup(bd, clo, kk, use);
    BvhBins bins;
    bins_decode(lv.bins + (size_t)t * kBinWords, bins);
    float cost;
    int axis, bin;
    bvh_best_split(bins, use, cost, axis, bin);
    uint32_t left = 0;
    for (int j = 0; axis >= 0 && j <= bin; ++j) left += bins.bc[axis][j];
    Split s = decide_node(st, k.node, k.first, k.count, k.depth, lo, hi, !bvh_leaf_before_bins(k.count, k.depth),
                          cost, axis, bin, left);
    lv.split[t] = s;
    if (s.how == kBvhLeaf) return;
    const TNode &n = st.nodes[k.node];
    Task kids[2] = {{(uint32_t)n.kid[0], k.first, s.left, k.depth + 1},
                    {(uint32_t)n.kid[1], k.first + s.left, k.count - s.left, k.depth + 1}};
    for (const Task &c : kids) {
        if (c.count > kSmall) lv.next[atomicAdd(lv.next_count, 1u)] = c;
        else st.small[atomicAdd(st.small_count, 1u)] = c;
    }
}

// Left flag of the item at position p of a task split by bin.
__device__ __forceinline__ bool goes_left(const State &st, const Level &lv, uint32_t t, const Split &s, uint32_t p) {
    const int *bd = lv.bounds + t * 12;
    float clo = funord(bd[6 + s.axis]);
    float ext = funord(bd[9 + s.axis]) - clo;
    float k = (float)kBvhBins / ext;
    return bvh_bin(comp(st.pc[st.idx[p]], s.axis), clo, k) <= s.bin;
}

__global__ void __launch_bounds__(kThreads) k_level_count(State st, Level lv) {
    uint32_t t, b, e;
    block_range(lv, t, b, e);
    const Split s = lv.split[t];
    if (s.how != kBvhByBin) return;
    uint32_t n = 0;
    for (uint32_t p = b + threadIdx.x; p < e; p += blockDim.x) n += goes_left(st, lv, t, s, p) ? 1u : 0u;
    n = __reduce_add_sync(0xFFFFFFFFu, n);
    __shared__ uint32_t part[kThreads / 32];
    if ((threadIdx.x & 31u) == 0) part[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (int w = 0; w < kThreads / 32; ++w) total += part[w];
        lv.blk_left[blockIdx.x] = total;
    }
}

__global__ void k_level_offsets(Level lv) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lv.task_count || lv.split[t].how != kBvhByBin) return;
    uint32_t run = 0;
    for (uint32_t b = lv.task_blk[t]; b < lv.task_blk[t + 1]; ++b) {
        uint32_t n = lv.blk_left[b];
        lv.blk_left[b] = run;
        run += n;
    }
}

// Stable scatter of a block's items: lefts after the lefts of earlier blocks, rights after all
// lefts and the rights of earlier blocks.
__global__ void __launch_bounds__(kThreads) k_level_scatter(State st, Level lv) {
    uint32_t t, b, e;
    block_range(lv, t, b, e);
    const Split s = lv.split[t];
    if (s.how != kBvhByBin) return;
    const Task k = lv.tasks[t];
    uint32_t lefts = lv.blk_left[blockIdx.x];  // lefts before this block
    uint32_t rights = (b - k.first) - lefts;
    __shared__ uint32_t wl[kThreads / 32];
    uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t base = b; base < e; base += blockDim.x) {
        uint32_t p = base + threadIdx.x;
        bool valid = p < e;
        bool left = valid && goes_left(st, lv, t, s, p);
        unsigned bl = __ballot_sync(0xFFFFFFFFu, left), bv = __ballot_sync(0xFFFFFFFFu, valid);
        if (lane == 0) wl[warp] = __popc(bl);
        __syncthreads();
        uint32_t before_l = 0;
        for (uint32_t w = 0; w < warp; ++w) before_l += wl[w];
        const uint32_t before_v = warp * 32;  // every earlier warp's items are valid when this one has any
        unsigned below = (1u << lane) - 1u;
        uint32_t rank_l = before_l + __popc(bl & below);
        uint32_t rank_r = (before_v - before_l) + __popc(bv & ~bl & below);
        if (valid) {
            uint32_t v = st.idx[p];
            if (left) st.tmp[k.first + lefts + rank_l] = v;
            else st.tmp[k.first + s.left + rights + rank_r] = v;
        }
        uint32_t round_l = 0;
        for (uint32_t w = 0; w < kThreads / 32; ++w) round_l += wl[w];
        uint32_t round_v = min((uint32_t)blockDim.x, e - base);
        lefts += round_l;
        rights += round_v - round_l;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreads) k_level_copy(State st, Level lv) {
    uint32_t t, b, e;
    block_range(lv, t, b, e);
    if (lv.split[t].how != kBvhByBin) return;
    for (uint32_t p = b + threadIdx.x; p < e; p += blockDim.x) st.idx[p] = st.tmp[p];
}

// ---- small nodes: a warp per subtree -------------------------------------------------------

// bvh_best_split over the bins images `sb` by a whole warp: lane k < kBvhBins of each used axis
// holds bin k, shuffle scans give the exact unions left of and right of every split, and the
// cheapest split wins with ties to the lowest (axis, bin), the order of the sequential sweep.
// Every lane returns the same cost, axis, bin and left count.
__device__ void warp_best_split(const int *sb, const bool use[3], float &best_cost, int &axis, int &bin,
                                uint32_t &left) {
    const unsigned all = 0xFFFFFFFFu;
    const int lane = (int)(threadIdx.x & 31u);
    const int k = lane & (kBvhBins - 1);
    float best = INFINITY;
    int key = 0x7FFFFFFF;  // axis * kBvhBins + bin of `best`
    uint32_t best_left = 0;
    for (int a = 0; a < 3; ++a) {
        if (!use[a]) continue;  // uniform
        const int *q = sb + (a * kBvhBins + k) * 7;
        uint32_t lc = (uint32_t)q[0], rc = lc;
        float ll[3], lh[3], rl[3], rh[3];
        for (int j = 0; j < 3; ++j) {
            ll[j] = rl[j] = funord(q[1 + j]);
            lh[j] = rh[j] = funord(q[4 + j]);
        }
        // inclusive scans within each half-warp: left over bins <= k, right over bins >= k
        for (int d = 1; d < kBvhBins; d <<= 1) {
            uint32_t c = __shfl_up_sync(all, lc, d, kBvhBins);
            uint32_t c2 = __shfl_down_sync(all, rc, d, kBvhBins);
            float t[12];
            for (int j = 0; j < 3; ++j) {
                t[j] = __shfl_up_sync(all, ll[j], d, kBvhBins);
                t[3 + j] = __shfl_up_sync(all, lh[j], d, kBvhBins);
                t[6 + j] = __shfl_down_sync(all, rl[j], d, kBvhBins);
                t[9 + j] = __shfl_down_sync(all, rh[j], d, kBvhBins);
            }
            if (k >= d) {
                lc += c;
                for (int j = 0; j < 3; ++j) {
                    ll[j] = bvh_min(ll[j], t[j]);
                    lh[j] = bvh_max(lh[j], t[3 + j]);
                }
            }
            if (k + d < kBvhBins) {
                rc += c2;
                for (int j = 0; j < 3; ++j) {
                    rl[j] = bvh_min(rl[j], t[6 + j]);
                    rh[j] = bvh_max(rh[j], t[9 + j]);
                }
            }
        }
        // the right side of split k is the suffix starting at bin k + 1
        uint32_t rcn = __shfl_down_sync(all, rc, 1, kBvhBins);
        float r1[6];
        for (int j = 0; j < 3; ++j) {
            r1[j] = __shfl_down_sync(all, rl[j], 1, kBvhBins);
            r1[3 + j] = __shfl_down_sync(all, rh[j], 1, kBvhBins);
        }
        if (lane < kBvhBins && k < kBvhBins - 1 && lc && rcn) {
            float c = bvh_half_area(ll, lh) * (float)lc + bvh_half_area(r1, r1 + 3) * (float)rcn;
            if (c < best) {  // per lane, one candidate per axis: axes in order keep the first
                best = c;
                key = a * kBvhBins + k;
                best_left = lc;
            }
        }
    }
    // warp argmin over (cost, key)
    for (int d = 16; d >= 1; d >>= 1) {
        float ob = __shfl_xor_sync(all, best, d);
        int ok = __shfl_xor_sync(all, key, d);
        uint32_t ol = __shfl_xor_sync(all, best_left, d);
        if (ob < best || (ob == best && ok < key)) {
            best = ob;
            key = ok;
            best_left = ol;
        }
    }
    best_cost = best;
    if (key == 0x7FFFFFFF) {
        axis = -1;
        bin = 0;
        left = 0;
    } else {
        axis = key / kBvhBins;
        bin = key % kBvhBins;
        left = best_left;
    }
}

constexpr int kSmallWarps = 4;

__global__ void __launch_bounds__(32 * kSmallWarps) k_small(State st, uint32_t count) {
    __shared__ int sbins[kSmallWarps][kBinWords];
    __shared__ uint32_t sstack[kSmallWarps][kWarpStack];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t w = blockIdx.x * kSmallWarps + warp;
    if (w >= count) return;  // warp-uniform
    int *sb = sbins[warp];
    uint32_t *stack = sstack[warp];
    const Task root = st.small[w];
    // a pending node's range and depth travel in its TNode
    if (lane == 0) {
        TNode &n = st.nodes[root.node];
        n.first = root.first;
        n.count = root.count;
        n.depth = root.depth;
        stack[0] = root.node;
    }
    __syncwarp();
    int sp = 1;
    const unsigned all = 0xFFFFFFFFu;
    while (sp > 0) {
        uint32_t id = stack[--sp];
        __syncwarp();
        const uint32_t first = st.nodes[id].first, cnt = st.nodes[id].count, depth = st.nodes[id].depth;
        const uint32_t end = first + cnt;
        int v[12];
        for (int a = 0; a < 3; ++a) {
            v[a] = v[6 + a] = ford(INFINITY);
            v[3 + a] = v[9 + a] = ford(-INFINITY);
        }
        for (uint32_t p = first + lane; p < end; p += 32) {
            uint32_t i = st.idx[p];
            float4 lo = st.plo[i], hi = st.phi[i], c = st.pc[i];
            for (int a = 0; a < 3; ++a) {
                v[a] = min(v[a], ford(comp(lo, a)));
                v[3 + a] = max(v[3 + a], ford(comp(hi, a)));
                v[6 + a] = min(v[6 + a], ford(comp(c, a)));
                v[9 + a] = max(v[9 + a], ford(comp(c, a)));
            }
        }
        for (int j = 0; j < 12; ++j) {
            bool low = j < 3 || (j >= 6 && j < 9);
            v[j] = low ? __reduce_min_sync(all, v[j]) : __reduce_max_sync(all, v[j]);
        }
        float lo[3], hi[3], clo[3], kk[3];
        bool use[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = funord(v[a]);
            hi[a] = funord(v[3 + a]);
        }
        bin_setup(v, clo, kk, use);
        const bool binned = !bvh_leaf_before_bins(cnt, depth);
        if (binned) {
            for (int j = lane; j < kBinWords; j += 32) {
                int q = j % 7;
                sb[j] = q == 0 ? 0 : ford(q <= 3 ? INFINITY : -INFINITY);
            }
            __syncwarp();
            for (uint32_t p = first + lane; p < end; p += 32) bin_add(st, st.idx[p], clo, kk, use, sb);
            __syncwarp();
        }
        float cost = INFINITY;
        int axis = -1, bin = 0;
        uint32_t left = 0;
        if (binned) warp_best_split(sb, use, cost, axis, bin, left);
        Split s{kBvhLeaf, -1, 0, 0};
        if (lane == 0) s = decide_node(st, id, first, cnt, depth, lo, hi, binned, cost, axis, bin, left);
        s.how = __shfl_sync(all, s.how, 0);
        s.axis = __shfl_sync(all, s.axis, 0);
        s.bin = __shfl_sync(all, s.bin, 0);
        s.left = __shfl_sync(all, s.left, 0);
        __syncwarp();
        if (s.how == kBvhLeaf) continue;
        if (s.how == kBvhByBin) {
            // stable partition through tmp, 32 items a round
            uint32_t lefts = 0, rights = 0;
            for (uint32_t base = first; base < end; base += 32) {
                uint32_t p = base + lane;
                bool valid = p < end;
                uint32_t item = valid ? st.idx[p] : 0u;
                bool left = valid && bvh_bin(comp(st.pc[item], s.axis), clo[s.axis], kk[s.axis]) <= s.bin;
                unsigned bl = __ballot_sync(all, left), bv = __ballot_sync(all, valid);
                unsigned below = (1u << lane) - 1u;
                if (valid) {
                    if (left) st.tmp[first + lefts + __popc(bl & below)] = item;
                    else st.tmp[first + s.left + rights + __popc(bv & ~bl & below)] = item;
                }
                lefts += __popc(bl);
                rights += __popc(bv & ~bl);
            }
            __syncwarp();
            for (uint32_t p = first + lane; p < end; p += 32) st.idx[p] = st.tmp[p];
            __syncwarp();
        }
        if (lane == 0) {
            const TNode &n = st.nodes[id];
            uint32_t k0 = (uint32_t)n.kid[0], k1 = (uint32_t)n.kid[1];
            TNode &a = st.nodes[k0];
            a.first = first;
            a.count = s.left;
            a.depth = depth + 1;
            TNode &b = st.nodes[k1];
            b.first = first + s.left;
            b.count = cnt - s.left;
            b.depth = depth + 1;
            if (sp + 2 <= kWarpStack) {
                stack[sp] = k1;  // the left child comes off first
                stack[sp + 1] = k0;
            } else {
                atomicExch(st.error, 1u);
            }
        }
        sp += 2;
        if (sp > kWarpStack) return;  // warp-uniform; the host reports the overflow
        __syncwarp();
    }
}

// ---- depth-first layout --------------------------------------------------------------------

struct Layout {
    const TNode *nodes;
    uint32_t total;  // TNodes
    uint32_t *size;  // inner nodes in the subtree of an inner node
    uint32_t *pos;   // depth-first position of an inner node
};

__global__ void k_sizes(Layout L, uint32_t depth) {
    uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= L.total) return;
    const TNode &n = L.nodes[id];
    if (n.depth != depth || !n.inner) return;
    uint32_t s = 1;
    for (int c = 0; c < 2; ++c)
        if (L.nodes[n.kid[c]].inner) s += L.size[n.kid[c]];
    L.size[id] = s;
}

__global__ void k_positions(Layout L, uint32_t depth) {
    uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= L.total) return;
    const TNode &n = L.nodes[id];
    if (n.depth != depth || !n.inner) return;
    uint32_t p = L.pos[id];
    const TNode &l = L.nodes[n.kid[0]];
    if (l.inner) L.pos[n.kid[0]] = p + 1;
    if (L.nodes[n.kid[1]].inner) L.pos[n.kid[1]] = p + 1 + (l.inner ? L.size[n.kid[0]] : 0u);
}

__device__ __forceinline__ int32_t child_ref(const Layout &L, int32_t kid) {
    const TNode &c = L.nodes[kid];
    return c.inner ? (int32_t)L.pos[kid] : ~(int32_t)((c.first << 3) | c.count);
}

__global__ void k_emit(Layout L, BvhNode *out) {
    uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= L.total) return;
    const TNode &n = L.nodes[id];
    if (id == 0 && !n.inner) {
        // the whole set is one leaf: the root holds it and an empty second child
        float lo[3] = {n.lo[0], n.lo[1], n.lo[2]}, hi[3] = {n.hi[0], n.hi[1], n.hi[2]};
        bvh_pad_box(lo, hi);
        BvhNode r{};
        r.c0[0] = lo[0]; r.c0[1] = hi[0]; r.c0[2] = lo[1]; r.c0[3] = hi[1];
        r.c1[0] = 1e30f; r.c1[1] = -1e30f; r.c1[2] = 1e30f; r.c1[3] = -1e30f;
        r.c2[0] = lo[2]; r.c2[1] = hi[2]; r.c2[2] = 1e30f; r.c2[3] = -1e30f;
        r.ref[0] = ~(int32_t)((n.first << 3) | n.count);
        r.ref[1] = ~0;
        out[0] = r;
        return;
    }
    if (!n.inner) return;
    const TNode &l = L.nodes[n.kid[0]], &r = L.nodes[n.kid[1]];
    float llo[3] = {l.lo[0], l.lo[1], l.lo[2]}, lhi[3] = {l.hi[0], l.hi[1], l.hi[2]};
    float rlo[3] = {r.lo[0], r.lo[1], r.lo[2]}, rhi[3] = {r.hi[0], r.hi[1], r.hi[2]};
    bvh_pad_box(llo, lhi);
    bvh_pad_box(rlo, rhi);
    BvhNode b{};
    b.c0[0] = llo[0]; b.c0[1] = lhi[0]; b.c0[2] = llo[1]; b.c0[3] = lhi[1];
    b.c1[0] = rlo[0]; b.c1[1] = rhi[0]; b.c1[2] = rlo[1]; b.c1[3] = rhi[1];
    b.c2[0] = llo[2]; b.c2[1] = lhi[2]; b.c2[2] = rlo[2]; b.c2[3] = rhi[2];
    b.ref[0] = child_ref(L, n.kid[0]);
    b.ref[1] = child_ref(L, n.kid[1]);
    out[L.pos[id]] = b;
}

// Triangles in leaf order: v0 (occluder index bits in w), e1 = v1 - v0, e2 = v2 - v0.
__global__ void k_leaf_triangles(DeviceBvhInput in, const uint32_t *idx, DeviceBvh out) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= in.occluders) return;
    uint32_t i = idx[k];
    uint32_t m = in.occ_mesh[i];
    const uint32_t *c = in.indices + in.mesh_index_base[m] + (size_t)in.occ_tri[i] * 3;
    uint32_t vb = in.mesh_vertex_base[m];
    f3 v[3];
    for (int j = 0; j < 3; ++j) {
        const float *q = in.positions + (size_t)(vb + c[j]) * 3;
        v[j] = f3{q[0], q[1], q[2]};
    }
    f3 e1 = sub(v[1], v[0]), e2 = sub(v[2], v[0]);
    float4 *t = out.tris + (size_t)k * 3;
    t[0] = make_float4(v[0].x, v[0].y, v[0].z, __uint_as_float(i));
    t[1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
    t[2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
    out.occ_leaf[i] = k;
}

uint32_t blocks_for(uint64_t n, uint32_t threads) { return (uint32_t)std::max<uint64_t>(1, (n + threads - 1) / threads); }

// Scratch device memory from the stream-ordered pool, freed on the build's stream when it ends,
// counted against the caller's device-memory cap.
struct Scratch {
    cudaStream_t stream;
    uint64_t *budget_held;
    uint64_t cap;
    std::vector<void *> held;
    uint64_t bytes = 0;
    template <class T>
    T *get(size_t n) {
        const size_t b = std::max<size_t>(n * sizeof(T), 16);
        if (budget_held && cap && *budget_held + b > cap)
            throw DeviceBvhError{cudaErrorMemoryAllocation, "device memory cap (BVH build scratch)"};
        void *p = nullptr;
        BK(cudaMallocAsync(&p, b, stream));
        held.push_back(p);
        bytes += b;
        if (budget_held) *budget_held += b;
        return static_cast<T *>(p);
    }
    ~Scratch() {
        for (void *p : held) cudaFreeAsync(p, stream);
        if (budget_held) *budget_held -= std::min(*budget_held, bytes);
    }
};

}  // namespace

void build_bvh_device(const DeviceBvhInput &in, const std::function<void *(size_t)> &alloc, cudaStream_t stream,
                      DeviceBvh &out) {
    const uint32_t n = in.occluders;
    out = DeviceBvh{};
    if (n == 0) return;
    Scratch sc{stream, in.held, in.cap, {}};
    State st;
    st.plo = sc.get<float4>(n);
    st.phi = sc.get<float4>(n);
    st.pc = sc.get<float4>(n);
    st.idx = sc.get<uint32_t>(n);
    st.tmp = sc.get<uint32_t>(n);
    const uint32_t cap = 2 * n;  // a binary tree over n leaves of >= 1 primitive has < 2n nodes
    st.nodes = sc.get<TNode>(cap);
    uint32_t *counters = sc.get<uint32_t>(4);
    st.node_count = counters;
    st.max_depth = counters + 1;
    st.error = counters + 2;
    st.small_count = counters + 3;
    st.small = sc.get<Task>(n);
    const uint32_t one[4] = {1, 0, 0, 0};  // the root is TNode 0
    BK(cudaMemcpyAsync(counters, one, sizeof one, cudaMemcpyHostToDevice, stream));
    k_prims<<<blocks_for(n, kThreads), kThreads, 0, stream>>>(in, st);
    BLAUNCHED("k_prims (bvh)");

    // large levels
    const uint32_t max_tasks = n / kSmall + 2;
    const uint32_t max_blocks = n / kChunk + 2 * max_tasks + 2;
    Task *tasks[2] = {sc.get<Task>(max_tasks), sc.get<Task>(max_tasks)};
    Level lv{};
    lv.bounds = sc.get<int>((size_t)max_tasks * 12);
    lv.bins = sc.get<int>((size_t)max_tasks * kBinWords);
    lv.split = sc.get<Split>(max_tasks);
    lv.blk_left = sc.get<uint32_t>(max_blocks);
    uint32_t *blk = sc.get<uint32_t>(2 * (size_t)max_blocks + max_tasks + 1);
    uint32_t *next_count = sc.get<uint32_t>(1);
    std::vector<Task> host_tasks;
    if (n > kSmall) {
        host_tasks.push_back(Task{0, 0, n, 1});
    } else {
        Task root{0, 0, n, 1};
        BK(cudaMemcpyAsync(st.small, &root, sizeof root, cudaMemcpyHostToDevice, stream));
        const uint32_t small_one = 1;
        BK(cudaMemcpyAsync(st.small_count, &small_one, 4, cudaMemcpyHostToDevice, stream));
    }
    std::vector<uint32_t> map;
    int cur = 0;
    while (!host_tasks.empty()) {
        const uint32_t T = (uint32_t)host_tasks.size();
        // block map: each task's positions in blocks of kChunk, tasks in order
        std::vector<uint32_t> btask, bstart, tblk(T + 1);
        for (uint32_t t = 0; t < T; ++t) {
            tblk[t] = (uint32_t)btask.size();
            for (uint32_t p = host_tasks[t].first; p < host_tasks[t].first + host_tasks[t].count; p += kChunk) {
                btask.push_back(t);
                bstart.push_back(p);
            }
        }
        tblk[T] = (uint32_t)btask.size();
        const uint32_t B = (uint32_t)btask.size();
        map.assign(btask.begin(), btask.end());
        map.insert(map.end(), bstart.begin(), bstart.end());
        map.insert(map.end(), tblk.begin(), tblk.end());
        BK(cudaMemcpyAsync(blk, map.data(), map.size() * 4, cudaMemcpyHostToDevice, stream));
        BK(cudaMemcpyAsync(tasks[cur], host_tasks.data(), T * sizeof(Task), cudaMemcpyHostToDevice, stream));
        BK(cudaMemsetAsync(next_count, 0, 4, stream));
        lv.tasks = tasks[cur];
        lv.task_count = T;
        lv.blk_task = blk;
        lv.blk_start = blk + B;
        lv.task_blk = blk + 2 * B;
        lv.next = tasks[cur ^ 1];
        lv.next_count = next_count;
        k_level_init<<<T, 128, 0, stream>>>(lv);
        k_level_bounds<<<B, kThreads, 0, stream>>>(st, lv);
        k_level_bins<<<B, kThreads, 0, stream>>>(st, lv);
        k_level_split<<<blocks_for(T, 128), 128, 0, stream>>>(st, lv);
        k_level_count<<<B, kThreads, 0, stream>>>(st, lv);
        k_level_offsets<<<blocks_for(T, 128), 128, 0, stream>>>(lv);
        k_level_scatter<<<B, kThreads, 0, stream>>>(st, lv);
        k_level_copy<<<B, kThreads, 0, stream>>>(st, lv);
        BLAUNCHED("large-node level (bvh)");
        uint32_t next = 0;
        BK(cudaMemcpyAsync(&next, next_count, 4, cudaMemcpyDeviceToHost, stream));
        BK(cudaStreamSynchronize(stream));
        host_tasks.resize(next);
        if (next) {
            BK(cudaMemcpyAsync(host_tasks.data(), tasks[cur ^ 1], next * sizeof(Task), cudaMemcpyDeviceToHost,
                               stream));
            BK(cudaStreamSynchronize(stream));
        }
        cur ^= 1;
    }

    // small subtrees
    uint32_t small = 0;
    BK(cudaMemcpyAsync(&small, st.small_count, 4, cudaMemcpyDeviceToHost, stream));
    BK(cudaStreamSynchronize(stream));
    if (small)
        k_small<<<blocks_for(small, kSmallWarps), 32 * kSmallWarps, 0, stream>>>(st, small);
    BLAUNCHED("k_small (bvh)");
    uint32_t c[4];
    BK(cudaMemcpyAsync(c, counters, sizeof c, cudaMemcpyDeviceToHost, stream));
    BK(cudaStreamSynchronize(stream));
    if (c[2]) {
        out.too_deep = true;
        return;
    }
    const uint32_t total = c[0];
    out.depth = c[1];

    // depth-first layout
    Layout L{st.nodes, total, sc.get<uint32_t>(total), sc.get<uint32_t>(total)};
    const uint32_t g = blocks_for(total, kThreads);
    for (uint32_t d = out.depth; d >= 1; --d) k_sizes<<<g, kThreads, 0, stream>>>(L, d);
    BK(cudaMemsetAsync(L.pos, 0, 4, stream));  // the root at 0
    for (uint32_t d = 1; d < out.depth; ++d) k_positions<<<g, kThreads, 0, stream>>>(L, d);
    BLAUNCHED("k_sizes/k_positions (bvh)");
    TNode root;
    BK(cudaMemcpyAsync(&root, st.nodes, sizeof root, cudaMemcpyDeviceToHost, stream));
    uint32_t inner = 1;
    BK(cudaStreamSynchronize(stream));
    if (root.inner) {
        BK(cudaMemcpyAsync(&inner, L.size, 4, cudaMemcpyDeviceToHost, stream));
        BK(cudaStreamSynchronize(stream));
    }
    out.node_count = inner;
    out.nodes = static_cast<BvhNode *>(alloc((size_t)inner * sizeof(BvhNode)));
    out.tris = static_cast<float4 *>(alloc((size_t)n * 3 * sizeof(float4)));
    out.occ_leaf = static_cast<uint32_t *>(alloc((size_t)n * 4));
    k_emit<<<g, kThreads, 0, stream>>>(L, out.nodes);
    k_leaf_triangles<<<blocks_for(n, kThreads), kThreads, 0, stream>>>(in, st.idx, out);
    BLAUNCHED("k_emit/k_leaf_triangles (bvh)");
    BK(cudaStreamSynchronize(stream));
}

}  // namespace dl
