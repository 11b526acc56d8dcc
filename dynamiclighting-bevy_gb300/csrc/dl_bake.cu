// The bake pipeline on one GPU and the C ABI (include/dynlight.h).
//
// Stages, all on one stream, each a kernel over the whole scene (every mesh at once):
//   setup      per triangle: face normal, crop rect, light association (mesh_bake.rs:141-173)
//   regions    per (mesh, light): union of crop rects -> one shadow grid (mesh_bake.rs:175-192)
//   texels     per triangle: owned grid, centered + touched texels (texels.rs, mesh_texels.rs)
//   burial     per texel: <= 8 closest-hit rays (mesh_texels.rs:57-88,111-135)
//   visibility per (pair, texel): point/area/sun/sky shadow rays (mesh_bake.rs:203-267)
//              batched: one persistent kernel over a device work queue, from a CUDA graph;
//              plain: one launch per mesh, a warp per triangle, lanes over texels
//   optimize   per triangle: drop lights with no lit texel nearby (shadows.rs:54-73)
//   seams      per region: pad unvisited texels (seams.rs:15-39)
//   serialize  per triangle/entry: header words, light data, cropped and dilated shadow words
//              (shadows.rs:87-159, seams.rs:43-71, triangle_words.rs:47-89)
// Sizes that decide later allocations are read back between stages (a handful of 8-byte copies).
#include <cub/cub.cuh>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "dl_bvh.hpp"
#include "dl_kernels.cuh"

namespace dl {

constexpr int kBlock = 128;
constexpr uint32_t kNoRect = 0xFFFFFFFFu;
constexpr uint64_t kBurialStream = 0x627572696564ull;  // mesh_texels.rs:26

struct Counters {
    unsigned long long rays, burial_rays, lights_removed, bounce_rays, photon_rays, cancelled;
    unsigned long long node_visits, tri_tests;  // instrumented visibility kernel only
    unsigned long long retests;                 // refined form: binary64 re-tests
    unsigned long long gather_node_visits, gather_tri_tests;  // instrumented gather kernel only
};

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    return v;
}
// Adds a whole warp's re-test counts to the counters (every lane calls it).
__device__ __forceinline__ void add_retests(Counters *ctr, unsigned long long n) {
    unsigned long long w = warp_sum(n);
    if (lane_id() == 0 && w) atomicAdd(&ctr->retests, w);
}

// ================================ setup and association ==================================

__global__ void k_setup(DevScene sc, float4 *tri_face, uint4 *tri_crop, uint32_t *tri_count) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sc.triangles) return;
    TriData d;
    load_tri(sc, t, d);
    f3 face = normalize_or_zero(cross(sub(d.v[1], d.v[0]), sub(d.v[2], d.v[0])));
    uint32_t count = 0;
    associate(sc, d, face, [&](uint32_t) { ++count; });
    Rect c = crop_rect(d.uv, d.res);
    tri_face[t] = make_float4(face.x, face.y, face.z, is_zero(face) ? 0.0f : 1.0f);
    tri_crop[t] = make_uint4(c.min_x, c.min_y, c.max_x, c.max_y);
    tri_count[t] = count;
}

__global__ void k_assoc_fill(DevScene sc, const float4 *tri_face, const uint4 *tri_crop, const uint32_t *tri_off,
                             uint32_t *pair_light, uint32_t *pair_tri, uint32_t *region_rect) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sc.triangles) return;
    TriData d;
    load_tri(sc, t, d);
    float4 f = tri_face[t];
    uint4 c = tri_crop[t];
    uint32_t p = tri_off[t];
    associate(sc, d, f3{f.x, f.y, f.z}, [&](uint32_t s) {
        pair_light[p] = s;
        pair_tri[p] = t;
        ++p;
        uint32_t *r = region_rect + ((size_t)d.mesh * sc.light_count + s) * 4;
        atomicMin(r, c.x);
        atomicMin(r + 1, c.y);
        atomicMax(r + 2, c.z);
        atomicMax(r + 3, c.w);
    });
}

__global__ void k_fill_u32(uint32_t *p, size_t n, uint32_t a, uint32_t b) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (i & 2) ? b : a;  // 4-word records (a, a, b, b)
}

// Words of each (mesh, light) region grid: bits for 1-bit lights, one byte per texel else.
__global__ void k_region_words(const uint32_t *region_rect, const DevLight *lights, uint32_t entries, uint32_t L,
                               uint32_t *words) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e > entries) return;
    if (e == entries) {
        words[e] = 0;
        return;
    }
    const uint32_t *r = region_rect + (size_t)e * 4;
    if (r[0] == kNoRect) {
        words[e] = 0;
        return;
    }
    uint64_t n = (uint64_t)(r[2] - r[0] + 1) * (r[3] - r[1] + 1);
    words[e] = lights[e % L].shadow_bits == 1 ? (uint32_t)((n + 31) / 32) : (uint32_t)((n + 3) / 4);
}

// ================================ texels ===============================================

// MODE 0: count centered texels and set the owned grid; MODE 1: count touched texels;
// MODE 2: write centered then touched texels at tex_off[t]. One warp per triangle.
template <int MODE>
__global__ void k_texels(DevScene sc, const float4 *tri_face, uint32_t *owned, const uint64_t *grid_off,
                         uint32_t *count, const uint32_t *tex_off, uint32_t *tex_xy, float4 *tex_pos, float4 *tex_nrm,
                         uint32_t *tex_tri) {
    uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    unsigned lane = lane_id();
    if (t >= sc.triangles) return;
    float4 f = tri_face[t];
    if (f.w == 0.0f) {
        if (MODE != 2 && lane == 0) count[t] = 0;
        return;
    }
    f3 face{f.x, f.y, f.z};
    TriData d;
    load_tri(sc, t, d);
    uint32_t res = d.res;
    uint32_t *own = owned + grid_off[d.mesh];
    uint32_t written = 0;
    uint32_t out = MODE == 2 ? tex_off[t] : 0;
    if (MODE == 0 || MODE == 2) {
        Rect r = center_rect(d.uv, res, 0.0f);
        uint32_t w = r.max_x - r.min_x + 1;
        uint64_t n = (uint64_t)w * (r.max_y - r.min_y + 1);
        for (uint64_t base = 0; base < n; base += 32) {
            uint64_t i = base + lane;
            bool inside = false;
            uint32_t x = 0, y = 0;
            f3 wts;
            if (i < n) {
                x = r.min_x + (uint32_t)(i % w);
                y = r.min_y + (uint32_t)(i / w);
                inside = uv_barycentrics(d.uv, texel_center(x, y, res), wts);
            }
            unsigned ballot = __ballot_sync(0xFFFFFFFFu, inside);
            if (inside) {
                if (MODE == 0) {
                    uint64_t bit = (uint64_t)x + (uint64_t)y * res;
                    atomicOr(own + bit / 32, 1u << (bit % 32));
                } else {
                    uint32_t o = out + written + __popc(ballot & ((1u << lane) - 1u));
                    f3 pos, nrm;
                    surface_at(d, face, wts, pos, nrm);
                    tex_xy[o] = x | (y << 16);
                    tex_pos[o] = make_float4(pos.x, pos.y, pos.z, 0.0f);
                    tex_nrm[o] = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
                    tex_tri[o] = t;
                }
            }
            written += __popc(ballot);
        }
        if (MODE == 0) {
            if (lane == 0) count[t] = written;
            return;
        }
    }
    // touched texels (texels.rs:78-121)
    float s = (float)res;
    f2 mn, mx;
    uv_bounds(d.uv, mn, mx);
    uint32_t x0 = f2u(fmaxf(floorf(mn.x * s), 0.0f)), y0 = f2u(fmaxf(floorf(mn.y * s), 0.0f));
    uint32_t x1 = f2u(fminf(floorf(mx.x * s), s - 1.0f)), y1 = f2u(fminf(floorf(mx.y * s), s - 1.0f));
    float half = 0.5f / s;
    uint32_t touched = 0;
    if (x1 >= x0 && y1 >= y0) {
        uint32_t w = x1 - x0 + 1;
        uint64_t n = (uint64_t)w * (y1 - y0 + 1);
        for (uint64_t base = 0; base < n; base += 32) {
            uint64_t i = base + lane;
            bool take = false;
            uint32_t x = 0, y = 0;
            f3 wts;
            if (i < n) {
                x = x0 + (uint32_t)(i % w);
                y = y0 + (uint32_t)(i / w);
                uint64_t bit = (uint64_t)x + (uint64_t)y * res;
                bool is_owned = (own[bit / 32] >> (bit % 32)) & 1u;
                if (!is_owned) {
                    f2 center = texel_center(x, y, res);
                    if (nearest_weights(d.uv, center, wts)) {
                        float nx = d.uv[0].x * wts.x + d.uv[1].x * wts.y + d.uv[2].x * wts.z;
                        float ny = d.uv[0].y * wts.x + d.uv[1].y * wts.y + d.uv[2].y * wts.z;
                        take = fmaxf(fabsf(nx - center.x), fabsf(ny - center.y)) <= half;
                    }
                }
            }
            unsigned ballot = __ballot_sync(0xFFFFFFFFu, take);
            if (MODE == 2 && take) {
                uint32_t o = out + written + touched + __popc(ballot & ((1u << lane) - 1u));
                f3 pos, nrm;
                surface_at(d, face, wts, pos, nrm);
                tex_xy[o] = x | (y << 16);
                tex_pos[o] = make_float4(pos.x, pos.y, pos.z, 0.0f);
                tex_nrm[o] = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
                tex_tri[o] = t;
            }
            touched += __popc(ballot);
        }
    }
    if (MODE == 1 && lane == 0) count[t] = touched;
}

// Burial test per texel (mesh_texels.rs:57-88). Buried texels are dropped from tracing.
template <bool REFINE>
__global__ void __launch_bounds__(kBlock) k_burial(DevScene sc, uint32_t texels, const uint32_t *tex_xy,
                                                   const float4 *tex_pos, const uint32_t *tex_tri,
                                                   const float4 *tri_face, uint8_t *buried, Counters *ctr) {
    __shared__ int stack[kStack * kBlock];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t rays = 0;
    Visits vis{0, 0, 0};
    if (i < texels) {
        uint32_t t = tex_tri[i];
        uint32_t m = sc.tri_mesh[t];
        float4 f = tri_face[t], p = tex_pos[i];
        f3 normal{f.x, f.y, f.z};
        uint32_t xy = tex_xy[i];
        f3 origin = add(f3{p.x, p.y, p.z}, scale(normal, kRayOffset));
        Pcg rng = stream6(sc.seed, sc.mesh_id[m], kBurialStream, t - sc.mesh_tri_base[m], xy & 0xFFFFu, xy >> 16);
        float turn = rng.next_f32();
        buried[i] = is_buried<REFINE>(sc, normal, origin, turn, stack + threadIdx.x, kBlock, rays, &vis) ? 1 : 0;
    }
    unsigned r = __reduce_add_sync(0xFFFFFFFFu, rays);
    if (lane_id() == 0 && r) atomicAdd(&ctr->burial_rays, (unsigned long long)r);
    if (REFINE) add_retests(ctr, vis.retests);
}

__global__ void k_add_u32(const uint32_t *a, const uint32_t *b, uint32_t *c, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) c[i] = a[i] + b[i];
    if (i == n) c[i] = 0;
}


// Per triangle: how many of its texels are not buried (warp per triangle).
template <bool WRITE>
__global__ void k_unburied(uint32_t triangles, const uint32_t *tex_off, const uint8_t *buried, uint32_t *count,
                           const uint32_t *ctex_off, const uint32_t *tex_xy, const float4 *tex_pos,
                           const float4 *tex_nrm, uint32_t *c_xy, float4 *c_pos, float4 *c_nrm) {
    uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    unsigned lane = lane_id();
    if (t >= triangles) return;
    uint32_t b = tex_off[t], e = tex_off[t + 1];
    uint32_t kept = 0;
    uint32_t out = WRITE ? ctex_off[t] : 0;
    for (uint32_t base = b; base < e; base += 32) {
        uint32_t i = base + lane;
        bool keep = i < e && !buried[i];
        unsigned ballot = __ballot_sync(0xFFFFFFFFu, keep);
        if (WRITE && keep) {
            uint32_t o = out + kept + __popc(ballot & ((1u << lane) - 1u));
            c_xy[o] = tex_xy[i];
            c_pos[o] = tex_pos[i];
            c_nrm[o] = tex_nrm[i];
        }
        kept += __popc(ballot);
    }
    if (!WRITE && lane == 0) count[t] = kept;
}

// ================================ visibility ===========================================

struct TraceArgs {
    const uint32_t *pair_tri, *pair_light;
    const uint32_t *ctex_off, *ctex_xy;
    const float4 *ctex_pos, *ctex_nrm, *tri_face;
    const uint64_t *grid_off;  // visited grid word offset per mesh
    uint32_t *visited;
    const uint32_t *region_rect, *region_off;
    uint32_t *region_pool;
    Counters *ctr;
    // batched queue: items of sky pairs first, then soft, then hard
    const uint32_t *order, *item_off;
    uint32_t pairs;
    unsigned long long items;
    unsigned long long *head;      // chunks claimed in the per-lane phase
    unsigned long long *head_sky;  // chunks claimed in the grouped sky phase
    const volatile uint32_t *cancel;
    uint32_t grab;         // warp-steps per claimed chunk
    uint32_t sky_items;    // items of the sky pairs at the front of the queue
    uint32_t sky_lanes;    // lanes sharing one sky texel's samples (1: no grouped phase)
    uint32_t sample_every; // tuning trials: claim one chunk in `sample_every` (1: all)
};

// The visibility result of (pair p, texel x, y of mesh m) into the visited grid and the light's
// region grid (mesh_bake.rs:231-248): a bit for 1-bit lights, an atomic max of the level otherwise.
__device__ __forceinline__ void store_texel(const DevScene &sc, const TraceArgs &a, uint32_t m, uint32_t s,
                                            uint32_t x, uint32_t y, uint32_t level, uint32_t bits) {
    uint32_t res = sc.mesh_res[m];
    uint64_t bit = (uint64_t)x + (uint64_t)y * res;
    atomicOr(a.visited + a.grid_off[m] + bit / 32, 1u << (bit % 32));
    size_t e = (size_t)m * sc.light_count + s;
    const uint32_t *r = a.region_rect + e * 4;
    uint32_t w = r[2] - r[0] + 1;
    uint64_t idx = (uint64_t)(x - r[0]) + (uint64_t)(y - r[1]) * w;
    uint32_t *g = a.region_pool + a.region_off[e];
    if (bits == 1) {
        if (level) atomicOr(g + idx / 32, 1u << (idx % 32));
    } else if (level) {
        uint32_t *word = g + idx / 4;
        uint32_t shift = (uint32_t)(idx % 4) * 8;
        uint32_t cur = *word;
        for (;;) {
            if (((cur >> shift) & 0xFFu) >= level) break;
            uint32_t want = (cur & ~(0xFFu << shift)) | (level << shift);
            uint32_t prev = atomicCAS(word, cur, want);
            if (prev == cur) break;
            cur = prev;
        }
    }
}

// One (pair, texel) of the visibility loop (mesh_bake.rs:231-248); returns the rays traced.
template <bool COUNT = false, bool REFINE = false>
__device__ __forceinline__ uint32_t trace_texel(const DevScene &sc, const TraceArgs &a, uint32_t p, uint32_t k,
                                                int *stack, int stride, Visits *vis = nullptr) {
    uint32_t t = a.pair_tri[p], s = a.pair_light[p];
    uint32_t m = sc.tri_mesh[t];
    uint32_t ci = a.ctex_off[t] + k;
    uint32_t xy = a.ctex_xy[ci];
    uint32_t x = xy & 0xFFFFu, y = xy >> 16;
    float4 pp = a.ctex_pos[ci], nn = a.ctex_nrm[ci], f = a.tri_face[t];
    f3 pos{pp.x, pp.y, pp.z}, nrm{nn.x, nn.y, nn.z};
    f3 origin = add(pos, scale(f3{f.x, f.y, f.z}, kRayOffset));
    const DevLight &l = sc.lights[s];
    Tracer<COUNT, REFINE> tr{sc, origin, (l.flags & kLightAlpha) != 0, stack, stride, vis};
    Vis v = texel_shadow(sc, s, sc.mesh_id[m], x, y, pos, nrm, tr);
    if (!v.some) return 0;
    store_texel(sc, a, m, s, x, y, v.level, l.shadow_bits);
    return v.rays;
}

// The pair holding queue item `item`: item_off[lo] <= item < item_off[lo + 1].
__device__ __forceinline__ uint32_t pair_of(const TraceArgs &a, unsigned long long item) {
    uint32_t lo = 0, hi = a.pairs;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if ((unsigned long long)a.item_off[mid] <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Whether a warp's lane 0 should stop claiming work: the cancel flag is read every 16th claim;
// once it is seen, the warp counts itself in `ctr->cancelled` and every later claim stops too.
constexpr uint32_t kStopped = 0x80000000u;
__device__ __forceinline__ bool cancel_seen(const volatile uint32_t *cancel, Counters *ctr, uint32_t &grabs) {
    if (grabs & kStopped) return true;
    if ((++grabs & 15u) == 0 && *cancel) {
        grabs |= kStopped;
        atomicAdd(&ctr->cancelled, 1ull);
        return true;
    }
    return false;
}

// Claims the next chunk of a queue phase for the warp: the first item of chunk c is
// first + c * size * sample_every. Returns `end` when the phase is drained or cancelled.
__device__ __forceinline__ unsigned long long claim(const TraceArgs &a, unsigned long long *head,
                                                    unsigned long long first, unsigned long long size,
                                                    unsigned long long end, uint32_t &grabs) {
    unsigned long long base = 0;
    if (lane_id() == 0) {
        if (cancel_seen(a.cancel, a.ctr, grabs)) {
            base = end;
        } else {
            unsigned long long c = atomicAdd(head, 1ull);
            base = first + c * size * a.sample_every;
            if (base > end) base = end;
        }
    }
    return __shfl_sync(0xFFFFFFFFu, base, 0);
}

// Batched form: persistent warps pull chunks of (pair, texel) items from one queue. Items are
// ordered sky pairs first, then soft, then hard, so the longest work starts first. The sky items
// run first in a grouped phase: W = sky_lanes lanes share one texel, each tracing every W-th rank
// of its samples in the shift-aligned coherent order, and the open counts are summed across the
// group (an integer sum, so the level is the same as one lane tracing them all in index order).
// MINB is the launch bound's blocks per SM (the register budget). The stack lives in dynamic
// shared memory.
template <bool COUNT, bool REFINE, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_trace_batched(DevScene sc, TraceArgs a) {
    extern __shared__ int stack[];
    int *my = stack + threadIdx.x;
    unsigned lane = lane_id();
    unsigned long long rays = 0;
    Visits vis{0, 0, 0};
    uint32_t grabs = 0;
    const uint32_t W = a.sky_lanes;
    unsigned long long first = 0;
    if (a.sky_items) {
        const uint32_t per_step = 32 / W, sub = lane % W;
        const unsigned long long end = a.sky_items;
        first = end;
        for (;;) {
            unsigned long long base = claim(a, a.head_sky, 0, (unsigned long long)per_step * a.grab, end, grabs);
            if (base >= end) break;
            uint32_t cur = pair_of(a, base);
            for (uint32_t g = 0; g < a.grab; ++g) {
                unsigned long long item = base + (unsigned long long)g * per_step + lane / W;
                bool valid = item < end;
                uint32_t open = 0, t = 0, s = 0, m = 0, x = 0, y = 0;
                if (valid) {
                    while ((unsigned long long)a.item_off[cur + 1] <= item) ++cur;
                    uint32_t p = a.order[cur];
                    t = a.pair_tri[p];
                    s = a.pair_light[p];
                    m = sc.tri_mesh[t];
                    uint32_t ci = a.ctex_off[t] + (uint32_t)(item - a.item_off[cur]);
                    uint32_t xy = a.ctex_xy[ci];
                    x = xy & 0xFFFFu;
                    y = xy >> 16;
                    float4 pp = a.ctex_pos[ci], nn = a.ctex_nrm[ci], f = a.tri_face[t];
                    f3 nrm{nn.x, nn.y, nn.z};
                    f3 origin = add(f3{pp.x, pp.y, pp.z}, scale(f3{f.x, f.y, f.z}, kRayOffset));
                    const DevLight &l = sc.lights[s];
                    Tracer<COUNT, REFINE> tr{sc, origin, (l.flags & kLightAlpha) != 0, my, kBlock, &vis};
                    // sky_visibility (sky.rs:30-44), samples sub, sub + W, ...
                    Pcg rng = stream5(sc.seed, sc.mesh_id[m], l.id, x, y);
                    f2 off;
                    off.x = rng.next_f32();
                    off.y = rng.next_f32();
                    f3 side, across;
                    ortho_pair(nrm, side, across);
                    // in the shift-aligned coherent order when the sample count allows it: the
                    // warp's texels (neighbours) then trace their rank-k rays in about one direction
                    const uint32_t n = sc.sky_samples;
                    const bool aligned = n >= 16 && n <= kMaxOrdered && !(n & (n - 1));
                    const uint32_t shift = aligned ? net_shift(n, off) : 0u;
                    for (uint32_t k = sub; k < n; k += W) {
                        uint32_t j = aligned ? shifted_sample(sc, n, shift, k) : sc.sky_order ? sc.sky_order[k] : k;
                        if (!tr(cosine_direction_basis(nrm, side, across, spread(j, off, true)), INFINITY)) ++open;
                    }
                }
                for (uint32_t o = 1; o < W; o <<= 1) open += __shfl_xor_sync(0xFFFFFFFFu, open, o);
                if (valid && sub == 0) {
                    uint32_t samples = sc.sky_samples;
                    float fraction = (float)open / (float)(samples > 1 ? samples : 1);
                    const DevLight &l = sc.lights[s];
                    store_texel(sc, a, m, s, x, y, level_of(fraction, l.shadow_bits), l.shadow_bits);
                    rays += samples;
                }
            }
        }
    }
    for (;;) {
        unsigned long long base = claim(a, a.head, first, 32ull * a.grab, a.items, grabs);
        if (base >= a.items) break;
        uint32_t cur = pair_of(a, base);  // per lane, advances monotonically over the chunk
        for (uint32_t g = 0; g < a.grab; ++g) {
            unsigned long long item = base + (unsigned long long)g * 32 + lane;
            if (item < a.items) {
                while ((unsigned long long)a.item_off[cur + 1] <= item) ++cur;
                rays += trace_texel<COUNT, REFINE>(sc, a, a.order[cur], (uint32_t)(item - a.item_off[cur]), my,
                                                   kBlock, &vis);
            }
        }
    }
    unsigned long long r = warp_sum(rays);
    if (lane == 0 && r) atomicAdd(&a.ctr->rays, r);
    if (COUNT) {
        unsigned long long n = warp_sum(vis.nodes), t = warp_sum(vis.tris);
        if (lane == 0) {
            atomicAdd(&a.ctr->node_visits, n);
            atomicAdd(&a.ctr->tri_tests, t);
        }
    }
    if (REFINE) add_retests(a.ctr, vis.retests);
}

// Plain form: one launch per mesh; a warp per triangle, its lights in order, lanes over texels.
__global__ void __launch_bounds__(kBlock) k_trace_plain(DevScene sc, TraceArgs a, uint32_t first_tri,
                                                         uint32_t tri_count, const uint32_t *tri_pair_off) {
    __shared__ int stack[kStack * kBlock];
    int *my = stack + threadIdx.x;
    unsigned lane = lane_id();
    unsigned long long rays = 0;
    uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < tri_count; w += warps) {
        uint32_t t = first_tri + w;
        uint32_t n = a.ctex_off[t + 1] - a.ctex_off[t];
        for (uint32_t p = tri_pair_off[t]; p < tri_pair_off[t + 1]; ++p)
            for (uint32_t k = lane; k < n; k += 32) rays += trace_texel(sc, a, p, k, my, kBlock);
    }
    unsigned long long r = warp_sum(rays);
    if (lane == 0 && r) atomicAdd(&a.ctr->rays, r);
}

// Queue construction: pairs in class order (sky, soft, hard) and their item prefix sums.
__global__ void k_pair_class(DevScene sc, const uint32_t *pair_light, uint32_t pairs, uint32_t cls, uint32_t *flag) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > pairs) return;
    if (p == pairs) {
        flag[p] = 0;
        return;
    }
    const DevLight &l = sc.lights[pair_light[p]];
    uint32_t c = l.shape == DL_SHAPE_SKY ? 0 : (l.shadow_bits > 1 ? 1 : 2);
    flag[p] = c == cls;
}
__global__ void k_pair_scatter(const uint32_t *flag, const uint32_t *pos, uint32_t pairs, uint32_t base,
                               uint32_t *order) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < pairs && flag[p]) order[base + pos[p]] = p;
}
__global__ void k_item_counts(const uint32_t *order, const uint32_t *pair_tri, const uint32_t *ctex_off,
                              uint32_t pairs, uint32_t *cnt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > pairs) return;
    if (i == pairs) {
        cnt[i] = 0;
        return;
    }
    uint32_t t = pair_tri[order[i]];
    cnt[i] = ctex_off[t + 1] - ctex_off[t];
}


// ================================ one bounce ===========================================

// PhotonCube::build (bounce.rs:48-70): every cube texel of every local bounce light.
template <bool REFINE>
__global__ void __launch_bounds__(kBlock) k_photons(DevScene sc, const uint32_t *cube_lights, uint32_t cubes,
                                                    uint32_t res, Photon *photons, Counters *ctr) {
    __shared__ int stack[kStack * kBlock];
    uint64_t per = 6ull * res * res;
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    Visits vis{0, 0, 0};
    if (i < per * cubes) {
        uint32_t cube = (uint32_t)(i / per);
        uint32_t rem = (uint32_t)(i % per);
        uint32_t face = rem / (res * res), y = (rem % (res * res)) / res, x = rem % res;
        const DevLight &l = sc.lights[cube_lights[cube]];
        photons[i] = make_photon<REFINE>(sc, l, cube_texel_direction(face, x, y, res), stack + threadIdx.x, kBlock,
                                         &vis);
    }
    if (REFINE) add_retests(ctr, vis.retests);
}

// Pairs whose light bakes bounce, in pair order.
__global__ void k_bounce_flag(DevScene sc, const uint32_t *pair_light, uint32_t pairs, uint32_t *flag) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > pairs) return;
    flag[p] = p < pairs && (sc.lights[pair_light[p]].flags & kLightBounce) ? 1u : 0u;
}

struct BounceArgs {
    const uint32_t *pair_tri, *pair_light;
    const uint32_t *ctex_off, *ctex_xy;
    const float4 *ctex_pos, *tri_face;
    const uint32_t *bpairs, *bitem_off;
    uint32_t bpair_count;
    unsigned long long items;
    const Photon *photons;
    uint32_t res;
    float4 *value;  // xyz: gathered value, w: 1 when gathered
    Counters *ctr;
    uint32_t lanes;         // lanes sharing one texel's samples (1, 2, 4, 8, 16 or 32)
    uint32_t sample_every;  // tuning trials: one claimed step in `sample_every` (1: all)
    uint32_t stack_depth;   // shared-memory stack entries per thread
    uint32_t buffered;      // sun samples a lane group can hold for the aligned order (0: none)
    float4 *scratch;        // per lane group (blockIdx * groups + group): 2 * buffered float4
    unsigned long long *head;  // steps claimed so far (32 / lanes items per step)
    const volatile uint32_t *cancel;  // the bake's cancel flag, read every 16th claim
};

// gather_triangle / gather_sun (bounce.rs:235-292, sun_bounce.rs:24-80): a group of `lanes`
// lanes per (bounce pair, texel) item. Each round, lane k of a group evaluates sample
// round * lanes + k; the group leader then adds the round's contributions in sample order, so
// the sum is the reference's sequential one for any group size.
// Sun gathers with a power-of-two sample count up to `buffered` take their samples in the
// shift-aligned coherent order instead (shifted_sample): round r of every group in the warp
// traces ranks r * lanes + k, so the warp's texels (neighbours along a triangle) send their rays
// in about the same directions. A sample whose closest hit faces the sun and is lit by it
// stores its value, its index and its shadow ray's origin in the next free slot of the group's
// scratch (global memory; slots are taken in arrival order, so a group touches only as many as
// it holds, a few lines that stay in L2) and sets its bit in the group's mask (shared memory).
// After the closest-hit rounds the group traces the held shadow rays together, W at a time
// (parallel rays towards the sun), marking blocked ones in a second mask; each open sample's
// value then moves to its rank among the open samples (popcounts of the masks), and the group
// loads those values W at a time while the leader adds them, in sample order, as the reference
// does (sun_bounce.rs:70). Dynamic shared memory holds only the traversal stacks and the groups'
// masks (the per-round contributions go to the leader by shuffles), so that the rest of each SM's
// unified L1/shared memory stays L1 cache for the BVH. MINB is the launch bound's blocks per SM
// (the register budget: 6, 8, 9 and 10 give 80, 64, 56 and 48 registers a thread).
template <bool COUNT, bool REFINE, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_gather(DevScene sc, BounceArgs a) {
    extern __shared__ int smem[];
    int *my = smem + threadIdx.x;
    const uint32_t lane = lane_id(), W = a.lanes, sub = lane % W, per_step = 32 / W;
    // this lane group's masks (shared memory: samples whose hit is lit, then those whose shadow
    // ray is blocked) and scratch (global memory) for aligned sun gathers
    const uint32_t group = (threadIdx.x >> 5) * per_step + lane / W, words = a.buffered / 32;
    const unsigned group_lanes = W == 32 ? 0xFFFFFFFFu : ((1u << W) - 1u) << (lane / W * W);
    uint32_t *lit = reinterpret_cast<uint32_t *>(smem + (size_t)a.stack_depth * kBlock) + (size_t)group * 2 * words;
    uint32_t *blocked = lit + words;
    float4 *scratch = a.scratch + ((size_t)blockIdx.x * (kBlock / W) + group) * 2 * a.buffered;
    for (uint32_t w = sub; w < 2 * words; w += W) lit[w] = 0u;
    __syncwarp();
    unsigned long long rays = 0;
    Visits vis{0, 0, 0};
    uint32_t grabs = 0;
    for (;;) {
        unsigned long long step = ~0ull;
        if (lane == 0 && !cancel_seen(a.cancel, a.ctr, grabs)) step = atomicAdd(a.head, 1ull);
        step = __shfl_sync(0xFFFFFFFFu, step, 0);
        if (step == ~0ull) break;  // cancelled (uniform across the warp)
        unsigned long long base = step * per_step * a.sample_every;
        if (base >= a.items) break;  // uniform across the warp
        unsigned long long item = base + lane / W;
        bool valid = item < a.items, active = false, sun = false;
        uint32_t samples = 0, s = 0;
        f3 pos{0, 0, 0}, normal{0, 0, 0}, origin{0, 0, 0};
        LocalGather lg;
        SunGather sg;
        if (valid) {
            uint32_t lo = 0, hi = a.bpair_count;
            while (hi - lo > 1) {
                uint32_t mid = (lo + hi) >> 1;
                if ((unsigned long long)a.bitem_off[mid] <= item) lo = mid;
                else hi = mid;
            }
            uint32_t p = a.bpairs[lo];
            uint32_t t = a.pair_tri[p];
            s = a.pair_light[p];
            uint32_t m = sc.tri_mesh[t];
            uint32_t ci = a.ctex_off[t] + (uint32_t)(item - a.bitem_off[lo]);
            uint32_t xy = a.ctex_xy[ci];
            float4 pp = a.ctex_pos[ci], f = a.tri_face[t];
            pos = f3{pp.x, pp.y, pp.z};
            normal = f3{f.x, f.y, f.z};
            origin = add(pos, scale(normal, kRayOffset));
            const DevLight &l = sc.lights[s];
            samples = l.bounce_samples;
            sun = l.shape == DL_SHAPE_SUN;
            if (sun) {
                sun_setup(sc, l, sc.mesh_id[m], xy & 0xFFFFu, xy >> 16, normal, sg);
                active = true;
            } else {
                active = local_setup(sc, l, sc.mesh_id[m], xy & 0xFFFFu, xy >> 16, pos, sub, lg);
            }
        }
        if (!active) samples = 0;
        const bool aligned = sun && samples >= 32 && samples <= a.buffered && !(samples & (samples - 1));
        const uint32_t shift = aligned ? net_shift(samples, sg.off) : 0u;
        FSum3<REFINE> sum;
        uint32_t filled = 0;  // aligned sun gathers: scratch slots filled so far (the same in the group)
        const uint32_t rounds = __reduce_max_sync(0xFFFFFFFFu, (samples + W - 1) / W);
        for (uint32_t r = 0; r < rounds; ++r) {
            const uint32_t k = r * W + sub;
            if (aligned) {
                SunHit h{f3{0.0f, 0.0f, 0.0f}, f3{0.0f, 0.0f, 0.0f}, false};
                uint32_t i = 0;
                if (k < samples) {
                    i = shifted_sample(sc, samples, shift, k);
                    h = sun_hit<COUNT, REFINE>(sc, sc.lights[s], origin, normal, sg, i, my, kBlock, &vis);
                    rays += h.pending ? 2 : 1;
                }
                // the group's pending samples of this round take the next slots, in lane order
                const unsigned mine = __ballot_sync(group_lanes, h.pending);
                if (h.pending) {
                    const uint32_t slot = filled + __popc(mine & ((1u << lane) - 1u));
                    scratch[2 * slot] = make_float4(h.value.x, h.value.y, h.value.z, __uint_as_float(i));
                    scratch[2 * slot + 1] = make_float4(h.point.x, h.point.y, h.point.z, 0.0f);
                    atomicOr(&lit[i >> 5], 1u << (i & 31u));
                }
                filled += __popc(mine);
                continue;  // no per-round sum: the phases below add the values in sample order
            }
            Contribution c{f3{0.0f, 0.0f, 0.0f}, false, 0};
            if (k < samples) {
                const DevLight &l = sc.lights[s];
                if (sun) {
                    c = sun_sample<COUNT, REFINE>(sc, l, origin, normal, sg, k, my, kBlock, &vis);
                } else {
                    Tracer<COUNT, REFINE> tr{sc, origin, (l.flags & kLightAlpha) != 0, my, kBlock, &vis};
                    c = local_sample(sc, l, a.photons + (size_t)l.cube * 6 * a.res * a.res, a.res, normal, lg, k, tr);
                    lg.rng.advance(2ull * (W - 1));  // to the lane's next sample, k + W
                }
                rays += c.rays;
            }
            // the leader adds the round's contributions in sample order, from the group's lanes
            const uint32_t lane0 = lane - sub, n = samples > r * W ? min(W, samples - r * W) : 0u;
            for (uint32_t j = 0; j < n; ++j) {
                const float x = __shfl_sync(group_lanes, c.value.x, lane0 + j);
                const float y = __shfl_sync(group_lanes, c.value.y, lane0 + j);
                const float z = __shfl_sync(group_lanes, c.value.z, lane0 + j);
                const int add = __shfl_sync(group_lanes, (int)c.add, lane0 + j);
                if (sub == 0 && add) sum.add(f3{x, y, z});
            }
        }
        __syncwarp();
        if (aligned) {
            // the shadow rays of the held samples, slot by slot across the group's lanes
            for (uint32_t j = sub; j < filled; j += W) {
                const float4 q = scratch[2 * j + 1];
                const uint32_t i = __float_as_uint(scratch[2 * j].w);
                if (!sun_open<COUNT, REFINE>(sc, sc.lights[s], f3{q.x, q.y, q.z}, my, kBlock, &vis))
                    atomicOr(&blocked[i >> 5], 1u << (i & 31u));
            }
        }
        __syncwarp();
        uint32_t open_count = 0;
        if (aligned) {
            // each open sample's value moves to its rank among the open samples in sample order
            // (into the shadow-ray origins' half of the slots, which is no longer read)
            for (uint32_t j = sub; j < filled; j += W) {
                const float4 v = scratch[2 * j];
                const uint32_t i = __float_as_uint(v.w), w = i >> 5, b = i & 31u;
                const uint32_t open = lit[w] & ~blocked[w];
                if ((open >> b) & 1u) {
                    uint32_t rank = __popc(open & ((1u << b) - 1u));
                    for (uint32_t u = 0; u < w; ++u) rank += __popc(lit[u] & ~blocked[u]);
                    scratch[2 * rank + 1] = v;
                }
            }
            for (uint32_t u = 0; u < samples / 32; ++u) open_count += __popc(lit[u] & ~blocked[u]);
        }
        __syncwarp();
        if (aligned) {
            // the group loads the ordered values W at a time; the leader adds them in order
            const uint32_t lane0 = lane - sub;
            for (uint32_t base = 0; base < open_count; base += W) {
                float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (base + sub < open_count) q = scratch[2 * (base + sub) + 1];
                const uint32_t n = min(W, open_count - base);
                for (uint32_t t = 0; t < n; ++t) {
                    const float x = __shfl_sync(group_lanes, q.x, lane0 + t);
                    const float y = __shfl_sync(group_lanes, q.y, lane0 + t);
                    const float z = __shfl_sync(group_lanes, q.z, lane0 + t);
                    if (sub == 0) sum.add(f3{x, y, z});
                }
            }
            for (uint32_t w = sub; w < 2 * words; w += W) lit[w] = 0u;  // lit, then blocked
        }
        __syncwarp();
        if (valid && sub == 0) {
            f3 v{0.0f, 0.0f, 0.0f};
            if (active) v = divs(scale(sum.value(), sc.lights[s].bounce_intensity), (float)samples);
            a.value[item] = make_float4(v.x, v.y, v.z, active ? 1.0f : 0.0f);
        }
    }
    unsigned long long total = warp_sum(rays);
    if (lane_id() == 0 && total) atomicAdd(&a.ctr->bounce_rays, total);
    if (COUNT) {
        unsigned long long n = warp_sum(vis.nodes), t = warp_sum(vis.tris);
        if (lane_id() == 0) {
            atomicAdd(&a.ctr->gather_node_visits, n);
            atomicAdd(&a.ctr->gather_tri_tests, t);
        }
    }
    if (REFINE) add_retests(a.ctr, vis.retests);
}

// ================================ maps for moving meshes =================================
// Baked when dynamic_geometry is not LightingOnly (src/bake/baker.rs:114-152).

constexpr uint32_t kCubeRes = 64;                     // DISTANCE_CUBE_RESOLUTION (distance_cubes.rs:22)
constexpr uint64_t kProbeStream = 0x736b7970726f6265ull;  // PROBE_STREAM (sky_probes.rs:22)

// bake_distance_cubes (distance_cubes.rs:29-75): one thread per word, texels 2w (low half) and
// 2w + 1 of face f of light l; a ray from the light's centre through the texel centre, its
// closest hit within the radius, else the radius, as f16.
template <bool REFINE>
__global__ void __launch_bounds__(kBlock) k_distance_cubes(DevScene sc, uint32_t lights, uint32_t *out,
                                                           Counters *ctr) {
    __shared__ int stack[kStack * kBlock];
    const uint32_t per_face = kCubeRes * kCubeRes / 2;
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    Visits vis{0, 0, 0};
    if (i < (uint64_t)lights * 6 * per_face) {
        uint32_t l = (uint32_t)(i / (6 * per_face)), face = (uint32_t)(i / per_face % 6), w = (uint32_t)(i % per_face);
        const DevLight &L = sc.lights[l];
        float d[2];
        for (uint32_t k = 0; k < 2; ++k) {
            uint32_t texel = 2 * w + k;
            f3 dir = cube_texel_direction(face, texel % kCubeRes, texel / kCubeRes, kCubeRes);
            Hit h;
            d[k] = traverse<false, false, REFINE>(sc, L.position, dir, L.radius, (L.flags & kLightAlpha) != 0,
                                                  stack + threadIdx.x, kBlock, h, &vis)
                       ? h.t
                       : L.radius;
        }
        out[i] = f16_bits(d[1]) << 16 | f16_bits(d[0]);
    }
    if (REFINE) add_retests(ctr, vis.retests);
}

// bake_sun_map (sun_map.rs:25-74): one thread per word (texels 2w and 2w + 1, rows of
// increasing y), a closest-hit ray along the sun's rays from the near plane, depth over the
// map's depth as unorm16; a miss (or the odd texel past the end) stores 1.
struct SunMapArgs {
    f3 side, up, along, bmin;
    float texel, depth;
    uint32_t res, words, alpha;
    uint32_t *out;
};
__device__ __forceinline__ uint32_t unorm16(float d) { return f2u(roundf(clampf(d, 0.0f, 1.0f) * 65535.0f)); }
template <bool REFINE>
__global__ void __launch_bounds__(kBlock) k_sun_map(DevScene sc, SunMapArgs a, Counters *ctr) {
    __shared__ int stack[kStack * kBlock];
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    Visits vis{0, 0, 0};
    if (w < a.words) {
        float d[2];
        for (uint32_t k = 0; k < 2; ++k) {
            uint32_t i = 2 * w + k;
            d[k] = 1.0f;
            if (i < a.res * a.res) {
                float across = a.bmin.x + ((float)(i % a.res) + 0.5f) * a.texel;
                float down = a.bmin.y + ((float)(i / a.res) + 0.5f) * a.texel;
                f3 origin = add(add(scale(a.side, across), scale(a.up, down)), scale(a.along, a.bmin.z));
                Hit h;
                if (traverse<false, false, REFINE>(sc, origin, a.along, a.depth, a.alpha != 0, stack + threadIdx.x,
                                                   kBlock, h, &vis))
                    d[k] = h.t / a.depth;
            }
        }
        a.out[w] = unorm16(d[1]) << 16 | unorm16(d[0]);
    }
    if (REFINE) add_retests(ctr, vis.retests);
}

// trace_probe (sky_probes.rs:83-109), one thread per (probe, axis): the sky samples around the
// axis, each a closest hit (a hit at distance 0 counts as none); the open share and the rays
// that reached a triangle's back.
struct ProbeArgs {
    f3 origin;
    float spacing;
    uint32_t cx, cy, alpha;
    unsigned long long jobs;  // probes * 6
    float *open;
    uint32_t *back;
};
template <bool REFINE>
__global__ void __launch_bounds__(kBlock) k_sky_probes(DevScene sc, ProbeArgs a, Counters *ctr) {
    __shared__ int stack[kStack * kBlock];
    unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    Visits vis{0, 0, 0};
    if (i < a.jobs) {
        uint64_t probe = i / 6;
        uint32_t axis = (uint32_t)(i % 6);
        uint32_t x = (uint32_t)(probe % a.cx), y = (uint32_t)(probe % ((uint64_t)a.cx * a.cy) / a.cx),
                 z = (uint32_t)(probe / ((uint64_t)a.cx * a.cy));
        f3 position = add(a.origin, f3{(float)x * a.spacing, (float)y * a.spacing, (float)z * a.spacing});
        f3 normal{0.0f, 0.0f, 0.0f};
        float sign = (axis & 1) ? -1.0f : 1.0f;
        if (axis < 2) normal.x = sign;
        else if (axis < 4) normal.y = sign;
        else normal.z = sign;
        Pcg rng = stream6(sc.seed, kProbeStream, x, y, z, axis);
        f2 off;
        off.x = rng.next_f32();
        off.y = rng.next_f32();
        f3 side, across;
        ortho_pair(normal, side, across);
        uint32_t open = 0, back = 0, samples = sc.sky_samples;
        for (uint32_t taken = 0; taken < samples; ++taken) {
            f3 dir = cosine_direction_basis(normal, side, across, spread(taken, off, true));
            Hit h;
            bool found = traverse<false, false, REFINE>(sc, position, dir, INFINITY, a.alpha != 0, stack + threadIdx.x,
                                                        kBlock, h, &vis) &&
                         h.t > 0.0f;
            if (found && dot(hit_face_normal(sc, h), dir) > 0.0f) ++back;
            if (!found) ++open;
        }
        a.open[i] = (float)open / (float)(samples > 1 ? samples : 1);
        a.back[i] = back;
    }
    if (REFINE) add_retests(ctr, vis.retests);
}

// The bounce window of a (mesh, light) entry: its crops' union grown by 4 (bounce_map.rs:30-43).
__host__ __device__ __forceinline__ Rect bounce_window(const uint32_t *r, uint32_t res) {
    uint32_t last = res - 1;
    return Rect{r[0] >= 4 ? r[0] - 4 : 0, r[1] >= 4 ? r[1] - 4 : 0, min(r[2] + 4, last), min(r[3] + 4, last)};
}

__global__ void k_window_sizes(DevScene sc, const uint32_t *region_rect, uint32_t entries, uint32_t *size) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e > entries) return;
    size[e] = 0;
    if (e == entries) return;
    const uint32_t *r = region_rect + (size_t)e * 4;
    uint32_t s = e % sc.light_count, m = e / sc.light_count;
    if (r[0] == kNoRect || !(sc.lights[s].flags & kLightBounce)) return;
    Rect w = bounce_window(r, sc.mesh_res[m]);
    size[e] = (w.max_x - w.min_x + 1) * (w.max_y - w.min_y + 1);
}

// Later triangles overwrite shared texels (bounce.rs:202-209): the highest triangle index that
// gathered a texel owns it; a second pass writes the owner's value.
template <bool WRITE>
__global__ void k_bounce_scatter(DevScene sc, BounceArgs a, const uint32_t *region_rect, const uint32_t *woff,
                                 uint32_t *owner, float4 *map) {
    unsigned long long item = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= a.items) return;
    float4 v = a.value[item];
    if (v.w == 0.0f) return;
    uint32_t lo = 0, hi = a.bpair_count;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if ((unsigned long long)a.bitem_off[mid] <= item) lo = mid;
        else hi = mid;
    }
    uint32_t p = a.bpairs[lo];
    uint32_t t = a.pair_tri[p], s = a.pair_light[p];
    uint32_t m = sc.tri_mesh[t];
    size_t e = (size_t)m * sc.light_count + s;
    Rect w = bounce_window(region_rect + e * 4, sc.mesh_res[m]);
    uint32_t xy = a.ctex_xy[a.ctex_off[t] + (uint32_t)(item - a.bitem_off[lo])];
    uint32_t x = xy & 0xFFFFu, y = xy >> 16;
    size_t idx = woff[e] + (size_t)(y - w.min_y) * (w.max_x - w.min_x + 1) + (x - w.min_x);
    uint32_t key = t - sc.mesh_tri_base[m] + 1;
    if (!WRITE)
        atomicMax(owner + idx, key);
    else if (owner[idx] == key)
        map[idx] = make_float4(v.x, v.y, v.z, 0.0f);
}

// dilate then separable blur (bounce_map.rs:67-112) of one window per block; A holds the
// scattered map on entry and B the filtered map on exit.
__global__ void __launch_bounds__(256) k_bounce_filter(DevScene sc, const uint32_t *region_rect, const uint32_t *woff,
                                                       const uint32_t *wsize, float4 *A, float4 *B, float w0, float w1,
                                                       float w2, float w3, float w4, float w5, float w6, float wsum) {
    size_t e = blockIdx.x;
    if (!wsize[e]) return;
    uint32_t m = (uint32_t)(e / sc.light_count);
    uint32_t res = sc.mesh_res[m];
    Rect w = bounce_window(region_rect + e * 4, res);
    uint32_t ww = w.max_x - w.min_x + 1, wh = w.max_y - w.min_y + 1, n = ww * wh;
    float4 *a = A + woff[e], *b = B + woff[e];
    auto get = [&](const float4 *g, int64_t x, int64_t y) -> float4 {
        if (x < (int64_t)w.min_x || y < (int64_t)w.min_y || x > (int64_t)w.max_x || y > (int64_t)w.max_y)
            return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return g[(size_t)(y - w.min_y) * ww + (x - w.min_x)];
    };
    const int order[9][2] = {{0, 0}, {-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        int64_t x = w.min_x + i % ww, y = w.min_y + i / ww;
        float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int k = 0; k < 9; ++k) {
            float4 v = get(a, x + order[k][0], y + order[k][1]);
            if (fmaxf(fmaxf(v.x, v.y), v.z) > 0.0f) {
                out = v;
                break;
            }
        }
        b[i] = out;
    }
    __syncthreads();
    const float wt[7] = {w0, w1, w2, w3, w4, w5, w6};
    int64_t last = (int64_t)res - 1;
    for (int pass = 0; pass < 2; ++pass) {
        const float4 *src = pass == 0 ? b : a;
        float4 *dst = pass == 0 ? a : b;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            int64_t x = w.min_x + i % ww, y = w.min_y + i / ww;
            float sx = 0.0f, sy = 0.0f, sz = 0.0f;
            for (int k = -3; k <= 3; ++k) {
                int64_t qx = pass == 0 ? min(max(x + k, (int64_t)0), last) : x;
                int64_t qy = pass == 0 ? y : min(max(y + k, (int64_t)0), last);
                float4 v = get(src, qx, qy);
                sx = sx + v.x * wt[k + 3];
                sy = sy + v.y * wt[k + 3];
                sz = sz + v.z * wt[k + 3];
            }
            dst[i] = make_float4(sx / wsum, sy / wsum, sz / wsum, 0.0f);
        }
        __syncthreads();
    }
}

// BounceMap::crop's "lit" test (bounce_map.rs:124-136) per bounce pair: a warp scans the
// triangle's crop in the filtered window.
__global__ void k_bounce_lit(DevScene sc, BounceArgs a, const uint4 *tri_crop, const uint32_t *region_rect,
                             const uint32_t *woff, const float4 *map, uint8_t *pair_bounce) {
    uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    unsigned lane = lane_id();
    if (b >= a.bpair_count) return;
    uint32_t p = a.bpairs[b];
    uint32_t t = a.pair_tri[p], s = a.pair_light[p];
    uint32_t m = sc.tri_mesh[t];
    size_t e = (size_t)m * sc.light_count + s;
    Rect w = bounce_window(region_rect + e * 4, sc.mesh_res[m]);
    uint32_t ww = w.max_x - w.min_x + 1;
    uint4 c = tri_crop[t];
    uint32_t cw = c.z - c.x + 1;
    uint64_t n = (uint64_t)cw * (c.w - c.y + 1);
    bool lit = false;
    for (uint64_t base = 0; base < n && !lit; base += 32) {
        uint64_t i = base + lane;
        bool l = false;
        if (i < n) {
            uint32_t x = c.x + (uint32_t)(i % cw), y = c.y + (uint32_t)(i / cw);
            float4 v = map[woff[e] + (size_t)(y - w.min_y) * ww + (x - w.min_x)];
            l = fmaxf(fmaxf(v.x, v.y), v.z) > 0.0f;
        }
        lit = __any_sync(0xFFFFFFFFu, l);
    }
    if (lane == 0) pair_bounce[p] = lit;
}

__device__ __forceinline__ uint64_t bounce_words(uint4 crop, uint32_t bits, bool colored) {
    uint64_t n = (uint64_t)(crop.z - crop.x + 5) * (crop.w - crop.y + 5);
    if (colored) return (n * 3 * bits + 31) / 32;
    uint32_t per = 32 / bits;
    return (n + per - 1) / per;
}

// pack_bounce / pack_bounce_rgb (bounce_pack.rs:28-71) of one kept entry: the padded crop grid
// of the filtered map, dithered from the stream [seed, mesh, light, triangle] in texel order.
__global__ void k_pack_bounce(DevScene sc, uint32_t entries, const uint32_t *entry_pair,
                              const unsigned long long *entry_bdst, const uint32_t *pair_tri,
                              const uint32_t *pair_light, const uint4 *tri_crop, const uint32_t *region_rect,
                              const uint32_t *woff, const float4 *map, uint32_t *words) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= entries) return;
    unsigned long long dst = entry_bdst[e];
    if (dst == ~0ull) return;
    uint32_t p = entry_pair[e];
    uint32_t t = pair_tri[p], s = pair_light[p];
    uint32_t m = sc.tri_mesh[t];
    const DevLight &l = sc.lights[s];
    if (l.bounce_bits == 8) return;  // undithered: k_pack_bounce8
    size_t re = (size_t)m * sc.light_count + s;
    Rect w = bounce_window(region_rect + re * 4, sc.mesh_res[m]);
    uint32_t ww = w.max_x - w.min_x + 1;
    uint4 c = tri_crop[t];
    int gw = (int)(c.z - c.x + 5), gh = (int)(c.w - c.y + 5);
    uint32_t bits = l.bounce_bits;
    Pcg rng = stream4(sc.seed, sc.mesh_id[m], l.id, t - sc.mesh_tri_base[m]);
    bool colored = sc.colored_bounce != 0;
    uint32_t pixel_bits = colored ? 3 * bits : bits;
    uint32_t per = 32 / bits;
    unsigned long long acc = 0;  // bits not yet written
    uint32_t acc_bits = 0;
    uint64_t out = dst;
    uint64_t n = (uint64_t)gw * gh;
    for (uint64_t i = 0; i < n; ++i) {
        int gx = (int)(i % gw), gy = (int)(i / gw);
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (gx >= 2 && gy >= 2 && gx < gw - 2 && gy < gh - 2) {
            uint32_t x = c.x + gx - 2, y = c.y + gy - 2;
            v = map[woff[re] + (size_t)(y - w.min_y) * ww + (x - w.min_x)];
        }
        uint32_t pixel;
        if (colored) {
            pixel = quantize_bounce(v.x, bits, rng);
            pixel |= quantize_bounce(v.y, bits, rng) << bits;
            pixel |= quantize_bounce(v.z, bits, rng) << (2 * bits);
        } else {
            pixel = quantize_bounce(v.x, bits, rng);
        }
        if (colored) {
            // one bit stream, pixels 3*bits wide
            acc |= (unsigned long long)pixel << acc_bits;
            acc_bits += pixel_bits;
            while (acc_bits >= 32) {
                words[out++] = (uint32_t)acc;
                acc >>= 32;
                acc_bits -= 32;
            }
        } else {
            // floor(32 / bits) pixels per word, the rest of each word left zero
            uint32_t j = (uint32_t)(i % per);
            acc |= (unsigned long long)pixel << (j * bits);
            if (j == per - 1) {
                words[out++] = (uint32_t)acc;
                acc = 0;
            }
        }
    }
    if (colored ? acc_bits > 0 : (n % per) != 0) words[out++] = (uint32_t)acc;
}

// pack_bounce(_rgb) for 8-bit bounce (bounce_pack.rs:28-86), which has no dither (its amplitude
// is 0, so no random draw is taken): every pixel quantizes on its own, so a warp packs one entry,
// each lane four consecutive pixels — one word of four 8-bit pixels, or three words of four
// 24-bit RGB pixels — in the padded crop grid's row-major order, as the sequential packer does.
__global__ void k_pack_bounce8(DevScene sc, uint32_t entries, const uint32_t *entry_pair,
                               const unsigned long long *entry_bdst, const uint32_t *pair_tri,
                               const uint32_t *pair_light, const uint4 *tri_crop, const uint32_t *region_rect,
                               const uint32_t *woff, const float4 *map, uint32_t *words) {
    const uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = lane_id();
    if (e >= entries) return;  // uniform across the warp
    const unsigned long long dst = entry_bdst[e];
    if (dst == ~0ull) return;
    const uint32_t p = entry_pair[e], t = pair_tri[p], s = pair_light[p], m = sc.tri_mesh[t];
    const DevLight &l = sc.lights[s];
    if (l.bounce_bits != 8) return;  // dithered: k_pack_bounce
    const size_t re = (size_t)m * sc.light_count + s;
    const Rect w = bounce_window(region_rect + re * 4, sc.mesh_res[m]);
    const uint32_t ww = w.max_x - w.min_x + 1, base = woff[re];
    const uint4 c = tri_crop[t];
    const int gw = (int)(c.z - c.x + 5), gh = (int)(c.w - c.y + 5);
    const uint64_t n = (uint64_t)gw * gh;
    const bool colored = sc.colored_bounce != 0;
    const uint64_t nwords = colored ? (n * 24 + 31) / 32 : (n + 3) / 4;
    Pcg none{0, 0};  // never drawn from at 8 bits
    for (uint64_t g = lane; g * 4 < n; g += 32) {
        uint32_t px[4];
        for (int k = 0; k < 4; ++k) {
            const uint64_t i = g * 4 + k;
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const int gx = (int)(i % gw), gy = (int)(i / gw);
            if (i < n && gx >= 2 && gy >= 2 && gx < gw - 2 && gy < gh - 2) {
                const uint32_t x = c.x + gx - 2, y = c.y + gy - 2;
                v = map[base + (size_t)(y - w.min_y) * ww + (x - w.min_x)];
            }
            px[k] = 0;
            if (i < n) {
                px[k] = quantize_bounce(v.x, 8, none);
                if (colored) px[k] |= quantize_bounce(v.y, 8, none) << 8 | quantize_bounce(v.z, 8, none) << 16;
            }
        }
        if (colored) {
            const uint32_t out[3] = {px[0] | px[1] << 24, px[1] >> 8 | px[2] << 16, px[2] >> 16 | px[3] << 8};
            for (int k = 0; k < 3; ++k)
                if (g * 3 + k < nwords) words[dst + g * 3 + k] = out[k];
        } else {
            words[dst + g] = px[0] | px[1] << 8 | px[2] << 16 | px[3] << 24;
        }
    }
}

// ================================ optimize, seams, serialize ===========================

__device__ __forceinline__ uint32_t region_get(const uint32_t *pool, uint32_t off, const uint32_t *r, uint32_t bits,
                                               int64_t x, int64_t y) {
    if (x < (int64_t)r[0] || y < (int64_t)r[1] || x > (int64_t)r[2] || y > (int64_t)r[3]) return 0;
    uint64_t w = r[2] - r[0] + 1;
    uint64_t idx = (uint64_t)(x - r[0]) + (uint64_t)(y - r[1]) * w;
    if (bits == 1) return (pool[off + idx / 32] >> (idx % 32)) & 1u;
    return (pool[off + idx / 4] >> ((idx % 4) * 8)) & 0xFFu;
}

// LightEntries::optimize (shadows.rs:54-73) + any_light (:136-144): a warp per pair scans the
// triangle's optimize rect within the light's region for any lit texel; marks used regions and
// counts kept entries per triangle.
__global__ void k_optimize(DevScene sc, uint32_t pairs, const uint32_t *pair_tri, const uint32_t *pair_light,
                           const uint32_t *region_rect, const uint32_t *region_off, const uint32_t *region_pool,
                           const uint8_t *pair_bounce, uint8_t *keep, uint32_t *kept_count, uint8_t *used,
                           Counters *ctr) {
    uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    unsigned lane = lane_id();
    if (p >= pairs) return;
    uint32_t t = pair_tri[p], s = pair_light[p];
    TriData d;
    load_tri(sc, t, d);
    size_t e = (size_t)d.mesh * sc.light_count + s;
    bool k = pair_bounce && pair_bounce[p];
    if (!k) {
        Rect o = center_rect(d.uv, d.res, 1.0f);
        const uint32_t *r = region_rect + e * 4;
        uint32_t min_x = max(o.min_x, r[0]), max_x = min(o.max_x, r[2]);
        uint32_t min_y = max(o.min_y, r[1]), max_y = min(o.max_y, r[3]);
        if (min_x <= max_x && min_y <= max_y) {
            uint32_t w = max_x - min_x + 1;
            uint64_t n = (uint64_t)w * (max_y - min_y + 1);
            uint32_t bits = sc.lights[s].shadow_bits, roff = region_off[e];
            for (uint64_t base = 0; base < n && !k; base += 32) {
                uint64_t i = base + lane;
                bool lit = i < n && region_get(region_pool, roff, r, bits, min_x + (uint32_t)(i % w),
                                               min_y + (uint32_t)(i / w)) != 0;
                k = __any_sync(0xFFFFFFFFu, lit);
            }
        }
    }
    if (lane == 0) {
        keep[p] = k;
        if (k) {
            used[e] = 1;
            atomicAdd(kept_count + t, 1u);
        } else {
            atomicAdd(&ctr->lights_removed, 1ull);
        }
    }
}

// pad_seams (seams.rs:15-39) on every used region; a block per (mesh, light) entry.
__global__ void k_pad_seams(DevScene sc, const uint8_t *used, const uint32_t *region_rect, const uint32_t *region_off,
                            uint32_t *region_pool, const uint32_t *visited, const uint64_t *grid_off) {
    size_t e = blockIdx.x;
    if (!used[e]) return;
    const uint32_t *r = region_rect + e * 4;
    uint32_t m = (uint32_t)(e / sc.light_count), s = (uint32_t)(e % sc.light_count);
    uint32_t res = sc.mesh_res[m];
    const uint32_t *vis = visited + grid_off[m];
    uint32_t bits = sc.lights[s].shadow_bits;
    uint32_t off = region_off[e];
    uint32_t w = r[2] - r[0] + 1, h = r[3] - r[1] + 1;
    auto visited_at = [&](int64_t x, int64_t y) -> bool {
        if (x < 0 || y < 0 || x >= (int64_t)res || y >= (int64_t)res) return false;
        uint64_t bit = (uint64_t)x + (uint64_t)y * res;
        return (vis[bit / 32] >> (bit % 32)) & 1u;
    };
    const int dxs[4] = {-1, 1, 0, 0}, dys[4] = {0, 0, -1, 1};
    for (uint64_t i = threadIdx.x; i < (uint64_t)w * h; i += blockDim.x) {
        int64_t x = r[0] + (int64_t)(i % w), y = r[1] + (int64_t)(i / w);
        if (visited_at(x, y)) continue;
        uint32_t level = 0;
        for (int k = 0; k < 4; ++k) {
            int64_t nx = x + dxs[k], ny = y + dys[k];
            if (visited_at(nx, ny))
                level = max(level, region_get(region_pool, off, r, bits, nx, ny));
            else if (visited_at(x + 2 * dxs[k], y + 2 * dys[k]))
                level = max(level, region_get(region_pool, off, r, bits, x + 2 * dxs[k], y + 2 * dys[k]));
        }
        if (!level) continue;  // unvisited texels hold 0 already
        if (bits == 1)
            atomicOr(region_pool + off + i / 32, 1u << (i % 32));
        else
            reinterpret_cast<uint8_t *>(region_pool + off)[i] = (uint8_t)level;
    }
}

__device__ __forceinline__ uint64_t shadow_words(uint4 crop, uint32_t bits) {
    uint64_t n = (uint64_t)(crop.z - crop.x + 5) * (crop.w - crop.y + 5);
    uint32_t per = 32 / bits;
    return (n + per - 1) / per;
}

// Words per triangle: light data (1 + stride per kept light) and payload.
__global__ void k_tri_words(DevScene sc, const uint32_t *tri_off, const uint32_t *pair_light, const uint8_t *keep,
                            const uint8_t *pair_bounce, const uint4 *tri_crop, uint32_t stride,
                            unsigned long long *ld_words, unsigned long long *pl_words) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > sc.triangles) return;
    if (t == sc.triangles) {
        ld_words[t] = pl_words[t] = 0;
        return;
    }
    uint4 c = tri_crop[t];
    unsigned long long ld = 1, pl = 0;
    for (uint32_t p = tri_off[t]; p < tri_off[t + 1]; ++p)
        if (keep[p]) {
            const DevLight &l = sc.lights[pair_light[p]];
            ld += stride;
            pl += shadow_words(c, l.shadow_bits);
            if (stride == 3 && pair_bounce[p]) pl += bounce_words(c, l.bounce_bits, sc.colored_bounce != 0);
        }
    ld_words[t] = ld;
    pl_words[t] = pl;
}

__global__ void k_mesh_words(DevScene sc, const unsigned long long *ld_scan, const unsigned long long *pl_scan,
                             unsigned long long *mesh_words) {
    uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m > sc.mesh_count) return;
    if (m == sc.mesh_count) {
        mesh_words[m] = 0;
        return;
    }
    uint32_t a = sc.mesh_tri_base[m], b = sc.mesh_tri_base[m + 1];
    mesh_words[m] = 4ull * (b - a) + (ld_scan[b] - ld_scan[a]) + (pl_scan[b] - pl_scan[a]);
}

// serialize_triangles (triangle_words.rs:47-89): headers, light data, and where each kept
// entry's shadow words go.
__global__ void k_serialize(DevScene sc, const uint32_t *tri_off, const uint32_t *pair_light, const uint8_t *keep,
                            const uint8_t *pair_bounce, const uint4 *tri_crop, uint32_t stride,
                            const unsigned long long *ld_scan, const unsigned long long *pl_scan,
                            const unsigned long long *mesh_base, const uint32_t *entry_off, uint32_t *words,
                            uint32_t *entry_pair, unsigned long long *entry_dst, unsigned long long *entry_bdst) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sc.triangles) return;
    uint32_t m = sc.tri_mesh[t];
    uint32_t first = sc.mesh_tri_base[m], tris = sc.mesh_tri_base[m + 1] - first;
    unsigned long long base = mesh_base[m];
    uint32_t ld_total = (uint32_t)(ld_scan[first + tris] - ld_scan[first]);
    uint32_t ld = 4 * tris + (uint32_t)(ld_scan[t] - ld_scan[first]);
    uint32_t pl = 4 * tris + ld_total + (uint32_t)(pl_scan[t] - pl_scan[first]);
    uint4 c = tri_crop[t];
    uint32_t lt = t - first;
    words[base + 4 * lt] = ld;
    words[base + 4 * lt + 1] = c.x - 2u;
    words[base + 4 * lt + 2] = c.y - 2u;
    words[base + 4 * lt + 3] = c.z - c.x + 5;
    uint32_t count = 0;
    uint32_t e = entry_off[t];
    for (uint32_t p = tri_off[t]; p < tri_off[t + 1]; ++p) {
        if (!keep[p]) continue;
        uint32_t s = pair_light[p];
        const DevLight &l = sc.lights[s];
        uint32_t at = ld + 1 + count * stride;
        words[base + at] = s;
        words[base + at + 1] = pl;
        entry_pair[e] = p;
        entry_dst[e] = base + pl;
        pl += (uint32_t)shadow_words(c, l.shadow_bits);
        entry_bdst[e] = ~0ull;
        if (stride == 3) {
            words[base + at + 2] = 0;
            if (pair_bounce[p]) {
                words[base + at + 2] = pl;
                entry_bdst[e] = base + pl;
                pl += (uint32_t)bounce_words(c, l.bounce_bits, sc.colored_bounce != 0);
            }
        }
        ++count;
        ++e;
    }
    words[base + ld] = count;
}

// crop_shadows (shadows.rs:148-159) with dilate_shadows (seams.rs:43-71), packed as
// ShadowGrid::into_words (shadow_grid.rs:91-106). A warp per kept entry, a lane per word; every
// texel of the padded grid is computed from the region directly:
//   interior: the region's level; inner ring: 3x3 max of the interior; outer ring: 3x3 max of
//   interior and inner ring.
__device__ __forceinline__ uint32_t crop_level(const uint32_t *pool, uint32_t off, const uint32_t *r, uint32_t bits,
                                               uint4 c, int gw, int gh, int gx, int gy) {
    auto interior = [&](int x, int y) -> uint32_t {
        if (x < 2 || y < 2 || x >= gw - 2 || y >= gh - 2) return 0;
        return region_get(pool, off, r, bits, (int64_t)c.x + x - 2, (int64_t)c.y + y - 2);
    };
    auto inner = [&](int x, int y) -> uint32_t {
        uint32_t v = 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) v = max(v, interior(x + dx, y + dy));
        return v;
    };
    bool outer = gx == 0 || gy == 0 || gx == gw - 1 || gy == gh - 1;
    if (outer) {
        uint32_t v = 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int x = gx + dx, y = gy + dy;
                if (x < 0 || y < 0 || x >= gw || y >= gh) continue;
                bool ring = x == 0 || y == 0 || x == gw - 1 || y == gh - 1;
                if (ring) continue;  // outer ring cells are 0 after the first pass
                bool in_ring = x == 1 || y == 1 || x == gw - 2 || y == gh - 2;
                v = max(v, in_ring ? inner(x, y) : interior(x, y));
            }
        return v;
    }
    bool in_ring = gx == 1 || gy == 1 || gx == gw - 2 || gy == gh - 2;
    return in_ring ? inner(gx, gy) : interior(gx, gy);
}

constexpr int kCropBytes = 2048;  // per-warp staging grid in shared memory (texels)

// 1-bit words LSB first (bits.rs:40-46): word w holds texels 32w .. 32w + 31, so lane j's texel of
// word w is bit j of a warp ballot. Each round of 32 words ends with one coalesced store per lane.
template <class Texel>
__device__ __forceinline__ void ballot_words(uint64_t n, uint64_t nw, uint32_t *out, unsigned lane, Texel texel) {
    for (uint64_t base = 0; base < nw; base += 32) {
        uint32_t mine = 0;
        for (uint32_t k = 0; k < 32 && base + k < nw; ++k) {
            uint64_t i = (base + k) * 32 + lane;
            uint32_t b = __ballot_sync(0xFFFFFFFFu, i < n && texel(i) != 0);
            if (lane == k) mine = b;
        }
        if (base + lane < nw) out[base + lane] = mine;
    }
}

__global__ void __launch_bounds__(kBlock) k_crop(DevScene sc, uint32_t entries, const uint32_t *entry_pair,
                                                const unsigned long long *entry_dst, const uint32_t *pair_tri,
                                                const uint32_t *pair_light, const uint4 *tri_crop,
                                                const uint32_t *region_rect, const uint32_t *region_off,
                                                const uint32_t *region_pool, uint32_t *words) {
    __shared__ uint8_t stage[kBlock / 32][kCropBytes];
    uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    unsigned lane = lane_id();
    if (e >= entries) return;
    uint8_t *g = stage[threadIdx.x >> 5];
    uint32_t p = entry_pair[e];
    uint32_t t = pair_tri[p], s = pair_light[p];
    uint32_t m = sc.tri_mesh[t];
    uint4 c = tri_crop[t];
    size_t re = (size_t)m * sc.light_count + s;
    const uint32_t *r = region_rect + re * 4;
    uint32_t off = region_off[re];
    uint32_t bits = sc.lights[s].shadow_bits;
    int gw = (int)(c.z - c.x + 5), gh = (int)(c.w - c.y + 5);
    uint64_t n = (uint64_t)gw * gh;
    uint32_t per = 32 / bits;
    uint64_t nw = (n + per - 1) / per;
    unsigned long long dst = entry_dst[e];
    if (n > (uint64_t)kCropBytes) {
        // large crops: every texel straight from the region
        if (bits == 1) {
            ballot_words(n, nw, words + dst, lane, [&](uint64_t i) {
                return crop_level(region_pool, off, r, bits, c, gw, gh, (int)(i % gw), (int)(i / gw));
            });
            return;
        }
        for (uint64_t wi = lane; wi < nw; wi += 32) {
            uint32_t word = 0;
            for (uint32_t j = 0; j < per; ++j) {
                uint64_t i = wi * per + j;
                if (i >= n) break;
                uint32_t v = crop_level(region_pool, off, r, bits, c, gw, gh, (int)(i % gw), (int)(i / gw));
                word |= (bits == 1 ? (v != 0) : v) << (j * bits);
            }
            words[dst + wi] = word;
        }
        return;
    }
    auto interior = [&](int x, int y) { return x >= 2 && y >= 2 && x < gw - 2 && y < gh - 2; };
    auto outer = [&](int x, int y) { return x == 0 || y == 0 || x == gw - 1 || y == gh - 1; };
    // the crop: interior texels from the region, padding rings zero
    for (int i = lane; i < (int)n; i += 32) {
        int x = i % gw, y = i / gw;
        g[i] = interior(x, y) ? (uint8_t)region_get(region_pool, off, r, bits, (int64_t)c.x + x - 2,
                                                     (int64_t)c.y + y - 2)
                              : 0;
    }
    __syncwarp();
    // first ring pass: inner ring = 3x3 max of the crop (only interior texels are non-zero there)
    for (int i = lane; i < (int)n; i += 32) {
        int x = i % gw, y = i / gw;
        if (interior(x, y) || outer(x, y)) continue;
        uint32_t v = 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
                if (interior(x + dx, y + dy)) v = max(v, (uint32_t)g[(y + dy) * gw + x + dx]);
        g[i] = (uint8_t)v;
    }
    __syncwarp();
    // second ring pass: outer ring = 3x3 max of interior and inner ring (outer cells are 0 then)
    for (int i = lane; i < (int)n; i += 32) {
        int x = i % gw, y = i / gw;
        if (!outer(x, y)) continue;
        uint32_t v = 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = x + dx, yy = y + dy;
                if (xx < 0 || yy < 0 || xx >= gw || yy >= gh || outer(xx, yy)) continue;
                v = max(v, (uint32_t)g[yy * gw + xx]);
            }
        g[i] = (uint8_t)v;
    }
    __syncwarp();
    if (bits == 1) {
        ballot_words(n, nw, words + dst, lane, [&](uint64_t i) { return (uint32_t)g[i]; });
        return;
    }
    for (uint64_t wi = lane; wi < nw; wi += 32) {
        uint32_t word = 0;
        for (uint32_t j = 0; j < per; ++j) {
            uint64_t i = wi * per + j;
            if (i >= n) break;
            word |= (uint32_t)g[i] << (j * bits);
        }
        words[dst + wi] = word;
    }
}

// ================================ payload on the device ====================================
// The .dynlight payload assembled next to the resident words and its CRC-32 computed there, so
// the host receives finished bytes (src/bake/format/mod.rs:101-119,170-213).

// One piece of the payload: `len` words from `src` (device memory) to payload word `dst`.
struct PayloadSegment {
    unsigned long long dst;
    const uint32_t *src;
    unsigned long long len;
};
__global__ void k_payload_gather(const PayloadSegment *seg, uint32_t *out) {
    PayloadSegment g = seg[blockIdx.x];
    for (unsigned long long i = threadIdx.x; i < g.len; i += blockDim.x) out[g.dst + i] = g.src[i];
}

constexpr uint32_t kCrcChunkWords = 16384;  // 64 KiB chunks, 128 threads x 512 bytes
struct CrcShifts {
    uint32_t m[7][32];  // shift of the CRC register by 512 * 2^l bytes, l = 0 .. 6, as GF(2) columns
};
__device__ __forceinline__ uint32_t gf2_times(const uint32_t *m, uint32_t v) {
    uint32_t r = 0;
    for (int i = 0; i < 32; ++i)
        if ((v >> i) & 1u) r ^= m[i];
    return r;
}
// The raw CRC-32 register (from zero, no inversion) of every full 64 KiB chunk: each of 128
// threads runs 512 bytes by slicing by 4 over little-endian words (Kounavis & Berry 2008), then
// the block combines the parts pairwise, raw(A B) = shift(raw(A), |B|) ^ raw(B).
__global__ void __launch_bounds__(128) k_crc_chunks(const uint32_t *data, unsigned long long chunks,
                                                    const uint32_t *tables, CrcShifts sh, uint32_t *out) {
    __shared__ uint32_t t[4][256];
    __shared__ uint32_t part[128];
    __shared__ uint32_t m[7][32];
    for (int i = threadIdx.x; i < 1024; i += 128) t[i / 256][i % 256] = tables[i];
    for (int i = threadIdx.x; i < 224; i += 128) m[i / 32][i % 32] = sh.m[i / 32][i % 32];
    __syncthreads();
    for (unsigned long long chunk = blockIdx.x; chunk < chunks; chunk += gridDim.x) {
        const uint32_t *p = data + chunk * kCrcChunkWords + threadIdx.x * 128;
        uint32_t c = 0;
        for (int i = 0; i < 128; ++i) {
            c ^= p[i];
            c = t[3][c & 0xFF] ^ t[2][(c >> 8) & 0xFF] ^ t[1][(c >> 16) & 0xFF] ^ t[0][c >> 24];
        }
        part[threadIdx.x] = c;
        __syncthreads();
        for (int l = 0; l < 7; ++l) {
            unsigned stride = 1u << l;
            if ((threadIdx.x & (2 * stride - 1)) == 0)
                part[threadIdx.x] = gf2_times(m[l], part[threadIdx.x]) ^ part[threadIdx.x + stride];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[chunk] = part[0];
        __syncthreads();
    }
}

// ================================ host side =================================================

namespace {

thread_local std::string g_error;
std::mutex g_busy;

struct CudaError {
    cudaError_t code;
    const char *what;
};

#define CK(x)                                                      \
    do {                                                           \
        cudaError_t e__ = (x);                                     \
        if (e__ != cudaSuccess) throw CudaError{e__, #x};          \
    } while (0)

// Launch errors surface here, named by the kernel that caused them.
#define LAUNCHED(name)                                       \
    do {                                                     \
        cudaError_t e__ = cudaGetLastError();                \
        if (e__ != cudaSuccess) throw CudaError{e__, name};  \
    } while (0)

// Device memory comes from the device's default stream-ordered pool, allocated and freed on the
// session's stream. The pool keeps what sessions free (its release threshold is raised once per
// device), so the next bake's allocations reuse it without new cudaMalloc/cudaFree calls;
// dl_release_memory hands it back to the driver.
std::mutex g_pool_lock;
std::vector<int> g_pooled_devices;  // devices whose default pool keeps freed memory
void keep_freed_device_memory(int device) {
    std::lock_guard<std::mutex> guard(g_pool_lock);
    if (std::find(g_pooled_devices.begin(), g_pooled_devices.end(), device) != g_pooled_devices.end()) return;
    cudaMemPool_t pool;
    CK(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = ~0ull;
    CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pooled_devices.push_back(device);
}
// Returns the pooled memory of every device the library has baked on (no other device is touched).
void release_pooled_device_memory() {
    std::lock_guard<std::mutex> guard(g_pool_lock);
    for (int d : g_pooled_devices) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, d) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    }
}
// The device memory a session holds (scene, BVH, its build scratch, every stage's buffers)
// against the caller's cap (dl_bake_config.max_device_mib; 0: none). An allocation past the cap
// fails like a failed cudaMallocAsync, so the bake reports DL_OUT_OF_MEMORY.
struct DeviceBudget {
    uint64_t cap = 0, held = 0;
    void reserve(size_t b) {
        if (cap && held + b > cap)
            throw CudaError{cudaErrorMemoryAllocation, "device memory cap (dl_bake_config.max_device_mib)"};
        held += b;
    }
    void release(size_t b) { held -= std::min<uint64_t>(held, b); }
};

void *dev_malloc(size_t bytes, cudaStream_t st, DeviceBudget *budget) {
    void *p = nullptr;
    const size_t b = std::max<size_t>(bytes, 16);
    if (budget) budget->reserve(b);
    cudaError_t e = cudaMallocAsync(&p, b, st);
    if (e != cudaSuccess) {
        if (budget) budget->release(b);
        throw CudaError{e, "cudaMallocAsync"};
    }
    return p;
}

template <class T>
T *dev_alloc(std::vector<void *> &owned, cudaStream_t st, size_t count, uint64_t &bytes, DeviceBudget *budget) {
    size_t b = std::max<size_t>(count * sizeof(T), 16);
    void *p = dev_malloc(b, st, budget);
    owned.push_back(p);
    bytes += b;
    return static_cast<T *>(p);
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

// A named pool of device buffers, grown on demand and reused across runs of one session;
// allocated and freed on the session's stream.
struct Pool {
    std::map<std::string, std::pair<void *, size_t>> bufs;
    cudaStream_t stream = nullptr;
    DeviceBudget *budget = nullptr;
    uint64_t bytes = 0;
    uint64_t generation = 0;  // bumped whenever a buffer moves
    template <class T>
    T *get(const std::string &name, size_t count) {
        size_t b = std::max<size_t>(count * sizeof(T), 16);
        auto it = bufs.find(name);
        if (it != bufs.end() && it->second.second >= b) return static_cast<T *>(it->second.first);
        if (it != bufs.end()) {
            cudaFreeAsync(it->second.first, stream);
            bytes -= it->second.second;
            if (budget) budget->release(it->second.second);
            bufs.erase(it);
        }
        void *p = dev_malloc(b, stream, budget);
        bufs[name] = {p, b};
        bytes += b;
        ++generation;
        return static_cast<T *>(p);
    }
    // Frees every buffer on the stream; the session calls it before destroying its stream.
    void release() {
        for (auto &kv : bufs) {
            cudaFreeAsync(kv.second.first, stream);
            if (budget) budget->release(kv.second.second);
        }
        bufs.clear();
        bytes = 0;
    }
};

}  // namespace dl

using namespace dl;

struct dl_session {
    HostScene host;
    dl_bake_options options{};
    dl_bake_config config{};
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr, side = nullptr;
    std::vector<void *> owned;
    uint64_t scene_bytes = 0;
    DevScene sc{};
    std::vector<uint64_t> grid_off;  // visited/owned word offset per mesh
    uint64_t grid_words = 0;
    std::vector<uint32_t> mesh_tri_base;
    Pool pool;
    DeviceBudget budget;  // device memory held against config.max_device_mib
    Counters *ctr = nullptr;
    uint32_t *cancel_dev = nullptr;
    dl_bake_report report{};
    uint64_t launches = 0;
    // last run's results (device)
    bool have_result = false;
    uint64_t out_words = 0;
    std::vector<unsigned long long> mesh_words;
    uint32_t *words_dev = nullptr;
    Counters counters{};
    uint64_t texels = 0;
    // last run's filtered bounce maps: window offsets per (mesh, light) entry, RGB texels, and the
    // entries' region rectangles (null when the run baked no bounce)
    const uint32_t *bounce_woff = nullptr;
    const float4 *bounce_map = nullptr;
    const uint32_t *region_rect = nullptr;
    // last run's maps for moving meshes (device buffers in the pool)
    const uint32_t *cube_words = nullptr;
    uint64_t cube_word_count = 0;
    std::vector<SunMapSetup> sun_setups;
    std::vector<const uint32_t *> sun_texels;
    ProbeGridSetup probe_grid;
    const float *probe_open = nullptr;
    const uint32_t *probe_back = nullptr;
    // batched-form graph over the visibility stage, rebuilt when the queue changes
    cudaEvent_t marks[9] = {};  // stage boundaries of the last run
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_generation = ~0ull;
    unsigned long long graph_items = 0;
    unsigned graph_blocks = 0;
    uint64_t graph_shape = 0;
    ~dl_session() {
        if (graph) cudaGraphExecDestroy(graph);
        for (auto &e : marks)
            if (e) cudaEventDestroy(e);
        if (stream) {
            // back to the stream-ordered pool (kept for the next session), in stream order
            pool.release();
            for (void *p : owned) cudaFreeAsync(p, stream);
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
        if (side) cudaStreamDestroy(side);
    }
};

namespace dl {
namespace {

void scan_u32(dl_session &s, const uint32_t *in, uint32_t *out, size_t n) {
    size_t temp = 0;
    CK(cub::DeviceScan::ExclusiveSum(nullptr, temp, in, out, n, s.stream));
    void *tmp = s.pool.get<uint8_t>("scan_tmp", temp);
    CK(cub::DeviceScan::ExclusiveSum(tmp, temp, in, out, n, s.stream));
    s.launches += 2;
}
void scan_u64(dl_session &s, const unsigned long long *in, unsigned long long *out, size_t n) {
    size_t temp = 0;
    CK(cub::DeviceScan::ExclusiveSum(nullptr, temp, in, out, n, s.stream));
    void *tmp = s.pool.get<uint8_t>("scan_tmp", temp);
    CK(cub::DeviceScan::ExclusiveSum(tmp, temp, in, out, n, s.stream));
    s.launches += 2;
}
template <class T>
T read_back(dl_session &s, const T *p) {
    T v;
    CK(cudaMemcpyAsync(&v, p, sizeof(T), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    return v;
}
unsigned grid_for(size_t n, unsigned block = kBlock) { return (unsigned)std::max<size_t>(1, (n + block - 1) / block); }

// Blocks the caller until the stream drains, forwarding a cancel request to the device flag. A
// forwarded request's copy (on the side stream) is waited for too, so that it cannot land after
// the next run has cleared the flag.
void wait(dl_session &s, dl_progress *progress) {
    bool forwarded = false;
    for (;;) {
        cudaError_t q = cudaStreamQuery(s.stream);
        if (q == cudaSuccess) {
            if (forwarded) CK(cudaStreamSynchronize(s.side));
            return;
        }
        if (q != cudaErrorNotReady) throw CudaError{q, "stream"};
        if (progress && progress->cancel && !forwarded) {
            static const uint32_t one = 1;
            CK(cudaMemcpyAsync(s.cancel_dev, &one, 4, cudaMemcpyHostToDevice, s.side));
            forwarded = true;
        }
        std::this_thread::yield();
    }
}

// A run that stops on the cancel flag: its report records how many warps of the device work
// queues saw the flag and stopped claiming work (0 when the request came between stages).
dl_status cancelled_run(dl_session &s) {
    Counters c{};
    CK(cudaMemcpyAsync(&c, s.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    s.report.cancel_stops = (uint32_t)c.cancelled;
    return DL_CANCELLED;
}

// Host buffers of freed results' words, handed to the next result. They are pinned (page-locked)
// when the driver allows it, so that the download runs as a DMA copy at the link's rate instead
// of through the driver's staging buffers, and a reused buffer needs no first-touch page faults
// either. At most kCacheBytes are held.
struct WordCache {
    static constexpr size_t kCacheBytes = size_t(2) << 30;
    struct Buffer {
        size_t cap;  // words
        uint32_t *p;
        bool pinned;
    };
    std::mutex lock;
    std::vector<Buffer> free;
    size_t held = 0;
    static void release(const Buffer &b) {
        if (b.pinned) cudaFreeHost(b.p);  // fails harmlessly once the runtime has shut down at exit
        else delete[] b.p;
    }
    Buffer take(size_t n) {
        {
            std::lock_guard<std::mutex> guard(lock);
            size_t best = free.size();
            for (size_t i = 0; i < free.size(); ++i)
                if (free[i].cap >= n && (best == free.size() || free[i].cap < free[best].cap)) best = i;
            if (best < free.size()) {
                Buffer b = free[best];
                free.erase(free.begin() + best);
                held -= b.cap * 4;
                return b;
            }
        }
        size_t cap = n ? n : 1;
        void *p = nullptr;
        if (cudaHostAlloc(&p, cap * 4, cudaHostAllocPortable) == cudaSuccess) return Buffer{cap, (uint32_t *)p, true};
        cudaGetLastError();  // no pinned memory to be had: a pageable buffer (a slower copy)
        return Buffer{cap, new uint32_t[cap], false};
    }
    void clear() {
        std::lock_guard<std::mutex> guard(lock);
        for (const Buffer &b : free) release(b);
        free.clear();
        held = 0;
    }
    void give(const Buffer &b) {
        std::lock_guard<std::mutex> guard(lock);
        while (held + b.cap * 4 > kCacheBytes && !free.empty()) {  // drop the oldest
            held -= free.front().cap * 4;
            release(free.front());
            free.erase(free.begin());
        }
        if (b.cap * 4 > kCacheBytes) {
            release(b);
            return;
        }
        free.push_back(b);
        held += b.cap * 4;
    }
};
WordCache &word_cache() {
    static WordCache *c = new WordCache;  // never destroyed: results may be freed during exit
    return *c;
}

// `progress`, when given, is checked for cancellation once validation has passed and before the
// first CUDA call: as in the reference (baker.rs:32-55), invalid input reports its own error even
// when the bake was already cancelled.
dl_status create(const dl_bake_input *in, const dl_bake_options *o, const dl_bake_config *cfg, dl_session *&out,
                 const dl_progress *progress = nullptr) {
    auto s = std::make_unique<dl_session>();
    s->options = *o;
    if (cfg) s->config = *cfg;
    if (s->config.form > DL_FORM_BOUNCE_REFINED) {
        g_error = "unknown bake form " + std::to_string(s->config.form);
        return DL_INVALID_ARGUMENT;
    }
    uint32_t lanes = s->config.sample_lanes;
    if (lanes > 32 || (lanes & (lanes - 1))) {
        g_error = "sample_lanes must be 0 or a power of two up to 32";
        return DL_INVALID_ARGUMENT;
    }
    const uint32_t mb = s->config.min_blocks, gmb = s->config.gather_min_blocks;
    if (!(mb == 0 || (mb >= 7 && mb <= 10) || mb == 12)) {
        g_error = "min_blocks must be 0, 7, 8, 9, 10 or 12";
        return DL_INVALID_ARGUMENT;
    }
    if (!(gmb == 0 || gmb == 6 || (gmb >= 8 && gmb <= 10))) {
        g_error = "gather_min_blocks must be 0, 6, 8, 9 or 10";
        return DL_INVALID_ARGUMENT;
    }
    float eps = s->config.refine_epsilon;
    if (!(eps >= 0.0f && eps <= 0.01f)) {
        g_error = "refine_epsilon must lie in [0, 0.01]";
        return DL_INVALID_ARGUMENT;
    }
    if (eps == 0.0f) s->config.refine_epsilon = 1.0e-4f;
    std::string err;
    auto t_prep = std::chrono::steady_clock::now();
    dl_status st = prepare_scene(*in, *o, s->host, err);
    if (st != DL_OK) {
        g_error = err;
        return st;
    }
    HostScene &h = s->host;
    for (uint32_t r : h.resolution)
        if (r > 65535) {
            g_error = "shadow maps larger than 65535 texels per side are not supported";
            return DL_UNSUPPORTED;
        }
    if (progress && progress->cancel) {
        g_error = "the bake was cancelled";
        return DL_CANCELLED;
    }
    s->report.ms_host[0] = ms_since(t_prep);
    // the occluder BVH: on the host's cores when asked, else on the device once the triangles
    // are uploaded (the same tree)
    const bool host_bvh = s->config.host_bvh != 0;
    if (host_bvh) {
        auto t_bvh = std::chrono::steady_clock::now();
        build_bvh(h);
        s->report.ms_host[1] = ms_since(t_bvh);
        // the traversal stack holds one entry per level below the root
        if (h.bvh_depth >= (uint32_t)kStack) {
            g_error = "occluder BVH deeper than the traversal stack";
            return DL_UNSUPPORTED;
        }
    }
    auto t_up = std::chrono::steady_clock::now();
    s->device = (int)s->config.device;
    CK(cudaSetDevice(s->device));
    CK(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device));
    CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
    keep_freed_device_memory(s->device);
    s->pool.stream = s->stream;
    s->budget.cap = (uint64_t)s->config.max_device_mib << 20;
    s->pool.budget = &s->budget;

    // flatten meshes
    uint32_t M = (uint32_t)h.meshes.size();
    std::vector<uint32_t> vbase(M + 1, 0), ibase(M + 1, 0), tbase(M + 1, 0), flags(M), alpha(M * 4, 0);
    std::vector<uint64_t> ids(M);
    std::vector<float> albedo(M * 3);
    std::vector<uint8_t> alpha_pool;
    for (uint32_t m = 0; m < M; ++m) {
        const dl_mesh &mm = *h.meshes[m];
        vbase[m + 1] = vbase[m] + mm.vertex_count;
        ibase[m + 1] = ibase[m] + (uint32_t)mm.index_count;
        tbase[m + 1] = tbase[m] + (uint32_t)(mm.index_count / 3);
        ids[m] = mm.id;
        for (int k = 0; k < 3; ++k) albedo[m * 3 + k] = mm.albedo[k];
        flags[m] = (mm.normals ? kMeshNormals : 0) | (mm.occludes ? kMeshOccludes : 0) |
                   (mm.alpha && mm.uv0 ? kMeshAlpha : 0);
        if (mm.alpha && mm.uv0) {
            alpha[m * 4] = (uint32_t)alpha_pool.size();
            alpha[m * 4 + 1] = mm.alpha->width;
            alpha[m * 4 + 2] = mm.alpha->height;
            std::memcpy(&alpha[m * 4 + 3], &mm.alpha->cutoff, 4);
            size_t n = (size_t)mm.alpha->width * mm.alpha->height;
            for (size_t i = 0; i < n; ++i) alpha_pool.push_back(mm.alpha->rgba8[i * 4 + 3]);
        }
    }
    uint32_t V = vbase[M], I = ibase[M], T = tbase[M];
    // The per-vertex and per-index arrays are flattened by the host's cores into one pinned
    // staging buffer (reused across sessions through the result-word cache), so that their
    // uploads run as DMA copies; the buffer goes back once the stream has drained.
    struct Staging {
        WordCache::Buffer b;
        cudaStream_t stream;
        ~Staging() {
            if (stream) cudaStreamSynchronize(stream);
            word_cache().give(b);
        }
    } staging{word_cache().take((size_t)V * 10 + I + T + 1), s->stream};
    float *pos = reinterpret_cast<float *>(staging.b.p), *nrm = pos + (size_t)V * 3, *uv1 = nrm + (size_t)V * 3,
          *uv0 = uv1 + (size_t)V * 2;
    uint32_t *idx = reinterpret_cast<uint32_t *>(uv0 + (size_t)V * 2), *tri_mesh = idx + I;
    auto flatten = [&](uint32_t m) {
        const dl_mesh &mm = *h.meshes[m];
        std::memcpy(&pos[(size_t)vbase[m] * 3], mm.positions, mm.vertex_count * 12ull);
        if (mm.normals) std::memcpy(&nrm[(size_t)vbase[m] * 3], mm.normals, mm.vertex_count * 12ull);
        else std::memset(&nrm[(size_t)vbase[m] * 3], 0, mm.vertex_count * 12ull);
        for (uint32_t v = 0; v < mm.vertex_count; ++v) {
            float a = mm.uv1[v * 2], b = mm.uv1[v * 2 + 1];
            bool ok = std::isfinite(a) && std::isfinite(b);  // mesh_builder.rs:30-40
            uv1[((size_t)vbase[m] + v) * 2] = ok ? a : 0.0f;
            uv1[((size_t)vbase[m] + v) * 2 + 1] = ok ? b : 0.0f;
        }
        if (mm.uv0) std::memcpy(&uv0[(size_t)vbase[m] * 2], mm.uv0, mm.vertex_count * 8ull);
        else std::memset(&uv0[(size_t)vbase[m] * 2], 0, mm.vertex_count * 8ull);
        std::memcpy(&idx[ibase[m]], mm.indices, mm.index_count * 4ull);
        for (uint32_t t = tbase[m]; t < tbase[m + 1]; ++t) tri_mesh[t] = m;
    };
    {
        // meshes split into contiguous runs of about equal vertex and index counts, one per thread
        const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        const uint64_t per = ((uint64_t)V + I) / hw + 1;
        std::vector<uint32_t> cut{0};
        uint64_t acc = 0;
        for (uint32_t m = 0; m < M; ++m) {
            acc += (uint64_t)h.meshes[m]->vertex_count + h.meshes[m]->index_count;
            if (acc >= per && m + 1 < M) {
                cut.push_back(m + 1);
                acc = 0;
            }
        }
        cut.push_back(M);
        std::vector<std::thread> pool;
        for (size_t r = 0; r + 2 < cut.size(); ++r)
            pool.emplace_back([&, r] {
                for (uint32_t m = cut[r]; m < cut[r + 1]; ++m) flatten(m);
            });
        for (uint32_t m = cut[cut.size() - 2]; m < cut.back(); ++m) flatten(m);
        for (auto &t : pool) t.join();
    }
    s->grid_off.resize(M + 1);
    s->grid_words = 0;
    for (uint32_t m = 0; m < M; ++m) {
        s->grid_off[m] = s->grid_words;
        s->grid_words += ((uint64_t)h.resolution[m] * h.resolution[m] + 31) / 32;
    }
    s->grid_off[M] = s->grid_words;
    s->mesh_tri_base = tbase;
    uint32_t N = (uint32_t)h.occ_mesh.size();

    uint64_t &bytes = s->scene_bytes;
    auto up = [&](const void *src, size_t n, auto *&dst) {
        using T = std::remove_const_t<std::remove_pointer_t<std::remove_reference_t<decltype(dst)>>>;
        T *p = dev_alloc<T>(s->owned, s->stream, n / sizeof(T) + 1, bytes, &s->budget);
        if (n) CK(cudaMemcpyAsync(p, src, n, cudaMemcpyHostToDevice, s->stream));
        dst = p;
        s->report.h2d_bytes += n;
    };
    DevScene &sc = s->sc;
    sc.occluders = N;
    up(h.occ_mesh.data(), N * 4ull, sc.occ_mesh);
    up(h.occ_tri.data(), N * 4ull, sc.occ_tri);
    sc.mesh_count = M;
    up(vbase.data(), vbase.size() * 4, sc.mesh_vertex_base);
    up(ibase.data(), ibase.size() * 4, sc.mesh_index_base);
    up(tbase.data(), tbase.size() * 4, sc.mesh_tri_base);
    up(h.resolution.data(), M * 4ull, sc.mesh_res);
    up(flags.data(), M * 4ull, sc.mesh_flags);
    up(ids.data(), M * 8ull, sc.mesh_id);
    up(albedo.data(), M * 12ull, sc.mesh_albedo);
    up(alpha.data(), M * 16ull, sc.mesh_alpha);
    up(alpha_pool.data(), alpha_pool.size(), sc.alpha_pool);
    up(pos, (size_t)V * 12, sc.positions);
    up(nrm, (size_t)V * 12, sc.normals);
    up(uv1, (size_t)V * 8, sc.uv1);
    up(uv0, (size_t)V * 8, sc.uv0);
    up(idx, (size_t)I * 4, sc.indices);
    double ms_bvh_device = 0.0;
    if (host_bvh) {
        std::vector<uint32_t> occ_leaf(N);
        for (uint32_t k = 0; k < N; ++k) {
            uint32_t occ;
            std::memcpy(&occ, &h.tris[k * 12 + 3], 4);
            occ_leaf[occ] = k;
        }
        up(h.nodes.data(), h.nodes.size() * sizeof(BvhNode), sc.nodes);
        up(h.tris.data(), h.tris.size() * 4, sc.tris);
        up(occ_leaf.data(), N * 4ull, sc.occ_leaf);
    } else {
        auto t_bvh = std::chrono::steady_clock::now();
        DeviceBvhInput bi{sc.positions, sc.indices, sc.mesh_vertex_base, sc.mesh_index_base, sc.occ_mesh,
                          sc.occ_tri, N, &s->budget.held, s->budget.cap};
        DeviceBvh db;
        try {
            build_bvh_device(bi, [&](size_t b) { return (void *)dev_alloc<uint8_t>(s->owned, s->stream, b, bytes, &s->budget); }, s->stream,
                             db);
        } catch (const DeviceBvhError &e) {
            throw CudaError{e.code, e.what};
        }
        ms_bvh_device = ms_since(t_bvh);
        s->report.ms_host[1] = ms_bvh_device;
        // the traversal stack holds one entry per level below the root
        if (db.too_deep || db.depth >= (uint32_t)kStack) {
            g_error = "occluder BVH deeper than the traversal stack";
            return DL_UNSUPPORTED;
        }
        h.bvh_depth = db.depth;
        h.bvh_node_count = db.node_count;
        sc.nodes = reinterpret_cast<const float4 *>(db.nodes);
        sc.tris = db.tris;
        sc.occ_leaf = db.occ_leaf;
        if (N == 0) {  // no occluders: small placeholders, which traversal never reads
            sc.nodes = dev_alloc<float4>(s->owned, s->stream, 4, bytes, &s->budget);
            sc.tris = dev_alloc<float4>(s->owned, s->stream, 3, bytes, &s->budget);
            sc.occ_leaf = dev_alloc<uint32_t>(s->owned, s->stream, 1, bytes, &s->budget);
        }
    }
    sc.triangles = T;
    up(tri_mesh, T * 4ull, sc.tri_mesh);
    sc.light_count = (uint32_t)h.lights.size();
    sc.local_lights = h.local_lights;
    up(h.lights.data(), h.lights.size() * sizeof(DevLight), sc.lights);
    sc.seed = o->seed;
    sc.area_samples = o->area_light_samples;
    sc.area_min_samples = o->area_light_min_samples;
    sc.sky_samples = o->sky_samples;
    std::vector<uint16_t> orders, cells, cell_samples;
    for (uint32_t n = 16; n <= kMaxOrdered; n *= 2) {
        std::vector<uint16_t> o16 = sky_sample_order(n);
        orders.insert(orders.end(), o16.begin(), o16.end());
        SampleCells c = sample_cells(n);
        cells.insert(cells.end(), c.cells.begin(), c.cells.end());
        cell_samples.insert(cell_samples.end(), c.samples.begin(), c.samples.end());
    }
    up(cells.data(), cells.size() * 2, sc.order_cells);
    up(cell_samples.data(), cell_samples.size() * 2, sc.cell_samples);
    std::vector<uint16_t> sky_order = sky_sample_order(o->sky_samples);
    up(orders.data(), orders.size() * 2, sc.orders);
    sc.sky_order = nullptr;
    if (o->sky_samples <= kMaxOrdered && !sky_order.empty()) {
        sc.sky_order = sc.orders + (o->sky_samples - 16);
    } else if (!sky_order.empty()) {
        up(sky_order.data(), sky_order.size() * 2, sc.sky_order);
    }
    sc.colored_bounce = o->colored_bounce;
    sc.refine_eps = s->config.refine_epsilon;
    sc.refine_eps2 = sc.refine_eps * sc.refine_eps;
    s->ctr = dev_alloc<Counters>(s->owned, s->stream, 1, bytes, &s->budget);
    s->cancel_dev = dev_alloc<uint32_t>(s->owned, s->stream, 1, bytes, &s->budget);
    CK(cudaStreamSynchronize(s->stream));  // allocations and uploads done (the side stream and
                                           // synchronous copies use them from here on)
    for (auto &e : s->marks) CK(cudaEventCreate(&e));
    s->report.ms_host[2] = ms_since(t_up) - ms_bvh_device;
    s->report.bvh_nodes = h.bvh_node_count;
    s->report.occluders = N;
    out = s.release();
    return DL_OK;
}


// The device pipeline of one bake. Reads back the sizes it needs between stages; everything
// else stays on the device until dl_session_result.
// ---- launch-shape autotuner of the batched visibility kernel ---------------------------------
// Knobs: chunk size (warp-steps per claimed chunk), sky sample lanes (lanes sharing one sky
// texel), the launch bound's blocks per SM (the register budget: 7, 8, 9, 10 or 12 blocks of 128
// threads give 72, 64, 56, 48 or 40 registers per thread) and the stack depth (the BVH's depth,
// rounded up; it sets the shared memory per block and so, with the registers, the resident
// blocks). Each candidate runs on every k-th chunk of the real queue (k = 8 from 4 M items, 4
// from 1 M) with scratch counters; its results are the same levels the real pass writes (OR and
// max), so the trials change no output. Chunk size and lanes are tried at 8 blocks per SM, then
// the other register budgets with the winning pair (more warps hide more of the traversal's L1
// and L2 latency, fewer registers spill more: on the outdoor scene 12 blocks ran the visibility
// stage in 135.7 ms, 9 in 137.8, 10 in 139.4, 8 in 141.9). The fastest shape is cached per
// process, keyed by the device and the queue's shape.
struct TraceTune {
    uint32_t grab = 1, sky_lanes = 1, minb = 7, stack_depth = kStack, blocks = 1, trials = 0;
    double ms = 0.0;
};
using TraceKernel = void (*)(DevScene, TraceArgs);

TraceKernel trace_kernel(bool count, bool refine, uint32_t minb) {
    if (count) return refine ? k_trace_batched<true, true, 7> : k_trace_batched<true, false, 7>;
    if (refine) return k_trace_batched<false, true, 7>;
    switch (minb) {
        case 8: return k_trace_batched<false, false, 8>;
        case 9: return k_trace_batched<false, false, 9>;
        case 10: return k_trace_batched<false, false, 10>;
        case 12: return k_trace_batched<false, false, 12>;
        default: return k_trace_batched<false, false, 7>;
    }
}

struct TuneKey {
    int device;
    uint64_t items, sky_items, pairs, occluders, nodes;
    uint32_t depth, flags, fixed, fixed_minb;
    bool operator<(const TuneKey &o) const {
        return std::tie(device, items, sky_items, pairs, occluders, nodes, depth, flags, fixed, fixed_minb) <
               std::tie(o.device, o.items, o.sky_items, o.pairs, o.occluders, o.nodes, o.depth, o.flags, o.fixed,
                        o.fixed_minb);
    }
};
std::mutex g_tune_lock;
std::map<TuneKey, TraceTune> g_tune_cache;

TraceTune trace_tune(dl_session &s, TraceArgs ta, bool refine, bool count, dl_progress *progress) {
    const dl_bake_config &c = s.config;
    TraceTune best;
    best.stack_depth = std::max<uint32_t>(8, (s.host.bvh_depth + 3) & ~3u);
    auto blocks_for = [&](uint32_t minb) {
        int per_sm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_kernel(count, refine, minb), kBlock,
                                                         (size_t)best.stack_depth * kBlock * sizeof(int)));
        if (c.blocks_per_sm) per_sm = std::min(per_sm, (int)c.blocks_per_sm);
        return (uint32_t)std::max(1, per_sm) * (uint32_t)s.sms;
    };
    std::vector<uint32_t> grabs = c.chunk_texels ? std::vector<uint32_t>{std::max(1u, c.chunk_texels / 32)}
                                                 : std::vector<uint32_t>{1, 2};
    std::vector<uint32_t> lanes = c.sample_lanes ? std::vector<uint32_t>{c.sample_lanes}
                                  : ta.sky_items  ? std::vector<uint32_t>{1, 2, 4, 8, 16}
                                                  : std::vector<uint32_t>{1};
    // the chunk and lane trials run at the first budget; untuned launches take 7 blocks per SM
    std::vector<uint32_t> minbs = (count || refine) ? std::vector<uint32_t>{7}
                                  : c.min_blocks    ? std::vector<uint32_t>{c.min_blocks}
                                                    : std::vector<uint32_t>{8, 7, 9, 10, 12};
    const uint32_t every = ta.items >= (4u << 20) ? 8 : ta.items >= (1u << 20) ? 4 : 0;
    const bool tune = !c.no_autotune && every && grabs.size() * lanes.size() * minbs.size() > 1 &&
                      !(progress && progress->cancel);
    best.grab = grabs[0];
    best.sky_lanes = lanes[0];
    best.minb = (count || refine || !c.min_blocks) ? 7u : c.min_blocks;
    if (!tune) {
        best.blocks = blocks_for(best.minb);
        return best;
    }
    TuneKey key{s.device, ta.items, ta.sky_items, ta.pairs, s.host.occ_mesh.size(), s.host.bvh_node_count,
                best.stack_depth, (count ? 1u : 0u) | (refine ? 2u : 0u),
                c.chunk_texels | (c.sample_lanes << 16) | (c.blocks_per_sm << 24), c.min_blocks};
    {
        std::lock_guard<std::mutex> guard(g_tune_lock);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            TraceTune hit = it->second;
            hit.trials = 0;
            hit.ms = 0.0;
            return hit;
        }
    }
    cudaStream_t st = s.stream;
    Counters *scratch = s.pool.get<Counters>("tune_counters", 1);
    ta.ctr = scratch;
    ta.sample_every = every;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    float best_ms = INFINITY;
    auto t0 = std::chrono::steady_clock::now();
    auto trial = [&](uint32_t minb, uint32_t w, uint32_t g) {
        const uint32_t blocks = blocks_for(minb);
        ta.grab = g;
        ta.sky_lanes = w;
        CK(cudaMemsetAsync(ta.head, 0, 2 * sizeof(unsigned long long), st));
        CK(cudaEventRecord(a, st));
        trace_kernel(count, refine, minb)<<<blocks, kBlock, (size_t)best.stack_depth * kBlock * sizeof(int), st>>>(
            s.sc, ta);
        CK(cudaGetLastError());
        CK(cudaEventRecord(b, st));
        CK(cudaEventSynchronize(b));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, a, b));
        ++best.trials;
        if (ms < best_ms) {
            best_ms = ms;
            best.grab = g;
            best.sky_lanes = w;
            best.minb = minb;
            best.blocks = blocks;
        }
    };
    for (uint32_t w : lanes)
        for (uint32_t g : grabs) trial(minbs[0], w, g);
    const uint32_t w = best.sky_lanes, g = best.grab;
    for (size_t k = 1; k < minbs.size(); ++k) trial(minbs[k], w, g);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    best.ms = ms_since(t0);
    std::lock_guard<std::mutex> guard(g_tune_lock);
    g_tune_cache[key] = best;
    return best;
}

// The gather kernel's lanes per texel, tuned the same way (trials on every k-th step of the real
// item list, value writes that the real pass overwrites).
struct GatherTune {
    uint32_t lanes = 1, minb = 6, stack_depth = kStack, blocks = 1, trials = 0, buffered = 0;
    double ms = 0.0;
};
using GatherKernel = void (*)(DevScene, BounceArgs);
// The gather kernel of a variant, allowed kGatherSmemMax bytes of dynamic shared memory (above
// the default 48 KB: 16-lane groups of 256 buffered samples need 74 KB with a 64-entry stack).
constexpr int kGatherSmemMax = 80 * 1024;
GatherKernel gather_kernel(bool refine, uint32_t minb, bool count = false) {
    GatherKernel k = count    ? k_gather<true, false, 6>
                     : refine ? k_gather<false, true, 8>
                     : minb == 8  ? k_gather<false, false, 8>
                     : minb == 9  ? k_gather<false, false, 9>
                     : minb == 10 ? k_gather<false, false, 10>
                                  : k_gather<false, false, 6>;
    CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kGatherSmemMax));
    return k;
}
// Shared memory of a gather launch: stacks and, for aligned sun gathers, two masks of `buffered`
// bits per lane group (kept small: what the block does not take stays L1 cache for the BVH).
size_t gather_smem(uint32_t depth, uint32_t lanes, uint32_t buffered) {
    return (size_t)depth * kBlock * sizeof(int) + (size_t)(kBlock / lanes) * 2 * (buffered / 32) * sizeof(uint32_t);
}
// The samples a lane group holds for aligned sun gathers: the largest power-of-two sun bounce
// sample count from 32 to 256 (0 when there is none).
uint32_t gather_buffer(const HostScene &h, uint32_t) {
    uint32_t most = 0;
    for (const DevLight &l : h.lights)
        if (l.shape == DL_SHAPE_SUN && (l.flags & kLightBounce)) {
            uint32_t n = l.bounce_samples;
            if (n >= 32 && n <= 256 && !(n & (n - 1))) most = std::max(most, n);
        }
    return most;
}
// The lane groups' scratch of a gather launch (2 float4 per held sample per group), from the
// session's pool: the largest launch (one lane per group) sizes it once.
float4 *gather_scratch(dl_session &s, uint32_t blocks, uint32_t lanes, uint32_t buffered) {
    return s.pool.get<float4>("gather_scratch", (size_t)blocks * (kBlock / lanes) * 2 * buffered);
}
std::map<TuneKey, GatherTune> g_gather_cache;

GatherTune gather_tune(dl_session &s, BounceArgs ba, uint32_t bpairs, bool refine, dl_progress *progress) {
    const dl_bake_config &c = s.config;
    GatherTune best;
    best.stack_depth = std::max<uint32_t>(8, (s.host.bvh_depth + 3) & ~3u);
    auto blocks_for = [&](uint32_t minb, uint32_t w) {
        int per_sm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gather_kernel(refine, minb), kBlock,
                                                         gather_smem(best.stack_depth, w, gather_buffer(s.host, w))));
        if (c.blocks_per_sm) per_sm = std::min(per_sm, (int)c.blocks_per_sm);
        return (uint32_t)std::max(1, per_sm) * (uint32_t)s.sms;
    };
    std::vector<uint32_t> lanes = c.sample_lanes ? std::vector<uint32_t>{c.sample_lanes}
                                                 : std::vector<uint32_t>{1, 4, 8, 16, 32};
    // register budgets (blocks per SM: 6, 8, 9, 10 give 80, 64, 56, 48 registers per thread); the
    // lane trials run at the first, the others with the two best lane counts
    std::vector<uint32_t> minbs = refine                ? std::vector<uint32_t>{8}
                                  : c.gather_min_blocks ? std::vector<uint32_t>{c.gather_min_blocks}
                                                        : std::vector<uint32_t>{8, 6, 9, 10};
    const uint32_t every = ba.items >= (1u << 20) ? 8 : ba.items >= (1u << 18) ? 4 : 0;
    best.lanes = lanes[0];
    // untuned: 6 blocks per SM; the refined gather always takes 8 (64 registers: 173 ms on the
    // outdoor scene against 178 ms at 80 registers and 173 ms at 48, its binary64 re-tests spill)
    best.minb = refine ? 8u : c.gather_min_blocks ? c.gather_min_blocks : 6u;
    best.buffered = gather_buffer(s.host, best.lanes);
    best.blocks = blocks_for(best.minb, best.lanes);
    if (c.no_autotune || !every || lanes.size() * minbs.size() == 1 || (progress && progress->cancel))
        return best;
    TuneKey key{s.device, ba.items, bpairs, 0, s.host.occ_mesh.size(), s.host.bvh_node_count, best.stack_depth,
                refine ? 2u : 0u, c.blocks_per_sm | (c.sample_lanes << 16), c.gather_min_blocks};
    {
        std::lock_guard<std::mutex> guard(g_tune_lock);
        auto it = g_gather_cache.find(key);
        if (it != g_gather_cache.end()) {
            GatherTune hit = it->second;
            hit.trials = 0;
            hit.ms = 0.0;
            return hit;
        }
    }
    cudaStream_t st = s.stream;
    ba.ctr = s.pool.get<Counters>("tune_counters", 1);
    ba.sample_every = every;
    ba.stack_depth = best.stack_depth;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    auto t0 = std::chrono::steady_clock::now();
    // One launch of a candidate shape over the sampled steps (every >= 2) or the whole queue.
    auto trial = [&](uint32_t minb, uint32_t w, uint32_t sample) {
        const uint32_t blocks = blocks_for(minb, w);
        ba.lanes = w;
        ba.buffered = gather_buffer(s.host, w);
        ba.scratch = gather_scratch(s, blocks, w, ba.buffered);
        ba.sample_every = sample;
        CK(cudaMemsetAsync(ba.head, 0, sizeof(unsigned long long), st));
        CK(cudaEventRecord(a, st));
        gather_kernel(refine, minb)<<<blocks, kBlock, gather_smem(best.stack_depth, w, ba.buffered), st>>>(s.sc,
                                                                                                            ba);
        CK(cudaGetLastError());
        CK(cudaEventRecord(b, st));
        CK(cudaEventSynchronize(b));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, a, b));
        ++best.trials;
        return ms;
    };
    // The sampled trials shortlist two shapes; those two then run over the whole queue, and the
    // faster wins. A sample has few steps per warp, so its load balance favours the finer
    // shapes more than the whole pass does (sampled trials alone picked 8 lanes per texel on the
    // outdoor gather, 3 % slower than the 4 lanes the whole pass prefers). More resident warps
    // hide more of the traversal's latency and fewer registers spill more: on the outdoor gather
    // 10 blocks per SM ran in 93.4 ms, 9 in 94.3, 8 in 97.1, 12 (40 registers) in 102.3.
    struct Candidate {
        float ms;
        uint32_t minb, w;
    };
    auto by_ms = [](const Candidate &x, const Candidate &y) { return x.ms < y.ms; };
    std::vector<Candidate> tried;
    for (uint32_t w : lanes) tried.push_back(Candidate{trial(minbs[0], w, every), minbs[0], w});
    std::stable_sort(tried.begin(), tried.end(), by_ms);
    const size_t lane_picks = std::min<size_t>(2, tried.size());
    for (size_t m = 1; m < minbs.size(); ++m)
        for (size_t k = 0; k < lane_picks; ++k)
            tried.push_back(Candidate{trial(minbs[m], tried[k].w, every), minbs[m], tried[k].w});
    std::stable_sort(tried.begin(), tried.end(), by_ms);
    float best_ms = INFINITY;
    for (size_t k = 0; k < std::min<size_t>(2, tried.size()); ++k) {
        const float ms = trial(tried[k].minb, tried[k].w, 1);
        if (ms < best_ms) {
            best_ms = ms;
            best.lanes = tried[k].w;
            best.minb = tried[k].minb;
            best.blocks = blocks_for(tried[k].minb, tried[k].w);
            best.buffered = gather_buffer(s.host, tried[k].w);
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    best.ms = ms_since(t0);
    std::lock_guard<std::mutex> guard(g_tune_lock);
    g_gather_cache[key] = best;
    return best;
}

// Distance cubes, sun maps and sky probes of the run (src/bake/baker.rs:114-152), queued on the
// session's stream; nothing for LightingOnly.
void bake_maps(dl_session &s, bool refine) {
    const HostScene &h = s.host;
    cudaStream_t st = s.stream;
    Pool &P = s.pool;
    s.cube_words = nullptr;
    s.cube_word_count = 0;
    s.sun_setups.clear();
    s.sun_texels.clear();
    s.probe_grid = ProbeGridSetup{};
    s.probe_open = nullptr;
    s.probe_back = nullptr;
    if (s.options.dynamic_geometry == DL_GEOMETRY_LIGHTING_ONLY) return;
    if (h.local_lights) {
        s.cube_word_count = (uint64_t)h.local_lights * 6 * kCubeRes * kCubeRes / 2;
        uint32_t *cubes = P.get<uint32_t>("cube_words", s.cube_word_count);
        (refine ? k_distance_cubes<true> : k_distance_cubes<false>)<<<grid_for(s.cube_word_count), kBlock, 0, st>>>(
            s.sc, h.local_lights, cubes, s.ctr);
        LAUNCHED("k_distance_cubes");
        ++s.launches;
        s.cube_words = cubes;
    }
    bool any_sky = false, sky_alpha = false;
    for (uint32_t slot = h.local_lights; slot < h.lights.size(); ++slot) {
        const DevLight &l = h.lights[slot];
        if (l.shape == DL_SHAPE_SKY) {
            any_sky = true;
            sky_alpha |= (l.flags & kLightAlpha) != 0;
        }
        if (l.shape != DL_SHAPE_SUN) continue;
        SunMapSetup m = sun_map_setup(h, slot, s.options.sun_map_resolution);
        const uint32_t *texels = nullptr;
        if (!m.empty) {
            SunMapArgs a{};
            a.side = m.side;
            a.up = m.up;
            a.along = m.along;
            a.bmin = m.bmin;
            a.texel = m.texel;
            a.depth = m.depth;
            a.res = m.resolution;
            a.words = (uint32_t)(((uint64_t)m.resolution * m.resolution + 1) / 2);
            a.alpha = (l.flags & kLightAlpha) != 0;
            a.out = P.get<uint32_t>("sun_map_" + std::to_string(s.sun_setups.size()), a.words);
            (refine ? k_sun_map<true> : k_sun_map<false>)<<<grid_for(a.words), kBlock, 0, st>>>(s.sc, a, s.ctr);
            LAUNCHED("k_sun_map");
            ++s.launches;
            texels = a.out;
        }
        s.sun_setups.push_back(m);
        s.sun_texels.push_back(texels);
    }
    if (any_sky) {
        s.probe_grid = sky_probe_grid(h, s.options.sky_probe_spacing);
        if (s.probe_grid.present) {
            ProbeArgs a{};
            a.origin = s.probe_grid.origin;
            a.spacing = s.probe_grid.spacing;
            a.cx = s.probe_grid.counts[0];
            a.cy = s.probe_grid.counts[1];
            a.alpha = sky_alpha;
            a.jobs = s.probe_grid.count() * 6;
            a.open = P.get<float>("probe_open", a.jobs);
            a.back = P.get<uint32_t>("probe_back", a.jobs);
            (refine ? k_sky_probes<true> : k_sky_probes<false>)<<<grid_for(a.jobs), kBlock, 0, st>>>(s.sc, a, s.ctr);
            LAUNCHED("k_sky_probes");
            ++s.launches;
            s.probe_open = a.open;
            s.probe_back = a.back;
        }
    }
}

dl_status run(dl_session &s, dl_progress *progress) {
    DevScene &sc = s.sc;
    const uint32_t T = sc.triangles, M = sc.mesh_count, L = sc.light_count;
    Pool &P = s.pool;
    cudaStream_t st = s.stream;
    const bool refine = s.config.form == DL_FORM_REFINED;
    // the refined predicates and compensated sums for the bounce stages only (photon cubes and
    // gathers): masks stay the bit-exact forms', bounce follows the refined form
    const bool refine_bounce = refine || s.config.form == DL_FORM_BOUNCE_REFINED;
    s.launches = 0;
    s.have_result = false;
    s.bounce_woff = nullptr;
    s.bounce_map = nullptr;
    s.region_rect = nullptr;
    if (progress && progress->cancel) return DL_CANCELLED;
    if (progress) {
        progress->stage = 2;  // BakeStage::Meshes (src/bake/progress.rs:8-16)
        progress->total = M;
        progress->done = 0;
    }
    auto check_cancel = [&]() { return progress && progress->cancel; };
    cudaEvent_t e0, e1, v0, v1, g0, g1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventCreate(&v0));
    CK(cudaEventCreate(&v1));
    CK(cudaEventCreate(&g0));
    CK(cudaEventCreate(&g1));
    struct EventGuard {
        cudaEvent_t *e[6];
        ~EventGuard() {
            for (auto *x : e) cudaEventDestroy(*x);
        }
    } guard{{&e0, &e1, &v0, &v1, &g0, &g1}};
    bool gathered = false;
    CK(cudaEventRecord(e0, st));
    CK(cudaMemsetAsync(s.ctr, 0, sizeof(Counters), st));
    CK(cudaMemsetAsync(s.cancel_dev, 0, 4, st));
    s.report.photon_rays = 0;
    s.report.tuned_chunk_texels = s.report.tuned_sample_lanes = s.report.tuned_blocks_per_sm = 0;
    s.report.tuned_stack_depth = s.report.tuned_min_blocks = s.report.tune_trials = 0;
    s.report.ms_tune = 0.0;
    s.report.tuned_gather_lanes = s.report.tuned_gather_min_blocks = s.report.tuned_gather_blocks_per_sm = 0;
    s.report.cancel_stops = 0;
    s.report.bounce_items = 0;
    if (T == 0) {
        // no triangles: every mesh serializes to no words (triangle_words.rs:47-56)
        CK(cudaEventRecord(v0, st));
        CK(cudaEventRecord(v1, st));
        s.launches = 0;
        bake_maps(s, refine);
        CK(cudaEventRecord(e1, st));
        CK(cudaStreamSynchronize(st));
        s.mesh_words.assign(M + 1, 0);
        s.counters = Counters{};
        s.out_words = 0;
        s.words_dev = nullptr;
        s.texels = 0;
        s.report.ms_device = s.report.ms_visibility = s.report.ms_gather = 0.0;
        s.report.pairs = 0;
        s.report.kernel_launches = s.launches;
        s.have_result = true;
        return DL_OK;
    }

    CK(cudaEventRecord(s.marks[0], st));
    // ---- setup + association
    float4 *tri_face = P.get<float4>("tri_face", T);
    uint4 *tri_crop = P.get<uint4>("tri_crop", T);
    uint32_t *tri_cnt = P.get<uint32_t>("tri_cnt", T + 1);
    uint32_t *tri_off = P.get<uint32_t>("tri_off", T + 1);
    CK(cudaMemsetAsync(tri_cnt + T, 0, 4, st));
    if (T) {
        k_setup<<<grid_for(T), kBlock, 0, st>>>(sc, tri_face, tri_crop, tri_cnt);
        LAUNCHED("k_setup");
        ++s.launches;
    }
    scan_u32(s, tri_cnt, tri_off, T + 1);
    const uint32_t pairs = read_back(s, tri_off + T);
    const size_t entries = (size_t)M * L;
    uint32_t *pair_light = P.get<uint32_t>("pair_light", pairs);
    uint32_t *pair_tri = P.get<uint32_t>("pair_tri", pairs);
    uint32_t *region_rect = P.get<uint32_t>("region_rect", entries * 4);
    if (entries) {
        k_fill_u32<<<grid_for(entries * 4), kBlock, 0, st>>>(region_rect, entries * 4, kNoRect, 0u);
        LAUNCHED("k_fill_u32");
        ++s.launches;
    }
    if (T) {
        k_assoc_fill<<<grid_for(T), kBlock, 0, st>>>(sc, tri_face, tri_crop, tri_off, pair_light, pair_tri,
                                                     region_rect);
        LAUNCHED("k_assoc_fill");
        ++s.launches;
    }
    uint32_t *region_words = P.get<uint32_t>("region_words", entries + 1);
    uint32_t *region_off = P.get<uint32_t>("region_off", entries + 1);
    k_region_words<<<grid_for(entries + 1), kBlock, 0, st>>>(region_rect, sc.lights, (uint32_t)entries, L ? L : 1,
                                                             region_words);
    LAUNCHED("k_region_words");
    ++s.launches;
    scan_u32(s, region_words, region_off, entries + 1);
    const uint32_t region_total = read_back(s, region_off + entries);
    uint32_t *region_pool = P.get<uint32_t>("region_pool", region_total);
    CK(cudaMemsetAsync(region_pool, 0, region_total * 4ull, st));

    CK(cudaEventRecord(s.marks[1], st));
    // ---- texels
    uint64_t *grid_off = P.get<uint64_t>("grid_off", M + 1);
    CK(cudaMemcpyAsync(grid_off, s.grid_off.data(), (M + 1) * 8ull, cudaMemcpyHostToDevice, st));
    uint32_t *owned = P.get<uint32_t>("owned", s.grid_words);
    uint32_t *visited = P.get<uint32_t>("visited", s.grid_words);
    CK(cudaMemsetAsync(owned, 0, s.grid_words * 4, st));
    CK(cudaMemsetAsync(visited, 0, s.grid_words * 4, st));
    uint32_t *cen = P.get<uint32_t>("cen", T + 1);
    uint32_t *tou = P.get<uint32_t>("tou", T + 1);
    uint32_t *tex_cnt = P.get<uint32_t>("tex_cnt", T + 1);
    uint32_t *tex_off = P.get<uint32_t>("tex_off", T + 1);
    const unsigned warp_grid = grid_for((size_t)T * 32);
    if (T) {
        k_texels<0><<<warp_grid, kBlock, 0, st>>>(sc, tri_face, owned, grid_off, cen, nullptr, nullptr, nullptr,
                                                  nullptr, nullptr);
        LAUNCHED("k_texels");
        k_texels<1><<<warp_grid, kBlock, 0, st>>>(sc, tri_face, owned, grid_off, tou, nullptr, nullptr, nullptr,
                                                  nullptr, nullptr);
        LAUNCHED("k_texels");
        s.launches += 2;
    }
    k_add_u32<<<grid_for(T + 1), kBlock, 0, st>>>(cen, tou, tex_cnt, T);
    LAUNCHED("k_add_u32");
    ++s.launches;
    scan_u32(s, tex_cnt, tex_off, T + 1);
    const uint32_t texels_all = read_back(s, tex_off + T);
    uint32_t *tex_xy = P.get<uint32_t>("tex_xy", texels_all);
    float4 *tex_pos = P.get<float4>("tex_pos", texels_all);
    float4 *tex_nrm = P.get<float4>("tex_nrm", texels_all);
    uint32_t *tex_tri = P.get<uint32_t>("tex_tri", texels_all);
    uint8_t *buried = P.get<uint8_t>("buried", texels_all);
    if (T) {
        k_texels<2><<<warp_grid, kBlock, 0, st>>>(sc, tri_face, owned, grid_off, nullptr, tex_off, tex_xy, tex_pos,
                                                  tex_nrm, tex_tri);
        LAUNCHED("k_texels");
        ++s.launches;
    }
    CK(cudaEventRecord(s.marks[2], st));
    if (texels_all) {
        auto burial = refine ? k_burial<true> : k_burial<false>;
        burial<<<grid_for(texels_all), kBlock, 0, st>>>(sc, texels_all, tex_xy, tex_pos, tex_tri, tri_face, buried,
                                                        s.ctr);
        LAUNCHED("k_burial");
        ++s.launches;
    }
    uint32_t *ctex_cnt = P.get<uint32_t>("ctex_cnt", T + 1);
    uint32_t *ctex_off = P.get<uint32_t>("ctex_off", T + 1);
    CK(cudaMemsetAsync(ctex_cnt + T, 0, 4, st));
    if (T) {
        k_unburied<false><<<warp_grid, kBlock, 0, st>>>(T, tex_off, buried, ctex_cnt, nullptr, nullptr, nullptr,
                                                        nullptr, nullptr, nullptr, nullptr);
        LAUNCHED("k_unburied");
        ++s.launches;
    }
    scan_u32(s, ctex_cnt, ctex_off, T + 1);
    const uint32_t texels = read_back(s, ctex_off + T);
    uint32_t *ctex_xy = P.get<uint32_t>("ctex_xy", texels);
    float4 *ctex_pos = P.get<float4>("ctex_pos", texels);
    float4 *ctex_nrm = P.get<float4>("ctex_nrm", texels);
    if (T) {
        k_unburied<true><<<warp_grid, kBlock, 0, st>>>(T, tex_off, buried, nullptr, ctex_off, tex_xy, tex_pos,
                                                       tex_nrm, ctex_xy, ctex_pos, ctex_nrm);
        LAUNCHED("k_unburied");
        ++s.launches;
    }
    s.texels = texels;
    if (check_cancel()) return DL_CANCELLED;

    CK(cudaEventRecord(s.marks[3], st));
    // ---- visibility
    TraceArgs ta{};
    ta.pair_tri = pair_tri;
    ta.pair_light = pair_light;
    ta.ctex_off = ctex_off;
    ta.ctex_xy = ctex_xy;
    ta.ctex_pos = ctex_pos;
    ta.ctex_nrm = ctex_nrm;
    ta.tri_face = tri_face;
    ta.grid_off = grid_off;
    ta.visited = visited;
    ta.region_rect = region_rect;
    ta.region_off = region_off;
    ta.region_pool = region_pool;
    ta.ctr = s.ctr;
    ta.cancel = s.cancel_dev;
    if (s.config.form == DL_FORM_PLAIN) {
        CK(cudaEventRecord(v0, st));
        for (uint32_t m = 0; m < M; ++m) {
            uint32_t first = s.mesh_tri_base[m], count = s.mesh_tri_base[m + 1] - first;
            if (!count) continue;
            unsigned blocks = (unsigned)std::min<size_t>(grid_for((size_t)count * 32), (size_t)s.sms * 16);
            k_trace_plain<<<blocks, kBlock, 0, st>>>(sc, ta, first, count, tri_off);
            LAUNCHED("k_trace_plain");
            ++s.launches;
            if (progress) progress->done = m + 1;
        }
        CK(cudaEventRecord(v1, st));
    } else {
        // queue: pairs ordered sky, soft, hard; item prefix sums over their texel counts
        uint32_t *order = P.get<uint32_t>("order", pairs + 1);
        uint32_t *flag = P.get<uint32_t>("flag", pairs + 1);
        uint32_t *fpos = P.get<uint32_t>("fpos", pairs + 1);
        uint32_t base = 0, sky_pairs = 0;
        for (uint32_t c = 0; c < 3; ++c) {
            k_pair_class<<<grid_for(pairs + 1), kBlock, 0, st>>>(sc, pair_light, pairs, c, flag);
            LAUNCHED("k_pair_class");
            scan_u32(s, flag, fpos, pairs + 1);
            k_pair_scatter<<<grid_for(pairs), kBlock, 0, st>>>(flag, fpos, pairs, base, order);
            LAUNCHED("k_pair_scatter");
            s.launches += 2;
            base += read_back(s, fpos + pairs);
            if (c == 0) sky_pairs = base;
        }
        uint32_t *icnt = P.get<uint32_t>("icnt", pairs + 1);
        uint32_t *item_off = P.get<uint32_t>("item_off", pairs + 1);
        k_item_counts<<<grid_for(pairs + 1), kBlock, 0, st>>>(order, pair_tri, ctex_off, pairs, icnt);
        LAUNCHED("k_item_counts");
        ++s.launches;
        scan_u32(s, icnt, item_off, pairs + 1);
        const uint32_t items = read_back(s, item_off + pairs);
        const uint32_t sky_items = sky_pairs ? read_back(s, item_off + sky_pairs) : 0;
        s.report.work_items = items;
        unsigned long long *heads = P.get<unsigned long long>("heads", 2);
        ta.order = order;
        ta.item_off = item_off;
        ta.pairs = pairs;
        ta.items = items;
        ta.head = heads;
        ta.head_sky = heads + 1;
        ta.sky_items = sky_items;
        ta.sample_every = 1;
        const bool count = s.config.count_visits != 0;  // instrumented variant: counts node visits
        TraceTune tune = trace_tune(s, ta, refine, count, progress);
        s.report.tuned_chunk_texels = tune.grab * 32;
        s.report.tuned_sample_lanes = tune.sky_lanes;
        s.report.tuned_blocks_per_sm = tune.blocks / (uint32_t)s.sms;
        s.report.tuned_stack_depth = tune.stack_depth;
        s.report.tuned_min_blocks = tune.minb;
        s.report.tune_trials = tune.trials;
        s.report.ms_tune = tune.ms;
        ta.grab = tune.grab;
        ta.sky_lanes = tune.sky_lanes;
        auto trace = trace_kernel(count, refine, tune.minb);
        const size_t smem = (size_t)tune.stack_depth * kBlock * sizeof(int);
        const unsigned blocks = tune.blocks;
        // The visibility stage runs from a CUDA graph: the memset of the queue heads and the
        // persistent kernel, captured once per queue layout and launch shape and replayed.
        const uint64_t shape = ((uint64_t)tune.grab << 40) ^ ((uint64_t)tune.sky_lanes << 32) ^
                               ((uint64_t)tune.minb << 24) ^ ((uint64_t)tune.stack_depth << 16) ^ (count ? 1 : 0) ^
                               (refine ? 2 : 0);
        if (!s.graph || s.graph_generation != P.generation || s.graph_items != items || s.graph_blocks != blocks ||
            s.graph_shape != shape) {
            if (s.graph) cudaGraphExecDestroy(s.graph);
            s.graph = nullptr;
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            cudaMemsetAsync(heads, 0, 2 * sizeof(unsigned long long), st);
            if (items) trace<<<blocks, kBlock, smem, st>>>(sc, ta);
            CK(cudaStreamEndCapture(st, &g));
            CK(cudaGraphInstantiate(&s.graph, g, 0));
            cudaGraphDestroy(g);
            s.graph_generation = P.generation;
            s.graph_items = items;
            s.graph_blocks = blocks;
            s.graph_shape = shape;
        }
        CK(cudaEventRecord(v0, st));
        CK(cudaGraphLaunch(s.graph, st));
        if (items) ++s.launches;
        CK(cudaEventRecord(v1, st));
    }
    wait(s, progress);
    if (check_cancel()) return cancelled_run(s);

    CK(cudaEventRecord(s.marks[4], st));
    // ---- one bounce: photon cubes, gathers, bounce maps (bounce.rs:48-217)
    const HostScene &hs = s.host;
    uint8_t *pair_bounce = P.get<uint8_t>("pair_bounce", pairs);
    CK(cudaMemsetAsync(pair_bounce, 0, pairs, st));
    uint32_t *woff = nullptr;
    float4 *bmap = nullptr;
    if (hs.bounce_in_scene && pairs) {
        const uint32_t res = s.options.photon_cube_resolution;
        const uint32_t cubes = (uint32_t)hs.cube_lights.size();
        const uint64_t photons_n = 6ull * res * res * cubes;
        Photon *photons = P.get<Photon>("photons", photons_n);
        if (cubes) {
            uint32_t *cube_lights = P.get<uint32_t>("cube_lights", cubes);
            CK(cudaMemcpyAsync(cube_lights, hs.cube_lights.data(), cubes * 4ull, cudaMemcpyHostToDevice, st));
            auto photon = refine_bounce ? k_photons<true> : k_photons<false>;
            photon<<<grid_for(photons_n), kBlock, 0, st>>>(sc, cube_lights, cubes, res, photons, s.ctr);
            LAUNCHED("k_photons");
            ++s.launches;
        }
        s.report.photon_rays = photons_n;
        uint32_t *bflag = P.get<uint32_t>("bflag", pairs + 1);
        uint32_t *bpos = P.get<uint32_t>("bpos", pairs + 1);
        k_bounce_flag<<<grid_for(pairs + 1), kBlock, 0, st>>>(sc, pair_light, pairs, bflag);
        LAUNCHED("k_bounce_flag");
        scan_u32(s, bflag, bpos, pairs + 1);
        const uint32_t bcount = read_back(s, bpos + pairs);
        uint32_t *bpairs = P.get<uint32_t>("bpairs", bcount + 1);
        k_pair_scatter<<<grid_for(pairs), kBlock, 0, st>>>(bflag, bpos, pairs, 0, bpairs);
        LAUNCHED("k_pair_scatter");
        uint32_t *bcnt = P.get<uint32_t>("bcnt", bcount + 1);
        uint32_t *bitem_off = P.get<uint32_t>("bitem_off", bcount + 1);
        k_item_counts<<<grid_for(bcount + 1), kBlock, 0, st>>>(bpairs, pair_tri, ctex_off, bcount, bcnt);
        LAUNCHED("k_item_counts");
        scan_u32(s, bcnt, bitem_off, bcount + 1);
        const uint32_t bitems = read_back(s, bitem_off + bcount);
        s.report.bounce_items = bitems;
        s.launches += 3;
        float4 *bval = P.get<float4>("bval", bitems);
        BounceArgs ba{};
        ba.pair_tri = pair_tri;
        ba.pair_light = pair_light;
        ba.ctex_off = ctex_off;
        ba.ctex_xy = ctex_xy;
        ba.ctex_pos = ctex_pos;
        ba.tri_face = tri_face;
        ba.bpairs = bpairs;
        ba.bitem_off = bitem_off;
        ba.bpair_count = bcount;
        ba.items = bitems;
        ba.photons = photons;
        ba.res = res;
        ba.value = bval;
        ba.ctr = s.ctr;
        ba.cancel = s.cancel_dev;
        if (bitems) {
            ba.head = P.get<unsigned long long>("gather_head", 1);
            ba.sample_every = 1;
            GatherTune g = gather_tune(s, ba, bcount, refine_bounce, progress);
            ba.lanes = g.lanes;
            ba.stack_depth = g.stack_depth;
            ba.buffered = g.buffered;
            ba.scratch = gather_scratch(s, g.blocks, g.lanes, g.buffered);
            s.report.tuned_gather_lanes = g.lanes;
            s.report.tuned_gather_min_blocks = g.minb;
            s.report.tuned_gather_blocks_per_sm = g.blocks / (uint32_t)s.sms;
            s.report.tune_trials += g.trials;
            s.report.ms_tune += g.ms;
            CK(cudaMemsetAsync(ba.head, 0, sizeof(unsigned long long), st));
            // the instrumented variant (counting node visits and triangle tests) when asked
            CK(cudaEventRecord(g0, st));
            gather_kernel(refine_bounce, g.minb, s.config.count_visits != 0 && !refine_bounce)<<<
                g.blocks, kBlock, gather_smem(g.stack_depth, g.lanes, g.buffered), st>>>(sc, ba);
            LAUNCHED("k_gather");
            CK(cudaEventRecord(g1, st));
            gathered = true;
            ++s.launches;
        }
        // windows per (mesh, bounce light)
        uint32_t *wsize = P.get<uint32_t>("wsize", entries + 1);
        woff = P.get<uint32_t>("woff", entries + 1);
        k_window_sizes<<<grid_for(entries + 1), kBlock, 0, st>>>(sc, region_rect, (uint32_t)entries, wsize);
        LAUNCHED("k_window_sizes");
        scan_u32(s, wsize, woff, entries + 1);
        const uint32_t wtotal = read_back(s, woff + entries);
        uint32_t *owner = P.get<uint32_t>("owner", wtotal);
        float4 *mapA = P.get<float4>("mapA", wtotal);
        bmap = P.get<float4>("mapB", wtotal);
        CK(cudaMemsetAsync(owner, 0, wtotal * 4ull, st));
        CK(cudaMemsetAsync(mapA, 0, wtotal * 16ull, st));
        if (bitems) {
            k_bounce_scatter<false><<<grid_for(bitems), kBlock, 0, st>>>(sc, ba, region_rect, woff, owner, mapA);
            LAUNCHED("k_bounce_scatter");
            k_bounce_scatter<true><<<grid_for(bitems), kBlock, 0, st>>>(sc, ba, region_rect, woff, owner, mapA);
            LAUNCHED("k_bounce_scatter");
            s.launches += 2;
        }
        const float *bw = hs.blur_weights;
        k_bounce_filter<<<(unsigned)entries, 256, 0, st>>>(sc, region_rect, woff, wsize, mapA, bmap, bw[0], bw[1], bw[2],
                                                           bw[3], bw[4], bw[5], bw[6], hs.blur_weight_sum);
        LAUNCHED("k_bounce_filter");
        if (bcount) {
            k_bounce_lit<<<grid_for((size_t)bcount * 32), kBlock, 0, st>>>(sc, ba, tri_crop, region_rect, woff, bmap,
                                                                           pair_bounce);
            LAUNCHED("k_bounce_lit");
            ++s.launches;
        }
        s.launches += 3;
    }

    CK(cudaEventRecord(s.marks[5], st));
    // ---- optimize, seams
    uint8_t *keep = P.get<uint8_t>("keep", pairs);
    uint32_t *kept_cnt = P.get<uint32_t>("kept_cnt", T + 1);
    uint32_t *entry_off = P.get<uint32_t>("entry_off", T + 1);
    uint8_t *used = P.get<uint8_t>("used", entries);
    CK(cudaMemsetAsync(used, 0, entries, st));
    CK(cudaMemsetAsync(kept_cnt, 0, (T + 1) * 4ull, st));
    if (pairs) {
        k_optimize<<<grid_for((size_t)pairs * 32), kBlock, 0, st>>>(sc, pairs, pair_tri, pair_light, region_rect,
                                                                    region_off, region_pool, pair_bounce, keep, kept_cnt,
                                                                    used, s.ctr);
        LAUNCHED("k_optimize");
        ++s.launches;
    }
    if (entries) {
        k_pad_seams<<<(unsigned)entries, kBlock, 0, st>>>(sc, used, region_rect, region_off, region_pool, visited,
                                                          grid_off);
        LAUNCHED("k_pad_seams");
        ++s.launches;
    }
    scan_u32(s, kept_cnt, entry_off, T + 1);
    const uint32_t kept = read_back(s, entry_off + T);

    CK(cudaEventRecord(s.marks[6], st));
    // ---- serialize
    const uint32_t stride = s.host.bounce_in_scene ? 3 : 2;
    unsigned long long *ld_words = P.get<unsigned long long>("ld_words", T + 1);
    unsigned long long *pl_words = P.get<unsigned long long>("pl_words", T + 1);
    unsigned long long *ld_scan = P.get<unsigned long long>("ld_scan", T + 1);
    unsigned long long *pl_scan = P.get<unsigned long long>("pl_scan", T + 1);
    k_tri_words<<<grid_for(T + 1), kBlock, 0, st>>>(sc, tri_off, pair_light, keep, pair_bounce, tri_crop, stride,
                                                    ld_words, pl_words);
    LAUNCHED("k_tri_words");
    ++s.launches;
    scan_u64(s, ld_words, ld_scan, T + 1);
    scan_u64(s, pl_words, pl_scan, T + 1);
    unsigned long long *mesh_words = P.get<unsigned long long>("mesh_words", M + 1);
    unsigned long long *mesh_base = P.get<unsigned long long>("mesh_base", M + 1);
    k_mesh_words<<<grid_for(M + 1), kBlock, 0, st>>>(sc, ld_scan, pl_scan, mesh_words);
    LAUNCHED("k_mesh_words");
    ++s.launches;
    scan_u64(s, mesh_words, mesh_base, M + 1);
    const unsigned long long total_words = read_back(s, mesh_base + M);
    uint32_t *words = P.get<uint32_t>("words", total_words);
    uint32_t *entry_pair = P.get<uint32_t>("entry_pair", kept);
    unsigned long long *entry_dst = P.get<unsigned long long>("entry_dst", kept);
    unsigned long long *entry_bdst = P.get<unsigned long long>("entry_bdst", kept);
    if (T) {
        k_serialize<<<grid_for(T), kBlock, 0, st>>>(sc, tri_off, pair_light, keep, pair_bounce, tri_crop, stride, ld_scan,
                                                    pl_scan, mesh_base, entry_off, words, entry_pair, entry_dst,
                                                    entry_bdst);
        LAUNCHED("k_serialize");
        ++s.launches;
    }
    if (kept) {
        k_crop<<<grid_for((size_t)kept * 32), kBlock, 0, st>>>(sc, kept, entry_pair, entry_dst, pair_tri, pair_light,
                                                               tri_crop, region_rect, region_off, region_pool, words);
        LAUNCHED("k_crop");
        ++s.launches;
        if (bmap) {
            k_pack_bounce<<<grid_for(kept), kBlock, 0, st>>>(sc, kept, entry_pair, entry_bdst, pair_tri, pair_light,
                                                             tri_crop, region_rect, woff, bmap, words);
            LAUNCHED("k_pack_bounce");
            k_pack_bounce8<<<grid_for((size_t)kept * 32), kBlock, 0, st>>>(
                sc, kept, entry_pair, entry_bdst, pair_tri, pair_light, tri_crop, region_rect, woff, bmap, words);
            LAUNCHED("k_pack_bounce8");
            s.launches += 2;
        }
    }
    CK(cudaEventRecord(s.marks[7], st));
    // ---- maps for moving meshes
    bake_maps(s, refine);
    CK(cudaEventRecord(s.marks[8], st));
    CK(cudaEventRecord(e1, st));
    s.mesh_words.resize(M + 1);
    CK(cudaMemcpyAsync(s.mesh_words.data(), mesh_words, (M + 1) * 8ull, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&s.counters, s.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    wait(s, progress);
    if (check_cancel()) return cancelled_run(s);
    float ms = 0.0f, vms = 0.0f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    CK(cudaEventElapsedTime(&vms, v0, v1));
    s.report.ms_device = ms;
    s.report.ms_visibility = vms;
    float gms = 0.0f;
    if (gathered) CK(cudaEventElapsedTime(&gms, g0, g1));
    s.report.ms_gather = gms;
    for (int k = 0; k < 8; ++k) {
        float ms_k = 0.0f;
        CK(cudaEventElapsedTime(&ms_k, s.marks[k], s.marks[k + 1]));
        s.report.ms_stages[k] = ms_k;
    }
    s.report.pairs = pairs;
    s.report.shadow_rays = s.counters.rays;
    s.report.burial_rays = s.counters.burial_rays;
    s.report.bounce_rays = s.counters.bounce_rays;
    s.report.node_visits = s.counters.node_visits;
    s.report.tri_tests = s.counters.tri_tests;
    s.report.gather_node_visits = s.counters.gather_node_visits;
    s.report.gather_tri_tests = s.counters.gather_tri_tests;
    s.report.retests = s.counters.retests;
    s.report.kernel_launches = s.launches;
    s.report.device_bytes = s.scene_bytes + P.bytes;
    s.out_words = total_words;
    s.words_dev = words;
    s.bounce_woff = woff;
    s.bounce_map = bmap;
    s.region_rect = region_rect;
    s.have_result = true;
    if (progress) {  // BakeStage::Done with its counters cleared, as progress.begin(Done, 0) leaves them
        progress->done = 0;
        progress->total = 0;
        progress->stage = 4;
    }
    return DL_OK;
}

// The result in one host allocation: the scene struct, its arrays, then the words.
struct HostResult {
    dl_baked_scene scene;
    std::vector<dl_baked_light> lights;
    std::vector<dl_light_bvh_node> bvh;
    std::vector<dl_baked_mesh> meshes;
    uint32_t *words = nullptr;  // buffer.p
    WordCache::Buffer buffer{0, nullptr, false};  // from word_cache()
    ~HostResult() {
        if (buffer.p) word_cache().give(buffer);
    }
    std::vector<uint32_t> cubes;
    std::vector<std::vector<uint32_t>> sun_words;
    std::vector<dl_sun_map> sun_maps;
    std::vector<uint32_t> probe_words;
    dl_sky_probes probes{};
};

// Copies n words into host memory mapped for the device (pinned, written over the CPU-GPU link
// by the SMs): 16-byte stores, the tail word by word.
__global__ void k_copy_words(const uint32_t *src, uint32_t *dst, uint64_t n) {
    const uint64_t n4 = n / 4, stride = (uint64_t)gridDim.x * blockDim.x;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) d4[i] = s4[i];
    for (uint64_t i = n4 * 4 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}

// The last run's scene. With `download` false the triangle words, distance cubes and sun map
// texels stay on the device and the scene's pointers to them are device pointers (for the
// device-side payload encode); everything else is on the host either way.
dl_status assemble(dl_session &s, std::unique_ptr<HostResult> &r, bool download) {
    if (!s.have_result) {
        g_error = "no finished run in this session";
        return DL_INVALID_ARGUMENT;
    }
    r = std::make_unique<HostResult>();
    const HostScene &h = s.host;
    const uint32_t *words = s.words_dev;
    if (download) {
        r->buffer = word_cache().take(s.out_words);
        r->words = r->buffer.p;
        uint32_t *mapped = nullptr;
        if (s.out_words && r->buffer.pinned &&
            cudaHostGetDevicePointer((void **)&mapped, r->words, 0) == cudaSuccess) {
            // the SMs write the words into the pinned buffer: as fast as the copy engine here,
            // and steadier (the copy engine's rate varied 10x between sessions on some machines)
            k_copy_words<<<s.sms * 8, 256, 0, s.stream>>>(s.words_dev, mapped, s.out_words);
            LAUNCHED("k_copy_words");
            CK(cudaStreamSynchronize(s.stream));
        } else if (s.out_words) {
            cudaGetLastError();  // a buffer the device cannot map: the copy engine
            CK(cudaMemcpy(r->words, s.words_dev, s.out_words * 4, cudaMemcpyDeviceToHost));
        }
        words = r->words;
        s.report.d2h_bytes = s.out_words * 4 + (s.mesh_words.size() * 8) + sizeof(Counters);
    }
    uint64_t at = 0;
    for (uint32_t m = 0; m < h.meshes.size(); ++m) {
        const dl_mesh &mm = *h.meshes[m];
        dl_baked_mesh b{};
        b.id = mm.id;
        b.content_hash = mm.content_hash;
        b.resolution = h.resolution[m];
        b.occludes = mm.occludes ? 1 : 0;
        b.triangles = words + at;
        b.word_count = s.mesh_words[m];
        at += s.mesh_words[m];
        r->meshes.push_back(b);
    }
    const dl_bake_options &o = s.options;
    for (size_t i = 0; i < h.light_ptrs.size(); ++i) {
        const dl_light &l = *h.light_ptrs[i];
        const DevLight &d = h.lights[i];
        dl_baked_light b{};
        b.id = l.id;
        for (int k = 0; k < 3; ++k) b.origin[k] = l.position[k];
        b.radius = l.radius;
        b.shape = l.shape;
        // the file's shape record (format/lights.rs:27-52): rotation and size only for area/sun
        bool shaped = l.shape != DL_SHAPE_POINT && l.shape != DL_SHAPE_SKY;
        b.rotation[0] = shaped ? l.rotation[0] : 0.0f;
        b.rotation[1] = shaped ? l.rotation[1] : 0.0f;
        b.rotation[2] = shaped ? l.rotation[2] : 0.0f;
        b.rotation[3] = shaped ? l.rotation[3] : 1.0f;
        b.size[0] = shaped ? l.size[0] : 0.0f;
        b.size[1] = (l.shape == DL_SHAPE_RECTANGLE || l.shape == DL_SHAPE_TUBE) ? l.size[1] : 0.0f;
        b.bounce_bits = d.bounce_bits;
        b.shadow_bits_per_texel = d.shadow_bits;
        r->lights.push_back(b);
    }
    r->bvh = h.light_bvh;
    dl_baked_scene &sc = r->scene;
    sc = dl_baked_scene{};
    sc.settings.bounce = h.bounce_in_scene;
    sc.settings.colored_bounce = h.bounce_in_scene && o.colored_bounce;
    sc.settings.dynamic_geometry = o.dynamic_geometry;
    sc.settings.pixel_density = o.pixel_density;
    sc.settings.max_lightmap_size = o.max_lightmap_size;
    sc.settings.distance_cube_resolution = 64;
    sc.light_count = r->lights.size();
    sc.lights = r->lights.data();
    sc.light_bvh_count = r->bvh.size();
    sc.light_bvh = r->bvh.data();
    sc.mesh_count = r->meshes.size();
    sc.meshes = r->meshes.data();
    // maps for moving meshes
    if (s.cube_word_count && download) {
        r->cubes.resize(s.cube_word_count);
        CK(cudaMemcpy(r->cubes.data(), s.cube_words, s.cube_word_count * 4, cudaMemcpyDeviceToHost));
    }
    std::vector<const uint32_t *> sun_dev;
    for (size_t i = 0; i < s.sun_setups.size(); ++i) {
        const SunMapSetup &m = s.sun_setups[i];
        dl_sun_map d{};
        std::vector<uint32_t> texels;
        const uint32_t *dev = nullptr;
        if (m.empty) {
            texels.assign(1, 0xFFFFFFFFu);  // pack_sun_depth(1, 1)
            d.resolution = 1;
        } else {
            d.resolution = m.resolution;
            for (int k = 0; k < 12; ++k) d.rows[k] = m.rows[k];
            d.word_count = ((uint64_t)m.resolution * m.resolution + 1) / 2;
            if (download) {
                texels.resize(d.word_count);
                CK(cudaMemcpy(texels.data(), s.sun_texels[i], texels.size() * 4, cudaMemcpyDeviceToHost));
            } else {
                dev = s.sun_texels[i];
            }
        }
        r->sun_words.push_back(std::move(texels));
        r->sun_maps.push_back(d);
        sun_dev.push_back(dev);
    }
    for (size_t i = 0; i < r->sun_maps.size(); ++i) {
        if (sun_dev[i]) {
            r->sun_maps[i].texels = sun_dev[i];
        } else {
            r->sun_maps[i].word_count = r->sun_words[i].size();
            r->sun_maps[i].texels = r->sun_words[i].data();
        }
    }
    if (s.probe_grid.present) {
        const ProbeGridSetup &g = s.probe_grid;
        std::vector<float> open(g.count() * 6);
        std::vector<uint32_t> back(g.count() * 6);
        CK(cudaMemcpy(open.data(), s.probe_open, open.size() * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(back.data(), s.probe_back, back.size() * 4, cudaMemcpyDeviceToHost));
        r->probe_words = sky_probe_words(g, open.data(), back.data(), o.sky_samples);
        dl_sky_probes &p = r->probes;
        p.origin[0] = g.origin.x;
        p.origin[1] = g.origin.y;
        p.origin[2] = g.origin.z;
        p.spacing = g.spacing;
        for (int k = 0; k < 3; ++k) p.counts[k] = g.counts[k];
        p.word_count = r->probe_words.size();
        p.words = r->probe_words.data();
    }
    if (download) {
        for (const auto &w : r->sun_words) s.report.d2h_bytes += w.size() * 4;
        s.report.d2h_bytes += r->cubes.size() * 4 + (s.probe_grid.present ? s.probe_grid.count() * 6 * 8 : 0);
        sc.distance_cube_words = r->cubes.size();
        sc.distance_cubes = r->cubes.empty() ? nullptr : r->cubes.data();
    } else {
        sc.distance_cube_words = s.cube_word_count;
        sc.distance_cubes = s.cube_words;
    }
    sc.sun_map_count = r->sun_maps.size();
    sc.sun_maps = r->sun_maps.empty() ? nullptr : r->sun_maps.data();
    sc.sky_probes = s.probe_grid.present ? &r->probes : nullptr;
    sc.stats.meshes = (uint32_t)h.meshes.size();
    sc.stats.triangles = h.triangles;
    sc.stats.texels = s.texels;
    sc.stats.rays = s.counters.rays;
    sc.stats.lights_removed = s.counters.lights_removed;
    sc.stats.bounce_rays = s.counters.bounce_rays;
    sc.stats.triangle_words = s.out_words;
    return DL_OK;
}

// Collects the payload as host-written runs and device word arrays (payload order, word units).
struct DeviceSink {
    std::vector<uint32_t> host;         // host-written words, in order
    std::vector<PayloadSegment> segs;   // src of a host run: offset into `host` until uploaded
    std::vector<bool> from_host;
    unsigned long long at = 0;          // payload words so far
    void run(uint32_t v) {
        if (segs.empty() || !from_host.back() || segs.back().dst + segs.back().len != at) {
            segs.push_back(PayloadSegment{at, reinterpret_cast<const uint32_t *>(host.size()), 0});
            from_host.push_back(true);
        }
        host.push_back(v);
        ++segs.back().len;
        ++at;
    }
    void u32(uint32_t v) { run(v); }
    void u64(uint64_t v) {
        run((uint32_t)v);
        run((uint32_t)(v >> 32));
    }
    void f32(float f) {
        uint32_t v;
        std::memcpy(&v, &f, 4);
        run(v);
    }
    void words(const uint32_t *w, uint64_t n) {
        u64(n);
        if (!n) return;
        cudaPointerAttributes attr{};
        bool device = cudaPointerGetAttributes(&attr, w) == cudaSuccess && attr.type == cudaMemoryTypeDevice;
        cudaGetLastError();  // a host pointer may leave an error behind on older drivers
        if (!device) {
            for (uint64_t i = 0; i < n; ++i) run(w[i]);
            return;
        }
        segs.push_back(PayloadSegment{at, w, n});
        from_host.push_back(false);
        at += n;
    }
};

// dl_session_encode_payload: the payload of the last run built on the device, its CRC-32 from
// per-chunk CRCs combined on the host.
dl_status encode_device(dl_session &s, uint8_t *&bytes, uint64_t &length, uint32_t &crc) {
    std::unique_ptr<HostResult> r;
    dl_status st = assemble(s, r, false);
    if (st != DL_OK) return st;
    DeviceSink sink;
    emit_payload(r->scene, sink);
    const unsigned long long words = sink.at;
    Pool &P = s.pool;
    cudaStream_t strm = s.stream;
    uint32_t *payload = P.get<uint32_t>("payload", words);
    uint32_t *host_dev = P.get<uint32_t>("payload_host", sink.host.size());
    CK(cudaMemcpyAsync(host_dev, sink.host.data(), sink.host.size() * 4, cudaMemcpyHostToDevice, strm));
    for (size_t i = 0; i < sink.segs.size(); ++i)
        if (sink.from_host[i]) sink.segs[i].src = host_dev + reinterpret_cast<uintptr_t>(sink.segs[i].src);
    PayloadSegment *segs = P.get<PayloadSegment>("payload_segs", sink.segs.size());
    CK(cudaMemcpyAsync(segs, sink.segs.data(), sink.segs.size() * sizeof(PayloadSegment), cudaMemcpyHostToDevice,
                       strm));
    k_payload_gather<<<(unsigned)sink.segs.size(), 256, 0, strm>>>(segs, payload);
    LAUNCHED("k_payload_gather");
    // CRC of the full chunks on the device
    const unsigned long long chunks = words / kCrcChunkWords;
    std::vector<uint32_t> chunk_crc(chunks);
    if (chunks) {
        uint32_t *tables = P.get<uint32_t>("crc_tables", 1024);
        CK(cudaMemcpyAsync(tables, crc32_tables(), 1024 * 4, cudaMemcpyHostToDevice, strm));
        CrcShifts sh{};
        for (int l = 0; l < 7; ++l)
            for (int i = 0; i < 32; ++i) sh.m[l][i] = crc32_shift(1u << i, 512ull << l);
        uint32_t *out = P.get<uint32_t>("chunk_crc", chunks);
        unsigned blocks = (unsigned)std::min<unsigned long long>(chunks, (unsigned long long)s.sms * 16);
        k_crc_chunks<<<blocks, 128, 0, strm>>>(payload, chunks, tables, sh, out);
        LAUNCHED("k_crc_chunks");
        CK(cudaMemcpyAsync(chunk_crc.data(), out, chunks * 4, cudaMemcpyDeviceToHost, strm));
    }
    length = words * 4;
    bytes = static_cast<uint8_t *>(std::malloc(length ? length : 1));
    if (!bytes) throw std::bad_alloc();
    CK(cudaMemcpyAsync(bytes, payload, length, cudaMemcpyDeviceToHost, strm));
    CK(cudaStreamSynchronize(strm));
    uint32_t shift64[32];
    for (int i = 0; i < 32; ++i) shift64[i] = crc32_shift(1u << i, (uint64_t)kCrcChunkWords * 4);
    uint32_t c = 0xFFFFFFFFu;
    for (unsigned long long k = 0; k < chunks; ++k) {
        uint32_t shifted = 0;
        for (int i = 0; i < 32; ++i)
            if ((c >> i) & 1u) shifted ^= shift64[i];
        c = shifted ^ chunk_crc[k];
    }
    uint64_t done = chunks * (uint64_t)kCrcChunkWords * 4;
    c = crc32_update(c, bytes + done, length - done);
    crc = c ^ 0xFFFFFFFFu;
    return DL_OK;
}

dl_status result(dl_session &s, dl_baked_scene *&out) {
    std::unique_ptr<HostResult> r;
    dl_status st = assemble(s, r, true);
    if (st != DL_OK) return st;
    out = &r.release()->scene;
    return DL_OK;
}

}  // namespace
}  // namespace dl

// ================================ C ABI ====================================================

#define DL_GUARD(body)                                                                \
    try {                                                                             \
        body                                                                          \
    } catch (const CudaError &e) {                                                    \
        g_error = std::string(e.what) + ": " + cudaGetErrorString(e.code);            \
        return e.code == cudaErrorMemoryAllocation ? DL_OUT_OF_MEMORY : DL_CUDA_ERROR; \
    } catch (const std::bad_alloc &) {                                                \
        g_error = "host allocation failed";                                           \
        return DL_OUT_OF_MEMORY;                                                      \
    } catch (...) {                                                                   \
        g_error = "unexpected failure";                                               \
        return DL_CUDA_ERROR;                                                         \
    }

// dl_session_create with an optional progress whose cancel flag create() checks.
static dl_status session_create(const dl_bake_input *input, const dl_bake_options *options,
                                const dl_bake_config *config, const dl_progress *progress, dl_session **out) {
    if (!input || !options || !out) {
        g_error = "null argument";
        return DL_INVALID_ARGUMENT;
    }
    *out = nullptr;
    DL_GUARD({
        dl_session *s = nullptr;
        auto t0 = std::chrono::steady_clock::now();
        dl_status st = create(input, options, config, s, progress);
        if (st != DL_OK) return st;
        s->report.ms_upload = ms_since(t0);
        *out = s;
        return DL_OK;
    })
}

extern "C" {

uint32_t dl_abi_version(void) { return DL_ABI_VERSION; }

const char *dl_status_string(dl_status status) {
    switch (status) {
        case DL_OK: return "ok";
        case DL_CANCELLED: return "cancelled";
        case DL_DUPLICATE_ID: return "duplicate id";
        case DL_INVALID_MESH: return "invalid mesh";
        case DL_INVALID_LIGHT: return "invalid light";
        case DL_INVALID_OPTIONS: return "invalid options";
        case DL_CUDA_ERROR: return "cuda error";
        case DL_OUT_OF_MEMORY: return "out of memory";
        case DL_QUEUE_TIMEOUT: return "queue timeout";
        case DL_BUSY: return "busy";
        case DL_UNSUPPORTED: return "unsupported";
        case DL_INVALID_ARGUMENT: return "invalid argument";
    }
    return "unknown";
}

const char *dl_last_error(void) { return g_error.c_str(); }

void dl_default_options(dl_bake_options *o) {
    if (!o) return;
    *o = dl_bake_options{};
    o->pixel_density = 128.0f;
    o->max_lightmap_size = 2048;
    o->bounce_compression = 8;
    o->dynamic_geometry = DL_GEOMETRY_ANGULAR;
    o->skip_bounce = 0;
    o->photon_cube_resolution = 512;
    o->area_light_samples = 64;
    o->area_light_min_samples = 16;
    o->sun_map_resolution = 2048;
    o->sky_samples = 64;
    o->sky_probe_spacing = 1.0f;
    o->colored_bounce = 0;
    o->seed = 0;
}

dl_status dl_session_create(const dl_bake_input *input, const dl_bake_options *options,
                            const dl_bake_config *config, dl_session **out) {
    return session_create(input, options, config, nullptr, out);
}

dl_status dl_session_run(dl_session *s, dl_progress *progress) {
    if (!s) {
        g_error = "null session";
        return DL_INVALID_ARGUMENT;
    }
    DL_GUARD({
        CK(cudaSetDevice(s->device));
        return run(*s, progress);
    })
}

dl_status dl_session_result(dl_session *s, dl_baked_scene **out) {
    if (!s || !out) {
        g_error = "null argument";
        return DL_INVALID_ARGUMENT;
    }
    *out = nullptr;
    DL_GUARD({
        CK(cudaSetDevice(s->device));
        auto t0 = std::chrono::steady_clock::now();
        dl_status st = result(*s, *out);
        s->report.ms_download = ms_since(t0);
        return st;
    })
}

dl_status dl_session_bounce_map(dl_session *s, uint64_t mesh_id, uint32_t slot, uint32_t rect[4], float *rgb,
                                uint32_t cap, uint32_t *texels) {
    if (!s || !rect || !texels || (cap && !rgb)) {
        g_error = "null argument";
        return DL_INVALID_ARGUMENT;
    }
    *texels = 0;
    if (!s->have_result) {
        g_error = "no finished run in this session";
        return DL_INVALID_ARGUMENT;
    }
    const HostScene &h = s->host;
    uint32_t m = 0;
    while (m < h.meshes.size() && h.meshes[m]->id != mesh_id) ++m;
    if (m == h.meshes.size() || slot >= h.lights.size()) {
        g_error = "no such mesh id or light slot";
        return DL_INVALID_ARGUMENT;
    }
    if (!s->bounce_map || !(h.lights[slot].flags & kLightBounce)) return DL_OK;
    DL_GUARD({
        CK(cudaSetDevice(s->device));
        size_t e = (size_t)m * h.lights.size() + slot;
        uint32_t r[4];
        uint32_t off[2];
        CK(cudaMemcpy(r, s->region_rect + e * 4, sizeof r, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(off, s->bounce_woff + e, sizeof off, cudaMemcpyDeviceToHost));
        if (r[0] == kNoRect) return DL_OK;
        Rect w = bounce_window(r, h.resolution[m]);
        rect[0] = w.min_x;
        rect[1] = w.min_y;
        rect[2] = w.max_x;
        rect[3] = w.max_y;
        uint32_t n = off[1] - off[0];
        *texels = n;
        if (cap) {
            std::vector<float4> v(std::min(n, cap));
            CK(cudaMemcpy(v.data(), s->bounce_map + off[0], v.size() * sizeof(float4), cudaMemcpyDeviceToHost));
            for (size_t k = 0; k < v.size(); ++k) {
                rgb[k * 3] = v[k].x;
                rgb[k * 3 + 1] = v[k].y;
                rgb[k * 3 + 2] = v[k].z;
            }
        }
        return DL_OK;
    })
}

dl_status dl_session_occluder_bvh(dl_session *s, void *nodes, uint64_t node_cap, float *triangles,
                                  uint64_t tri_cap, uint32_t *node_count, uint32_t *depth) {
    if (!s || !node_count || !depth || (node_cap && !nodes) || (tri_cap && !triangles)) {
        g_error = "null argument";
        return DL_INVALID_ARGUMENT;
    }
    const HostScene &h = s->host;
    *node_count = h.bvh_node_count;
    *depth = h.bvh_depth;
    DL_GUARD({
        CK(cudaSetDevice(s->device));
        uint64_t n = std::min<uint64_t>(node_cap, h.bvh_node_count);
        if (n) CK(cudaMemcpy(nodes, s->sc.nodes, n * sizeof(BvhNode), cudaMemcpyDeviceToHost));
        uint64_t t = std::min<uint64_t>(tri_cap, s->sc.occluders);
        if (t) CK(cudaMemcpy(triangles, s->sc.tris, t * 3 * sizeof(float4), cudaMemcpyDeviceToHost));
        return DL_OK;
    })
}

dl_status dl_session_encode_payload(dl_session *s, uint8_t **bytes, uint64_t *length, uint32_t *crc) {
    if (!s || !bytes || !length) {
        g_error = "null argument";
        return DL_INVALID_ARGUMENT;
    }
    *bytes = nullptr;
    *length = 0;
    DL_GUARD({
        CK(cudaSetDevice(s->device));
        uint8_t *b = nullptr;
        uint64_t n = 0;
        uint32_t c = 0;
        dl_status st = encode_device(*s, b, n, c);
        if (st != DL_OK) {
            std::free(b);
            return st;
        }
        *bytes = b;
        *length = n;
        if (crc) *crc = c;
        return DL_OK;
    })
}

dl_status dl_session_report(const dl_session *s, dl_bake_report *report) {
    if (!s || !report) {
        g_error = "null argument";
        return DL_INVALID_ARGUMENT;
    }
    *report = s->report;
    return DL_OK;
}

void dl_session_destroy(dl_session *s) { delete s; }

void dl_release_memory(void) {
    word_cache().clear();
    release_pooled_device_memory();
}

void dl_baked_scene_free(dl_baked_scene *scene) { delete reinterpret_cast<HostResult *>(scene); }

dl_status dl_bake_ex(const dl_bake_input *input, const dl_bake_options *options, const dl_bake_config *config,
                     dl_progress *progress, dl_baked_scene **out, dl_bake_report *report) {
    if (!input || !options || !out) {
        g_error = "null argument";
        return DL_INVALID_ARGUMENT;
    }
    *out = nullptr;
    std::unique_lock<std::mutex> lock(g_busy, std::try_to_lock);
    if (!lock.owns_lock()) {
        g_error = "another bake is running in this process";
        return DL_BUSY;
    }
    auto t0 = std::chrono::steady_clock::now();
    if (progress) progress->stage = 0;
    dl_session *s = nullptr;
    dl_status st = session_create(input, options, config, progress, &s);
    if (st != DL_OK) return st;
    std::unique_ptr<dl_session> owner(s);
    st = dl_session_run(s, progress);
    if (st == DL_CANCELLED) {
        g_error = "the bake was cancelled";
        if (report) {
            *report = s->report;
            report->ms_total = ms_since(t0);
        }
    }
    if (st != DL_OK) return st;
    st = dl_session_result(s, out);
    if (report) {
        *report = s->report;
        report->ms_total = ms_since(t0);
    }
    return st;
}

dl_status dl_bake(const dl_bake_input *input, const dl_bake_options *options, dl_progress *progress,
                  dl_baked_scene **out) {
    dl_bake_config cfg{};
    return dl_bake_ex(input, options, &cfg, progress, out, nullptr);
}

dl_status dl_encode_payload(const dl_baked_scene *scene, uint8_t **bytes, uint64_t *length, uint32_t *crc) {
    if (!scene || !bytes || !length) {
        g_error = "null argument";
        return DL_INVALID_ARGUMENT;
    }
    try {
        std::vector<uint8_t> p = encode_payload(*scene);
        uint8_t *b = static_cast<uint8_t *>(std::malloc(p.size() ? p.size() : 1));
        if (!b) {
            g_error = "host allocation failed";
            return DL_OUT_OF_MEMORY;
        }
        if (!p.empty()) std::memcpy(b, p.data(), p.size());
        *bytes = b;
        *length = p.size();
        if (crc) *crc = crc32_ieee(p.data(), p.size());
        return DL_OK;
    } catch (...) {
        g_error = "host allocation failed";
        return DL_OUT_OF_MEMORY;
    }
}

void dl_free(void *p) { std::free(p); }

}  // extern "C"

// ================================ non-allocating bounce filter ============================
//
// dl_filter_bounce_window_noalloc: the bounce map filter of the bake (dilate, then the 7-tap
// separable blur; the body of k_bounce_filter) on one window held in caller-owned device
// buffers, for callers that cannot allocate device memory — an engine applying the filter from
// inside its own fixed memory budget, or from code that must not call cudaMalloc (while a
// stream is being captured, or on a frame thread). The blur's intermediate lives in the
// fixed array below, which every device that loads the library holds until the process exits.

namespace dl {

constexpr uint32_t kNoallocMaxTexels = DL_NOALLOC_MAX_TEXELS;
static __device__ __align__(256) float g_noalloc_scratch[3 * (size_t)kNoallocMaxTexels];

namespace {

constexpr int kNoallocDevices = 64;
std::mutex g_noalloc_mutex;
float *g_noalloc_ptr[kNoallocDevices] = {};

// Dilation (bounce_map.rs:67-87): the first positive texel among itself and its 8 neighbours in
// a fixed order; outside the window reads 0.
__global__ void k_noalloc_dilate(const float *in, float *out, uint32_t w, uint32_t h) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    int x = (int)(i % w), y = (int)(i / w);
    const int order[9][2] = {{0, 0}, {-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
    float r = 0.0f, g = 0.0f, b = 0.0f;
    for (int k = 0; k < 9; ++k) {
        int xx = x + order[k][0], yy = y + order[k][1];
        if (xx < 0 || yy < 0 || xx >= (int)w || yy >= (int)h) continue;
        const float *v = in + ((size_t)yy * w + xx) * 3;
        if (fmaxf(fmaxf(v[0], v[1]), v[2]) > 0.0f) {
            r = v[0];
            g = v[1];
            b = v[2];
            break;
        }
    }
    out[(size_t)i * 3] = r;
    out[(size_t)i * 3 + 1] = g;
    out[(size_t)i * 3 + 2] = b;
}

struct BlurWeights {
    float w[7];
    float sum;
};

// One blur pass (bounce_map.rs:92-112): sample coordinates clamped to the map, reads outside
// the window are 0, sum in tap order, divided by the weights' sum.
__global__ void k_noalloc_blur(const float *src, float *dst, uint32_t w, uint32_t h, uint32_t x0, uint32_t y0,
                               uint32_t map_size, int vertical, BlurWeights bw) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    int64_t x = x0 + (int64_t)(i % w), y = y0 + (int64_t)(i / w);
    int64_t last = (int64_t)map_size - 1;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    for (int k = -3; k <= 3; ++k) {
        int64_t qx = vertical ? x : min(max(x + k, (int64_t)0), last);
        int64_t qy = vertical ? min(max(y + k, (int64_t)0), last) : y;
        float r = 0.0f, g = 0.0f, b = 0.0f;
        if (qx >= (int64_t)x0 && qy >= (int64_t)y0 && qx < (int64_t)x0 + w && qy < (int64_t)y0 + h) {
            const float *v = src + ((size_t)(qy - y0) * w + (size_t)(qx - x0)) * 3;
            r = v[0];
            g = v[1];
            b = v[2];
        }
        sx = sx + r * bw.w[k + 3];
        sy = sy + g * bw.w[k + 3];
        sz = sz + b * bw.w[k + 3];
    }
    dst[(size_t)i * 3] = sx / bw.sum;
    dst[(size_t)i * 3 + 1] = sy / bw.sum;
    dst[(size_t)i * 3 + 2] = sz / bw.sum;
}

// gaussian_weights(7, 5.0) (bounce_map.rs:140-151) in f32, exp rounded once from binary64.
BlurWeights blur_weights() {
    BlurWeights bw{};
    const float sigma2 = 5.0f * 5.0f;
    float sum = 0.0f;
    for (int i = -3; i <= 3; ++i) {
        float w = (1.0f / sqrtf(2.0f * kPiF * sigma2)) * (float)std::exp((double)(-(float)(i * i) / (2.0f * sigma2)));
        bw.w[i + 3] = w;
        sum += w;
    }
    for (int k = 0; k < 7; ++k) {
        bw.w[k] = bw.w[k] / sum;
        bw.sum += bw.w[k];
    }
    return bw;
}

}  // namespace
}  // namespace dl

extern "C" dl_status dl_filter_bounce_window_noalloc(const float *in_rgb, float *out_rgb, uint32_t width,
                                                     uint32_t height, uint32_t x0, uint32_t y0, uint32_t map_size,
                                                     void *stream) {
    using namespace dl;
    if (!in_rgb || !out_rgb) {
        g_error = "the input and output windows must be device buffers";
        return DL_INVALID_ARGUMENT;
    }
    uint64_t n = (uint64_t)width * height;
    if (width == 0 || height == 0 || n > kNoallocMaxTexels) {
        g_error = "window of " + std::to_string(width) + " x " + std::to_string(height) +
                  " texels: the non-allocating filter takes 1 to " + std::to_string(kNoallocMaxTexels) + " texels";
        return DL_INVALID_ARGUMENT;
    }
    {
        // the output is written while the input is still read: the two byte ranges must not meet
        const uintptr_t a = reinterpret_cast<uintptr_t>(in_rgb), b = reinterpret_cast<uintptr_t>(out_rgb);
        const uintptr_t bytes = (uintptr_t)(n * 3 * sizeof(float));
        if (a < b + bytes && b < a + bytes) {
            g_error = "the input and output windows overlap; they must be distinct device buffers";
            return DL_INVALID_ARGUMENT;
        }
    }
    if ((uint64_t)x0 + width > map_size || (uint64_t)y0 + height > map_size) {
        g_error = "the window does not lie inside the map";
        return DL_INVALID_ARGUMENT;
    }
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) {
        g_error = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
        return DL_CUDA_ERROR;
    }
    if (device < 0 || device >= kNoallocDevices) {
        g_error = "the non-allocating filter runs on devices 0 to " + std::to_string(kNoallocDevices - 1) +
                  ", the current device is " + std::to_string(device);
        return DL_UNSUPPORTED;
    }
    float *scratch = nullptr;
    {
        // set-up, once per device, with that device current: the scratch array's device address
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[device]) {
            e = cudaGetSymbolAddress((void **)&g_noalloc_ptr[device], g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_noalloc_ptr[device] = nullptr;
                g_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
                return DL_CUDA_ERROR;
            }
        }
        scratch = g_noalloc_ptr[device];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    BlurWeights bw = blur_weights();
    unsigned blocks = (unsigned)((n + 255) / 256);
    // dilate into the output, blur across into the scratch, blur down into the output; every
    // scratch texel is written before it is read, so nothing needs clearing between calls
    k_noalloc_dilate<<<blocks, 256, 0, st>>>(in_rgb, out_rgb, width, height);
    k_noalloc_blur<<<blocks, 256, 0, st>>>(out_rgb, scratch, width, height, x0, y0, map_size, 0, bw);
    k_noalloc_blur<<<blocks, 256, 0, st>>>(scratch, out_rgb, width, height, x0, y0, map_size, 1, bw);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        g_error = std::string("bounce filter launch: ") + cudaGetErrorString(e);
        return DL_CUDA_ERROR;
    }
    return DL_OK;
}

// ================================ cache read bandwidth =================================
// No counterpart in the reference. The roofline of the traversal kernels: their node and
// triangle reads come from the L1 and L2 caches (the scene's BVH fits in L2), so their bound is
// the read bandwidth of those caches, which this measures with a plain streaming read.

namespace dl {
namespace {

// Each thread reads four float4 per iteration (independent loads in flight). Level 2: the
// blocks stream the whole buffer with L1-bypassing loads (ld.global.cg), `passes` times, so
// every byte comes from L2 (for a buffer that fits in it). Level 1: each block re-reads its own `slice` float4s with cached
// loads (ld.global.nc), so after the first pass every byte comes from its SM's L1.
__global__ void __launch_bounds__(256) k_probe_read(const float4 *__restrict__ buf, uint64_t n4, uint32_t passes,
                                                    uint32_t level, uint64_t slice, float *sink) {
    float acc = 0.0f;
    const float4 *base = buf;
    uint64_t count = n4, first = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, stride =
        (uint64_t)gridDim.x * blockDim.x;
    if (level == 1) {
        base = buf + ((uint64_t)blockIdx.x * slice) % (n4 - slice + 1);
        count = slice;
        first = threadIdx.x;
        stride = blockDim.x;
    }
    for (uint32_t p = 0; p < passes; ++p) {
        uint64_t i = first;
        for (; i + 3 * stride < count; i += 4 * stride) {
            float4 a, b, c, d;
            if (level == 1) {
                a = __ldg(base + i);
                b = __ldg(base + i + stride);
                c = __ldg(base + i + 2 * stride);
                d = __ldg(base + i + 3 * stride);
            } else {
                a = __ldcg(base + i);
                b = __ldcg(base + i + stride);
                c = __ldcg(base + i + 2 * stride);
                d = __ldcg(base + i + 3 * stride);
            }
            acc += (a.x + b.y) + (c.z + d.w);
        }
        for (; i < count; i += stride) {
            float4 a = level == 1 ? __ldg(base + i) : __ldcg(base + i);
            acc += a.x;
        }
    }
    if (acc == -1.0f) sink[0] = acc;  // never true for the zero buffer; keeps the loads
}

}  // namespace
}  // namespace dl

extern "C" dl_status dl_probe_read_bandwidth(int device, uint32_t level, uint64_t bytes, uint32_t passes,
                                             double *gbs) {
    using namespace dl;
    if (!gbs || (level != 1 && level != 2) || passes == 0 || bytes < (1u << 20) || bytes > (1ull << 32)) {
        g_error = "dl_probe_read_bandwidth: level 1 or 2, 1 MiB to 4 GiB and at least one pass";
        return DL_INVALID_ARGUMENT;
    }
    *gbs = 0.0;
    int previous = 0;
    cudaError_t e = cudaGetDevice(&previous);
    if (e == cudaSuccess) e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        g_error = std::string("dl_probe_read_bandwidth: cudaSetDevice: ") + cudaGetErrorString(e);
        return DL_CUDA_ERROR;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float4 *buf = nullptr;
    float *sink = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    dl_status st = DL_OK;
    const uint64_t n4 = bytes / sizeof(float4);
    const uint64_t slice = 32 * 1024 / sizeof(float4);  // level 1: 32 KiB per block, 4 blocks per SM
    const unsigned blocks = (unsigned)std::max(1, sms) * 4;
    double best = 0.0;
    e = cudaMalloc(&buf, n4 * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(buf, 0, n4 * sizeof(float4));
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    for (int rep = 0; e == cudaSuccess && rep < 6; ++rep) {
        // the first run is a warm-up: it brings the buffer into L2 (and the slices into L1)
        cudaEventRecord(t0, 0);
        k_probe_read<<<blocks, 256>>>(buf, n4, passes, level, slice, sink);
        cudaEventRecord(t1, 0);
        e = cudaEventSynchronize(t1);
        if (e != cudaSuccess) break;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, t0, t1);
        const double read = level == 1 ? (double)blocks * slice * sizeof(float4) * passes
                                       : (double)n4 * sizeof(float4) * passes;
        if (rep > 0 && ms > 0.0f) best = std::max(best, read / (ms * 1e-3) / 1e9);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        g_error = std::string("dl_probe_read_bandwidth: ") + cudaGetErrorString(e);
        st = e == cudaErrorMemoryAllocation ? DL_OUT_OF_MEMORY : DL_CUDA_ERROR;
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (buf) cudaFree(buf);
    if (sink) cudaFree(sink);
    cudaSetDevice(previous);
    *gbs = best;
    return st;
}
