// Device side of the bake: the resident scene, the ray queries and per-texel visibility.
//
// Ray queries restate the reference's Occluders (src/bake/occluder.rs:171-251): two-sided
// Möller–Trumbore with hits for 0 <= t <= max, any-hit for shadow rays, closest-hit with ties
// going to the lowest occluder index, optional alpha test. The BVH only prunes: node boxes are
// padded and the slab test keeps a relative slack, so no triangle the exact test would report is
// ever culled and results equal a scan over every occluder.
#pragma once

#include <cuda_runtime.h>

#include "dl_host.hpp"
#include "dl_math.cuh"

namespace dl {

// Everything the kernels read, as device pointers (one struct passed by value).
struct DevScene {
    // BVH and triangles in leaf order
    const float4 *nodes;  // 4 float4 per node
    // triangles as 3 float4 each, one 48-byte record per triangle (a leaf's triangles are
    // contiguous): v0 (w: occluder index bits), e1 = v1 - v0, e2 = v2 - v0
    const float4 *tris;
    uint32_t occluders;
    // occluder index -> mesh, triangle in mesh, position in leaf order
    const uint32_t *occ_mesh, *occ_tri, *occ_leaf;
    // meshes (sorted order)
    uint32_t mesh_count;
    const uint32_t *mesh_vertex_base, *mesh_index_base, *mesh_tri_base, *mesh_res;
    const uint32_t *mesh_flags;  // kMesh* bits
    const uint64_t *mesh_id;
    const float *mesh_albedo;     // 3 per mesh
    const uint32_t *mesh_alpha;   // 4 per mesh: byte offset, width, height, cutoff bits
    const uint8_t *alpha_pool;
    // vertex data (global vertex index = base + local)
    const float *positions, *normals, *uv1, *uv0;  // 3, 3, 2, 2 per vertex
    const uint32_t *indices;                       // local vertex indices
    // triangles
    uint32_t triangles;
    const uint32_t *tri_mesh;
    // lights in slot order
    uint32_t light_count, local_lights;
    const DevLight *lights;
    // options
    uint64_t seed;
    uint32_t area_samples, area_min_samples, sky_samples;
    uint32_t colored_bounce;
    // refined form: the epsilon of the binary64 re-test and its square
    float refine_eps, refine_eps2;
    // coherent sample orders (sky_sample_order) for n = 16, 32, ..., kMaxOrdered back to back
    // (the table of n starts at n - 16); sky_order is the sky's, or null
    const uint16_t *orders;
    const uint16_t *sky_order;
    // sample_cells (dl_host.hpp) for the same n, laid out like `orders`
    const uint16_t *order_cells, *cell_samples;
};
constexpr uint32_t kMaxOrdered = 4096;
// The shift of a net of n samples (n a power of two from 16 to kMaxOrdered) by `off` in whole
// cells, packed as x | y << 8 | xbits << 16 | ybits << 24.
__device__ __forceinline__ uint32_t net_shift(uint32_t n, f2 off) {
    uint32_t m = 31 - __clz(n), xb = (m + 1) / 2, yb = m / 2;
    uint32_t sx = min((1u << xb) - 1, (uint32_t)(off.x * (float)(1u << xb)));
    uint32_t sy = min((1u << yb) - 1, (uint32_t)(off.y * (float)(1u << yb)));
    return sx | sy << 8 | xb << 16 | yb << 24;
}
// Sample of rank k of a net of n samples shifted by `shift` (net_shift): the point of the cell of
// rank k moved back by the shift, so that texels with different shifts send their rank-k rays in
// about the same direction. A permutation of 0 .. n-1 over k.
__device__ __forceinline__ uint32_t shifted_sample(const DevScene &sc, uint32_t n, uint32_t shift, uint32_t k) {
    const uint32_t c = sc.order_cells[n - 16 + k];
    const uint32_t xb = (shift >> 16) & 0xFFu, yb = shift >> 24;
    const uint32_t cx = ((c & 0xFFu) - (shift & 0xFFu)) & ((1u << xb) - 1u);
    const uint32_t cy = ((c >> 8) - ((shift >> 8) & 0xFFu)) & ((1u << yb) - 1u);
    return sc.cell_samples[n - 16 + (cy << xb | cx)];
}
enum : uint32_t { kMeshNormals = 1, kMeshOccludes = 2, kMeshAlpha = 4 };

__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }

// AlphaTexture::is_opaque (src/bake/input.rs:79-97) at the hit's interpolated UV0.
__device__ __forceinline__ uint32_t wrap_texel(float coordinate, uint32_t size) {
    float r = fmodf(coordinate, 1.0f);
    if (r < 0.0f) r = r + 1.0f;
    float t = floorf(r * (float)size);
    if (isfinite(t)) {
        uint32_t u = f2u(t);
        return u < size - 1 ? u : size - 1;
    }
    return 0;
}
__device__ __noinline__ bool alpha_blocks(const DevScene &sc, uint32_t occ, float u, float v) {
    uint32_t m = sc.occ_mesh[occ];
    if (!(sc.mesh_flags[m] & kMeshAlpha)) return true;
    const uint32_t *tex = sc.mesh_alpha + m * 4;
    uint32_t width = tex[1], height = tex[2];
    if (width == 0 || height == 0) return true;
    const uint32_t *c = sc.indices + sc.mesh_index_base[m] + (size_t)sc.occ_tri[occ] * 3;
    uint32_t vb = sc.mesh_vertex_base[m];
    float wx = 1.0f - u - v;
    const float *a = sc.uv0 + (size_t)(vb + c[0]) * 2, *b = sc.uv0 + (size_t)(vb + c[1]) * 2,
                *d = sc.uv0 + (size_t)(vb + c[2]) * 2;
    float uvx = a[0] * wx + b[0] * u + d[0] * v;
    float uvy = a[1] * wx + b[1] * u + d[1] * v;
    uint32_t x = wrap_texel(uvx, width), y = wrap_texel(uvy, height);
    uint8_t alpha = sc.alpha_pool[tex[0] + (size_t)y * width + x];
    return (float)alpha / 255.0f >= __uint_as_float(tex[3]);
}

// intersect (occluder.rs:225-251) on a triangle stored as v0, e1 = v1 - v0, e2 = v2 - v0.
__device__ __forceinline__ bool tri_test(float4 v0, float4 e1v, float4 e2v, f3 o, f3 d, float max, float &t,
                                         float &u, float &v) {
    f3 e1{e1v.x, e1v.y, e1v.z}, e2{e2v.x, e2v.y, e2v.z};
    f3 p = cross(d, e2);
    float det = dot(e1, p);
    if (det == 0.0f || !isfinite(det)) return false;
    float inv = 1.0f / det;
    f3 s{o.x - v0.x, o.y - v0.y, o.z - v0.z};
    u = dot(s, p) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    f3 q = cross(s, e1);
    v = dot(d, q) * inv;
    if (v < 0.0f || u + v > 1.0f) return false;
    t = dot(e2, q) * inv;
    return t >= 0.0f && t <= max;
}

struct Hit {
    float t, u, v;
    uint32_t occluder;
};

// Node visits and triangle tests of traversals, counted only in the instrumented kernel variant
// the benchmark uses for its roofline bytes; `retests` counts the refined form's binary64
// re-tests.
struct Visits {
    unsigned long long nodes, tris, retests;
};

// The ray/triangle test of occluder `occ` in binary64 on its original vertices (the stored
// e1/e2 are rounded binary32 differences). The operation order is intersect's; u, v and t are
// rounded to binary32 once at the end.
__device__ __noinline__ bool tri_test_fp64(const DevScene &sc, uint32_t occ, f3 o, f3 d, float max, float &t,
                                           float &u, float &v) {
    uint32_t m = sc.occ_mesh[occ];
    const uint32_t *c = sc.indices + sc.mesh_index_base[m] + (size_t)sc.occ_tri[occ] * 3;
    uint32_t vb = sc.mesh_vertex_base[m];
    const float *pa = sc.positions + (size_t)(vb + c[0]) * 3, *pb = sc.positions + (size_t)(vb + c[1]) * 3,
                *pc = sc.positions + (size_t)(vb + c[2]) * 3;
    d3 a{pa[0], pa[1], pa[2]};
    d3 e1 = sub(d3{pb[0], pb[1], pb[2]}, a), e2 = sub(d3{pc[0], pc[1], pc[2]}, a);
    d3 dd = widen(d);
    d3 p = cross(dd, e2);
    double det = dot(e1, p);
    if (det == 0.0 || !isfinite(det)) return false;
    double inv = 1.0 / det;
    d3 s = sub(widen(o), a);
    double ud = dot(s, p) * inv;
    if (!(ud >= 0.0 && ud <= 1.0)) return false;
    d3 q = cross(s, e1);
    double vd = dot(dd, q) * inv;
    if (vd < 0.0 || ud + vd > 1.0) return false;
    double td = dot(e2, q) * inv;
    if (!(td >= 0.0 && td <= (double)max)) return false;
    t = (float)td;
    u = (float)ud;
    v = (float)vd;
    return true;
}

// The refined form's test: the binary32 test decides unless the ray is nearly parallel to the
// plane (|det| <= eps |e1| |d x e2|) or u, v, u + v or t lie within eps of their bounds (t's
// margin is eps * max(1, max) for a finite max, eps otherwise); those rays are re-tested in
// binary64. Outside the margins the binary32 verdict and hit equal tri_test's.
__device__ __forceinline__ bool tri_test_refined(const DevScene &sc, float4 v0, float4 e1v, float4 e2v, f3 o, f3 d,
                                                 float max, float &t, float &u, float &v, Visits *vis) {
    const float eps = sc.refine_eps;
    f3 e1{e1v.x, e1v.y, e1v.z}, e2{e2v.x, e2v.y, e2v.z};
    f3 p = cross(d, e2);
    float det = dot(e1, p);
    if (det * det > sc.refine_eps2 * (dot(e1, e1) * dot(p, p))) {
        float inv = 1.0f / det;
        f3 s{o.x - v0.x, o.y - v0.y, o.z - v0.z};
        u = dot(s, p) * inv;
        if (!(u >= -eps && u <= 1.0f + eps)) return false;
        f3 q = cross(s, e1);
        v = dot(d, q) * inv;
        if (!(v >= -eps) || u + v > 1.0f + eps) return false;
        t = dot(e2, q) * inv;
        float margin = eps * (isfinite(max) ? fmaxf(max, 1.0f) : 1.0f);
        if (!(t >= -margin && t <= max + margin)) return false;
        bool near = u < eps || u > 1.0f - eps || v < eps || u + v > 1.0f - eps || t < margin || t > max - margin;
        if (!near) return true;
    }
    ++vis->retests;
    return tri_test_fp64(sc, __float_as_uint(v0.w), o, d, max, t, u, v);
}

constexpr int kStack = 64;  // >= BVH depth; the host refuses deeper trees

// Slab test of both children of a node against the ray [0, tmax]. Boxes are padded on the host
// and the exit distance gets a relative slack, so the test only ever errs towards visiting.
__device__ __forceinline__ void box2(const float4 &a, const float4 &b, const float4 &c, f3 inv, f3 oinv, float tmax,
                                     bool &h0, bool &h1, float &n0, float &n1) {
    float lx0 = __fmaf_rn(a.x, inv.x, -oinv.x), hx0 = __fmaf_rn(a.y, inv.x, -oinv.x);
    float ly0 = __fmaf_rn(a.z, inv.y, -oinv.y), hy0 = __fmaf_rn(a.w, inv.y, -oinv.y);
    float lz0 = __fmaf_rn(c.x, inv.z, -oinv.z), hz0 = __fmaf_rn(c.y, inv.z, -oinv.z);
    float lx1 = __fmaf_rn(b.x, inv.x, -oinv.x), hx1 = __fmaf_rn(b.y, inv.x, -oinv.x);
    float ly1 = __fmaf_rn(b.z, inv.y, -oinv.y), hy1 = __fmaf_rn(b.w, inv.y, -oinv.y);
    float lz1 = __fmaf_rn(c.z, inv.z, -oinv.z), hz1 = __fmaf_rn(c.w, inv.z, -oinv.z);
    float en0 = fmaxf(fmaxf(fminf(lx0, hx0), fminf(ly0, hy0)), fmaxf(fminf(lz0, hz0), 0.0f));
    float ex0 = fminf(fminf(fmaxf(lx0, hx0), fmaxf(ly0, hy0)), fminf(fmaxf(lz0, hz0), tmax));
    float en1 = fmaxf(fmaxf(fminf(lx1, hx1), fminf(ly1, hy1)), fmaxf(fminf(lz1, hz1), 0.0f));
    float ex1 = fminf(fminf(fmaxf(lx1, hx1), fmaxf(ly1, hy1)), fminf(fmaxf(lz1, hz1), tmax));
    const float slack = 1.0f + 2.0e-6f;
    h0 = en0 <= ex0 * slack;
    h1 = en1 <= ex1 * slack;
    n0 = en0;
    n1 = en1;
}

// The reciprocal direction for the slab tests. It only prunes, so the fast reciprocal (within
// 2 ulp) serves: each axis' slab distances all scale by one factor within 2^-22 of 1, so entry
// and exit move by under 5e-7 of their value, inside box2's relative exit slack (2e-6).
__device__ __forceinline__ f3 safe_inv(f3 d) {
    return f3{__fdividef(1.0f, d.x == 0.0f ? copysignf(1e-30f, d.x) : d.x),
              __fdividef(1.0f, d.y == 0.0f ? copysignf(1e-30f, d.y) : d.y),
              __fdividef(1.0f, d.z == 0.0f ? copysignf(1e-30f, d.z) : d.z)};
}

// Any-hit (ANY) or closest-hit traversal of the BVH2. Child references: >= 0 an inner node,
// < 0 a leaf ~(first << 3 | count). `stack` points at this thread's first stack slot in shared
// memory, slots `stride` apart. For closest-hit, `hit` gets the nearest t (ties to the lowest
// occluder index, as occluder.rs:205-210) and that test's barycentrics, which equal the ones
// the reference recomputes with max = infinity.
template <bool ANY, bool COUNT = false, bool REFINE = false>
__device__ bool traverse(const DevScene &sc, f3 o, f3 dir, float max, bool alpha, int *stack, int stride, Hit &hit,
                         Visits *vis = nullptr) {
    hit.t = INFINITY;
    hit.u = hit.v = 0.0f;
    hit.occluder = 0xFFFFFFFFu;
    if (sc.occluders == 0) return false;
    f3 d{dir.x + 0.0f, dir.y + 0.0f, dir.z + 0.0f};  // -0 -> +0 (occluder.rs:171-178)
    f3 inv = safe_inv(d);
    f3 oinv{o.x * inv.x, o.y * inv.y, o.z * inv.z};
    float tmax = fmaxf(max, 0.0f);
    bool found = false;
    int sp = 0;
    int ref = 0;
    // while-while traversal (Aila & Laine 2009): descend inner nodes until a leaf is reached,
    // then test leaves until an inner node comes off the stack, so a warp's lanes run the same
    // loop body together instead of alternating node and leaf work per lane.
    for (;;) {
        while (ref >= 0) {
            const float4 *nd = sc.nodes + (size_t)ref * 4;
            float4 a = ldg4(nd), b = ldg4(nd + 1), c = ldg4(nd + 2), r = ldg4(nd + 3);
            if (COUNT) ++vis->nodes;
            bool h0, h1;
            float n0, n1;
            box2(a, b, c, inv, oinv, ANY ? tmax : fminf(tmax, hit.t), h0, h1, n0, n1);
            // an empty child (~0, only beside a root leaf) reads as a leaf of no triangles
            int r0 = __float_as_int(r.x), r1 = __float_as_int(r.y);
            if (h0 && h1) {
                bool swap = n1 < n0;
                stack[sp * stride] = swap ? r0 : r1;
                ++sp;
                ref = swap ? r1 : r0;
            } else if (h0 || h1) {
                ref = h0 ? r0 : r1;
            } else {
                if (sp == 0) return found;
                ref = stack[--sp * stride];
            }
        }
        while (ref < 0) {
            uint32_t packed = (uint32_t)(~ref);
            uint32_t first = packed >> 3, count = packed & 7u;
            for (uint32_t k = 0; k < count; ++k) {
                uint32_t i = first + k;
                const float4 *tp = sc.tris + (size_t)i * 3;
                float4 v0 = ldg4(tp);
                if (COUNT) ++vis->tris;
                float t, u, v;
                bool ok = REFINE ? tri_test_refined(sc, v0, ldg4(tp + 1), ldg4(tp + 2), o, d, max, t, u, v, vis)
                                 : tri_test(v0, ldg4(tp + 1), ldg4(tp + 2), o, d, max, t, u, v);
                if (!ok) continue;
                uint32_t occ = __float_as_uint(v0.w);
                // the refined form orders closest-hit candidates by their binary64 distance (and
                // takes their barycentrics from it), so the winner is the binary64 intersection's
                if (!ANY && REFINE) {
                    ++vis->retests;
                    if (!tri_test_fp64(sc, occ, o, d, max, t, u, v)) continue;
                }
                if (alpha && !alpha_blocks(sc, occ, u, v)) continue;
                if (ANY) return true;
                if (isfinite(t) && (t < hit.t || (t == hit.t && occ < hit.occluder))) {
                    found = true;
                    hit.t = t;
                    hit.u = u;
                    hit.v = v;
                    hit.occluder = occ;
                }
            }
            if (sp == 0) return found;
            ref = stack[--sp * stride];
        }
    }
}

template <bool COUNT = false, bool REFINE = false>
__device__ __forceinline__ bool occluded(const DevScene &sc, f3 o, f3 d, float max, bool alpha, int *stack,
                                         int stride, Visits *vis = nullptr) {
    Hit h;
    return traverse<true, COUNT, REFINE>(sc, o, d, max, alpha, stack, stride, h, vis);
}

}  // namespace dl
