// TEST INFRASTRUCTURE — the parity oracle, not the product.
//
// Geometry, texel generation, the light BVH and the occluder ray queries of the reference
// baker, restated operation for operation in f32 (see oracle_math.hpp for the arithmetic
// conventions). Each function cites the reference function it follows.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "../include/dynlight.h"
#include "oracle_math.hpp"

namespace oracle {

// ---- small parallel-for (rayon's role; every reduction used with it is commutative) -----------
inline unsigned &thread_count() {
    static unsigned n = 0;
    return n;
}
inline void parallel_for(size_t n, const std::function<void(size_t)> &f) {
    unsigned threads = thread_count();
    if (threads <= 1 || n < 2) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (;;) {
            size_t i = next.fetch_add(1);
            if (i >= n) break;
            f(i);
        }
    };
    std::vector<std::thread> pool;
    unsigned t = (unsigned)std::min<size_t>(threads, n);
    for (unsigned k = 1; k < t; ++k) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
}

// ---- TexelRect (src/bake/bits.rs:7-38) ----------------------------------------------------------
struct Rect {
    uint32_t min_x, min_y, max_x, max_y;
    uint32_t width() const { return max_x - min_x + 1; }
    uint32_t height() const { return max_y - min_y + 1; }
    Rect unite(Rect o) const {
        return Rect{std::min(min_x, o.min_x), std::min(min_y, o.min_y), std::max(max_x, o.max_x),
                    std::max(max_y, o.max_y)};
    }
    bool contains(int64_t x, int64_t y) const {
        return x >= (int64_t)min_x && y >= (int64_t)min_y && x <= (int64_t)max_x &&
               y <= (int64_t)max_y;
    }
};

// ---- BitGrid (src/bake/bits.rs:40-101), LSB-first row-major -------------------------------------
struct BitGrid {
    uint32_t width = 0, height = 0;
    std::vector<uint32_t> words;
    BitGrid() = default;
    BitGrid(uint32_t w, uint32_t h) : width(w), height(h), words(((size_t)w * h + 31) / 32, 0) {}
    bool get(uint32_t x, uint32_t y) const {
        size_t i = (size_t)x + (size_t)y * width;
        return (words[i / 32] >> (i % 32)) & 1u;
    }
    bool get_or_false(int64_t x, int64_t y) const {
        return x >= 0 && y >= 0 && x < (int64_t)width && y < (int64_t)height &&
               get((uint32_t)x, (uint32_t)y);
    }
    void set(uint32_t x, uint32_t y, bool v) {
        size_t i = (size_t)x + (size_t)y * width;
        if (v)
            words[i / 32] |= 1u << (i % 32);
        else
            words[i / 32] &= ~(1u << (i % 32));
    }
    // AtomicBitGrid::set (bits.rs:121-125)
    void set_atomic(uint32_t x, uint32_t y) {
        size_t i = (size_t)x + (size_t)y * width;
        __atomic_fetch_or(&words[i / 32], 1u << (i % 32), __ATOMIC_RELAXED);
    }
};

// ---- ShadowGrid (src/bake/shadow_grid.rs:20-107) + AtomicShadowGrid::raise (:136-143) ----------
inline uint8_t level(float fraction, uint32_t bits) {
    float max = (float)((1u << bits) - 1);
    return f2u8_sat(std::round(clampf(fraction, 0.0f, 1.0f) * max));
}
// level() of a fraction held in binary64: rounded in binary64 in the F64 mode, else level() of
// the binary32 fraction
inline uint8_t level_of(double fraction, uint32_t bits) {
    if (active_mode() != PREC_F64) return level((float)fraction, bits);
    double max = (double)((1u << bits) - 1);
    double v = std::round(std::min(std::max(fraction, 0.0), 1.0) * max);
    return (uint8_t)v;
}
struct ShadowGrid {
    uint32_t width = 0, height = 0, bits = 1;
    std::vector<uint8_t> levels;  // one per texel; packed on output
    ShadowGrid() = default;
    ShadowGrid(uint32_t w, uint32_t h, uint32_t b)
        : width(w), height(h), bits(b <= 1 ? 1 : std::min(b, 8u)), levels((size_t)w * h, 0) {}
    uint8_t get(uint32_t x, uint32_t y) const { return levels[(size_t)x + (size_t)y * width]; }
    uint8_t get_or_zero(int64_t x, int64_t y) const {
        bool inside = x >= 0 && y >= 0 && x < (int64_t)width && y < (int64_t)height;
        return inside ? get((uint32_t)x, (uint32_t)y) : 0;
    }
    void set(uint32_t x, uint32_t y, uint8_t level) {
        levels[(size_t)x + (size_t)y * width] = bits == 1 ? (level != 0) : level;
    }
    void raise_atomic(uint32_t x, uint32_t y, uint8_t level) {
        if (bits == 1 && level == 0) return;
        uint8_t *p = &levels[(size_t)x + (size_t)y * width];
        uint8_t v = bits == 1 ? 1 : level;
        uint8_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
        while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, true, __ATOMIC_RELAXED,
                                                       __ATOMIC_RELAXED)) {
        }
    }
    // into_words (shadow_grid.rs:91-106): 1 bit = BitGrid layout, else floor(32/bits) per word.
    std::vector<uint32_t> into_words() const {
        std::vector<uint32_t> out;
        size_t n = levels.size();
        if (bits == 1) {
            out.assign((n + 31) / 32, 0);
            for (size_t i = 0; i < n; ++i)
                if (levels[i]) out[i / 32] |= 1u << (i % 32);
            return out;
        }
        size_t per = 32 / bits;
        out.assign((n + per - 1) / per, 0);
        for (size_t i = 0; i < n; ++i) out[i / per] |= (uint32_t)levels[i] << ((i % per) * bits);
        return out;
    }
};
struct ShadowRegion {
    Rect rect;
    ShadowGrid grid;
    // ShadowRegion::get (shadow_grid.rs:165-178)
    uint8_t get(int64_t x, int64_t y) const {
        return grid.get_or_zero(x - (int64_t)rect.min_x, y - (int64_t)rect.min_y);
    }
};

// ---- geometry (src/bake/geometry.rs) -------------------------------------------------------------
struct Aabb {
    V3 min, max;
    static Aabb empty() { return Aabb{V3{INFINITY, INFINITY, INFINITY}, V3{-INFINITY, -INFINITY, -INFINITY}}; }
    static Aabb from_sphere(V3 c, float r) { return Aabb{c - V3{r, r, r}, c + V3{r, r, r}}; }
    Aabb grow(V3 p) const { return Aabb{vmin(min, p), vmax(max, p)}; }
    Aabb unite(Aabb o) const { return Aabb{vmin(min, o.min), vmax(max, o.max)}; }
    bool intersects(const Aabb &o) const {
        return min.x <= o.max.x && min.y <= o.max.y && min.z <= o.max.z && o.min.x <= max.x &&
               o.min.y <= max.y && o.min.z <= max.z;
    }
    // half_area_x2 (geometry.rs:49-55)
    float half_area_x2() const {
        V3 e = max - min;
        if (fmin_r(fmin_r(e.x, e.y), e.z) < 0.0f) return 0.0f;
        return 2.0f * (e.x * e.y + e.y * e.z + e.z * e.x);
    }
};
// geometry.rs:59-61
inline float triangle_area(V3 a, V3 b, V3 c) { return length(cross(b - a, c - a)) * 0.5f; }
// geometry.rs:66-70
inline uint32_t lightmap_size(float area, float density, uint32_t max_size) {
    float size = std::ceil(std::sqrt(density * density * area));
    if (std::isnan(size)) size = 0.0f;
    uint32_t s = f2u_sat(fmin_r(size, (float)max_size));
    uint32_t hi = std::max(max_size, 2u);
    return std::min(std::max(s, 2u), hi);
}
// geometry.rs:73-108 (Ericson)
inline V3 closest_point_on_triangle(V3 p, V3 a, V3 b, V3 c) {
    V3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    V3 bp = p - b;
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return a + ab * (d1 / (d1 - d3));
    V3 cp = p - c;
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return a + ac * (d2 / (d2 - d6));
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
        return b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)));
    float denom = 1.0f / (va + vb + vc);
    return a + ab * (vb * denom) + ac * (vc * denom);
}
// geometry.rs:111-114
inline bool sphere_intersects_triangle(V3 center, float r, V3 a, V3 b, V3 c) {
    V3 closest = closest_point_on_triangle(center, a, b, c);
    return distance_squared(closest, center) <= r * r;
}
// geometry.rs:117-121
inline float signed_area(V2 a, V2 b, V2 c) {
    V2 aa = a - c, bb = b - c;
    return (aa.x * bb.y - aa.y * bb.x) * 0.5f;
}
// geometry.rs:125-134
inline bool uv_barycentrics(const V2 t[3], V2 p, V3 &w) {
    float area = signed_area(t[0], t[1], t[2]);
    if (area == 0.0f) return false;
    float a1 = signed_area(t[1], t[2], p) / area;
    float a2 = signed_area(t[2], t[0], p) / area;
    float a3 = signed_area(t[0], t[1], p) / area;
    if (a1 >= 0.0f && a2 >= 0.0f && a3 >= 0.0f) {
        w = V3{a1, a2, a3};
        return true;
    }
    return false;
}

// ---- rects (src/bake/mesh_builder.rs:103-135) ---------------------------------------------------
inline uint32_t clamp_texel(float v, uint32_t size) { return f2u_sat(clampf(v, 0.0f, (float)(size - 1))); }
inline void uv_bounds(const V2 uv[3], V2 &mn, V2 &mx) {
    mn = vmin2(vmin2(uv[0], uv[1]), uv[2]);
    mx = vmax2(vmax2(uv[0], uv[1]), uv[2]);
}
inline Rect crop_rect(const V2 uv[3], uint32_t size) {
    V2 mn, mx;
    uv_bounds(uv, mn, mx);
    float s = (float)size;
    return Rect{clamp_texel(std::floor(mn.x * s) - 2.0f, size), clamp_texel(std::floor(mn.y * s) - 2.0f, size),
                clamp_texel(std::ceil(mx.x * s) + 2.0f, size), clamp_texel(std::ceil(mx.y * s) + 2.0f, size)};
}
inline Rect grown_center_rect(const V2 uv[3], uint32_t size, float grow) {
    V2 mn, mx;
    uv_bounds(uv, mn, mx);
    float s = (float)size;
    return Rect{clamp_texel(std::floor(mn.x * s - 0.5f) - grow, size),
                clamp_texel(std::floor(mn.y * s - 0.5f) - grow, size),
                clamp_texel(std::ceil(mx.x * s - 0.5f) + grow, size),
                clamp_texel(std::ceil(mx.y * s - 0.5f) + grow, size)};
}
inline Rect trace_rect(const V2 uv[3], uint32_t size) { return grown_center_rect(uv, size, 0.0f); }
inline Rect optimize_rect(const V2 uv[3], uint32_t size) { return grown_center_rect(uv, size, 1.0f); }

// ---- texels (src/bake/texels.rs) ------------------------------------------------------------------
struct SurfaceTexel {
    uint32_t x, y;
    V3 position, normal;
};
// texels.rs:24-37
inline bool uv_to_surface(const V3 v[3], const V3 n[3], const V2 uv[3], V3 face, V2 p, V3 &pos, V3 &nrm) {
    V3 w;
    if (!uv_barycentrics(uv, p, w)) return false;
    pos = v[0] * w.x + v[1] * w.y + v[2] * w.z;
    bool ok;
    V3 t = try_normalize(n[0] * w.x + n[1] * w.y + n[2] * w.z, ok);
    nrm = ok ? t : face;
    return true;
}
// texels.rs:40-45
inline V2 texel_center(uint32_t x, uint32_t y, uint32_t size) {
    return V2{((float)x + 0.5f) / (float)size, ((float)y + 0.5f) / (float)size};
}
// texels.rs:48-72
inline void triangle_texels(const V3 v[3], const V3 n[3], const V2 uv[3], V3 face, uint32_t size,
                            std::vector<SurfaceTexel> &out) {
    Rect r = trace_rect(uv, size);
    for (uint32_t y = r.min_y; y <= r.max_y; ++y)
        for (uint32_t x = r.min_x; x <= r.max_x; ++x) {
            V3 pos, nrm;
            if (uv_to_surface(v, n, uv, face, texel_center(x, y, size), pos, nrm))
                out.push_back(SurfaceTexel{x, y, pos, nrm});
        }
}
// texels.rs:125-141
inline bool nearest_weights(const V2 uv[3], V2 point, V3 &w_out) {
    V3 a{uv[0].x, uv[0].y, 0.0f}, b{uv[1].x, uv[1].y, 0.0f}, c{uv[2].x, uv[2].y, 0.0f};
    V3 nearest3 = closest_point_on_triangle(V3{point.x, point.y, 0.0f}, a, b, c);
    V3 nearest{nearest3.x, nearest3.y, 0.0f};
    float area = cross(b - a, c - a).z;
    if (area == 0.0f || !std::isfinite(area)) return false;
    auto weight = [&](V2 p, V2 q) {
        return cross(V3{p.x, p.y, 0.0f} - nearest, V3{q.x, q.y, 0.0f} - nearest).z;
    };
    V3 w = V3{weight(uv[1], uv[2]), weight(uv[2], uv[0]), weight(uv[0], uv[1])} / area;
    w = vmax(w, V3{0, 0, 0});
    float sum = (w.x + w.y) + w.z;
    w_out = w / fmax_r(sum, 1.17549435e-38f);
    return true;
}
// texels.rs:78-121
template <class Owned>
inline void touched_texels(const V3 v[3], const V3 n[3], const V2 uv[3], V3 face, uint32_t size,
                           Owned owned, std::vector<SurfaceTexel> &out) {
    float s = (float)size;
    V2 mn, mx;
    uv_bounds(uv, mn, mx);
    V2 first{fmax_r(std::floor(mn.x * s), 0.0f), fmax_r(std::floor(mn.y * s), 0.0f)};
    V2 last{fmin_r(std::floor(mx.x * s), s - 1.0f), fmin_r(std::floor(mx.y * s), s - 1.0f)};
    float half = 0.5f / s;
    uint32_t y0 = f2u_sat(first.y), y1 = f2u_sat(last.y), x0 = f2u_sat(first.x), x1 = f2u_sat(last.x);
    for (uint64_t y = y0; y <= y1; ++y)
        for (uint64_t x = x0; x <= x1; ++x) {
            if (owned((uint32_t)x, (uint32_t)y)) continue;
            V2 center = texel_center((uint32_t)x, (uint32_t)y, size);
            V3 w;
            if (!nearest_weights(uv, center, w)) continue;
            V2 nearest = uv[0] * w.x + uv[1] * w.y + uv[2] * w.z;
            V2 d = nearest - center;
            if (fmax_r(std::fabs(d.x), std::fabs(d.y)) > half) continue;
            V3 pos = v[0] * w.x + v[1] * w.y + v[2] * w.z;
            bool ok;
            V3 t = try_normalize(n[0] * w.x + n[1] * w.y + n[2] * w.z, ok);
            out.push_back(SurfaceTexel{(uint32_t)x, (uint32_t)y, pos, ok ? t : face});
        }
}

// ---- light BVH (src/bake/light_bvh.rs:59-219) ---------------------------------------------------
struct LightBvh {
    std::vector<dl_light_bvh_node> nodes;
    std::vector<size_t> order;
    std::vector<Aabb> light_bounds;
    // query (light_bvh.rs:196-219): equals the brute-force scan of light_bounds.
    void query(const Aabb &box, std::vector<uint32_t> &out) const {
        if (nodes.empty()) return;
        for (uint32_t s = 0; s < light_bounds.size(); ++s)
            if (light_bounds[s].intersects(box)) out.push_back(s);
    }
};
struct LightBvhBuilder {
    const std::vector<V3> &pos;
    const std::vector<float> &rad;
    std::vector<size_t> idx;
    std::vector<dl_light_bvh_node> nodes;
    Aabb bounds_of(size_t l) const { return Aabb::from_sphere(pos[l], rad[l]); }
    void update_bounds(size_t node) {
        auto &n = nodes[node];
        Aabb a = Aabb::empty();
        for (size_t k = n.left_first; k < (size_t)n.left_first + n.count; ++k) a = a.unite(bounds_of(idx[k]));
        n.aabb_min[0] = a.min.x; n.aabb_min[1] = a.min.y; n.aabb_min[2] = a.min.z;
        n.aabb_max[0] = a.max.x; n.aabb_max[1] = a.max.y; n.aabb_max[2] = a.max.z;
    }
    static float axis(V3 v, int a) { return a == 0 ? v.x : a == 1 ? v.y : v.z; }
    float split_cost(size_t first, size_t count, int ax, float split) const {
        Aabb l = Aabb::empty(), r = Aabb::empty();
        uint32_t lc = 0, rc = 0;
        for (size_t k = first; k < first + count; ++k) {
            size_t light = idx[k];
            if (axis(pos[light], ax) < split) { ++lc; l = l.unite(bounds_of(light)); }
            else { ++rc; r = r.unite(bounds_of(light)); }
        }
        if (lc == 0 || rc == 0) return 3.40282347e+38f;
        return (float)lc * l.half_area_x2() + (float)rc * r.half_area_x2();
    }
    void subdivide(size_t node) {
        uint32_t lf = nodes[node].left_first, count = nodes[node].count;
        if (count <= 2) return;
        size_t first = lf;
        Aabb box{V3{nodes[node].aabb_min[0], nodes[node].aabb_min[1], nodes[node].aabb_min[2]},
                 V3{nodes[node].aabb_max[0], nodes[node].aabb_max[1], nodes[node].aabb_max[2]}};
        float parent_cost = (float)count * box.half_area_x2();
        bool found = false;
        int best_axis = 0;
        float best_split = 0, best_cost = 3.40282347e+38f;
        for (int ax = 0; ax < 3; ++ax)
            for (size_t k = 0; k < count; ++k) {
                float cand = axis(pos[idx[first + k]], ax);
                float cost = split_cost(first, count, ax, cand);
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_split = cand; found = true; }
            }
        if (!found || best_cost >= parent_cost) return;
        int64_t i = (int64_t)first, j = (int64_t)(first + count) - 1;
        while (i <= j) {
            if (axis(pos[idx[(size_t)i]], best_axis) < best_split) ++i;
            else { std::swap(idx[(size_t)i], idx[(size_t)j]); --j; }
        }
        size_t left_count = (size_t)i - first;
        if (left_count == 0 || left_count == count) return;
        size_t left = nodes.size();
        dl_light_bvh_node a{}, b{};
        a.left_first = (uint32_t)first; a.count = (uint32_t)left_count;
        b.left_first = (uint32_t)i; b.count = (uint32_t)(count - left_count);
        nodes.push_back(a);
        nodes.push_back(b);
        nodes[node].left_first = (uint32_t)left;
        nodes[node].count = 0;
        update_bounds(left);
        update_bounds(left + 1);
        subdivide(left);
        subdivide(left + 1);
    }
};
inline LightBvh build_light_bvh(const std::vector<V3> &pos, const std::vector<float> &rad) {
    LightBvh out;
    if (pos.empty()) return out;
    LightBvhBuilder b{pos, rad, {}, {}};
    for (size_t i = 0; i < pos.size(); ++i) b.idx.push_back(i);
    dl_light_bvh_node root{};
    root.left_first = 0;
    root.count = (uint32_t)pos.size();
    b.nodes.push_back(root);
    b.update_bounds(0);
    b.subdivide(0);
    out.nodes = b.nodes;
    out.order = b.idx;
    for (size_t i : b.idx) out.light_bounds.push_back(Aabb::from_sphere(pos[i], rad[i]));
    return out;
}

// ---- occluders (src/bake/occluder.rs) ----------------------------------------------------------
struct OccluderTriangle {
    V3 v[3];
    uint32_t mesh, triangle;
};

// intersect (occluder.rs:225-251): two-sided Möller–Trumbore, hits with 0 <= t <= max.
inline bool intersect_f32(const V3 v[3], V3 o, V3 d, float max, float &t_out, V3 &w_out) {
    V3 e1 = v[1] - v[0];
    V3 e2 = v[2] - v[0];
    V3 p = cross(d, e2);
    float det = dot(e1, p);
    if (det == 0.0f || !std::isfinite(det)) return false;
    float inv = 1.0f / det;
    V3 s = o - v[0];
    float u = dot(s, p) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    V3 q = cross(s, e1);
    float vv = dot(d, q) * inv;
    if (vv < 0.0f || u + vv > 1.0f) return false;
    float t = dot(e2, q) * inv;
    if (t >= 0.0f && t <= max) {
        t_out = t;
        w_out = V3{1.0f - u - vv, u, vv};
        return true;
    }
    return false;
}

// The same test in binary64 on the widened vertices and ray; t, u, v are rounded to binary32
// once and w = (1 - u - v, u, v) is formed from the rounded u, v in binary32.
inline bool intersect_f64(const V3 v[3], V3 o, V3 d, float max, float &t_out, V3 &w_out) {
    D3 a = widen(v[0]);
    D3 e1 = widen(v[1]) - a, e2 = widen(v[2]) - a;
    D3 dd = widen(d);
    D3 p = cross(dd, e2);
    double det = dot(e1, p);
    if (det == 0.0 || !std::isfinite(det)) return false;
    double inv = 1.0 / det;
    D3 s = widen(o) - a;
    double u = dot(s, p) * inv;
    if (!(u >= 0.0 && u <= 1.0)) return false;
    D3 q = cross(s, e1);
    double vv = dot(dd, q) * inv;
    if (vv < 0.0 || u + vv > 1.0) return false;
    double t = dot(e2, q) * inv;
    if (!(t >= 0.0 && t <= (double)max)) return false;
    float uf = (float)u, vf = (float)vv;
    t_out = (float)t;
    w_out = V3{1.0f - uf - vf, uf, vf};
    return true;
}

inline std::atomic<uint64_t> &retest_count() {
    static std::atomic<uint64_t> n{0};
    return n;
}

// The refined form's test: binary32 decides unless the ray is nearly parallel to the plane
// (det^2 <= eps^2 |e1|^2 |d x e2|^2) or u, v, u + v or t lie within eps of their bounds (t's
// margin eps * max(1, max) for a finite max, else eps); then intersect_f64 decides.
inline bool intersect_refined(const V3 v[3], V3 o, V3 d, float max, float &t_out, V3 &w_out) {
    const float eps = precision().eps;
    V3 e1 = v[1] - v[0];
    V3 e2 = v[2] - v[0];
    V3 p = cross(d, e2);
    float det = dot(e1, p);
    if (det * det > precision().eps2 * (dot(e1, e1) * dot(p, p))) {
        float inv = 1.0f / det;
        V3 s = o - v[0];
        float u = dot(s, p) * inv;
        if (!(u >= -eps && u <= 1.0f + eps)) return false;
        V3 q = cross(s, e1);
        float vv = dot(d, q) * inv;
        if (!(vv >= -eps) || u + vv > 1.0f + eps) return false;
        float t = dot(e2, q) * inv;
        float margin = eps * (std::isfinite(max) ? fmax_r(max, 1.0f) : 1.0f);
        if (!(t >= -margin && t <= max + margin)) return false;
        bool near = u < eps || u > 1.0f - eps || vv < eps || u + vv > 1.0f - eps || t < margin || t > max - margin;
        if (!near) {
            t_out = t;
            w_out = V3{1.0f - u - vv, u, vv};
            return true;
        }
    }
    retest_count().fetch_add(1, std::memory_order_relaxed);
    return intersect_f64(v, o, d, max, t_out, w_out);
}

inline bool intersect(const V3 v[3], V3 o, V3 d, float max, float &t_out, V3 &w_out) {
    switch (active_mode()) {
    case PREC_F64: return intersect_f64(v, o, d, max, t_out, w_out);
    case PREC_REFINED: return intersect_refined(v, o, d, max, t_out, w_out);
    default: return intersect_f32(v, o, d, max, t_out, w_out);
    }
}

// AlphaTexture::is_opaque (input.rs:79-97)
inline uint32_t wrap_texel(float coordinate, uint32_t size) {
    float r = std::fmod(coordinate, 1.0f);
    if (r < 0.0f) r = r + 1.0f;
    float texel = std::floor(r * (float)size);
    if (std::isfinite(texel)) return std::min(f2u_sat(texel), size - 1);
    return 0;
}
inline bool is_opaque(const dl_alpha_texture &a, V2 uv) {
    if (a.width == 0 || a.height == 0) return true;
    uint32_t x = wrap_texel(uv.x, a.width), y = wrap_texel(uv.y, a.height);
    uint8_t alpha = a.rgba8[((size_t)y * a.width + x) * 4 + 3];
    return (float)alpha / 255.0f >= a.cutoff;
}

struct SurfaceHit {
    float distance;
    uint32_t occluder;
    V3 w;
};

// The occluder set and its queries. The reference traverses obvhs's CWBVH; any-hit and
// tie-broken closest-hit depend only on the triangle set as long as box culling is
// conservative, so this oracle uses its own binary BVH with conservative slab tests (or brute
// force when asked), never a culling that could drop a hit the triangle test would report.
struct Occluders {
    std::vector<OccluderTriangle> triangles;
    const std::vector<const dl_mesh *> *meshes = nullptr;
    bool brute_force = false;

    struct Node {
        float lo[3], hi[3];
        uint32_t left, count;  // count > 0: leaf over prims[left .. left+count)
    };
    std::vector<Node> nodes;
    std::vector<uint32_t> prims;

    void build(const std::vector<const dl_mesh *> &sorted) {
        meshes = &sorted;
        for (uint32_t m = 0; m < sorted.size(); ++m) {
            const dl_mesh &mesh = *sorted[m];
            if (!mesh.occludes) continue;
            for (uint64_t t = 0; t < mesh.index_count / 3; ++t) {
                V3 v[3];
                for (int k = 0; k < 3; ++k) {
                    uint32_t i = mesh.indices[t * 3 + k];
                    v[k] = V3{mesh.positions[i * 3], mesh.positions[i * 3 + 1], mesh.positions[i * 3 + 2]};
                }
                V3 nrm = cross(v[1] - v[0], v[2] - v[0]);
                if (length_squared(nrm) > 0.0f && v3_finite(nrm))
                    triangles.push_back(OccluderTriangle{{v[0], v[1], v[2]}, m, (uint32_t)t});
            }
        }
        build_bvh();
    }

    void build_bvh() {
        nodes.clear();
        prims.resize(triangles.size());
        for (uint32_t i = 0; i < prims.size(); ++i) prims[i] = i;
        if (triangles.empty()) return;
        std::vector<V3> centroid(triangles.size());
        for (size_t i = 0; i < triangles.size(); ++i) {
            const auto &t = triangles[i];
            centroid[i] = V3{(t.v[0].x + t.v[1].x + t.v[2].x) / 3.0f, (t.v[0].y + t.v[1].y + t.v[2].y) / 3.0f,
                             (t.v[0].z + t.v[1].z + t.v[2].z) / 3.0f};
        }
        nodes.reserve(triangles.size() * 2 / 2 + 1);
        build_node(0, (uint32_t)prims.size(), centroid);
    }
    uint32_t build_node(uint32_t first, uint32_t count, const std::vector<V3> &centroid) {
        Node n{};
        Aabb box = Aabb::empty(), cbox = Aabb::empty();
        for (uint32_t k = first; k < first + count; ++k) {
            const auto &t = triangles[prims[k]];
            for (int j = 0; j < 3; ++j) box = box.grow(t.v[j]);
            cbox = cbox.grow(centroid[prims[k]]);
        }
        n.lo[0] = box.min.x; n.lo[1] = box.min.y; n.lo[2] = box.min.z;
        n.hi[0] = box.max.x; n.hi[1] = box.max.y; n.hi[2] = box.max.z;
        uint32_t index = (uint32_t)nodes.size();
        nodes.push_back(n);
        V3 ext = cbox.max - cbox.min;
        int ax = ext.x >= ext.y && ext.x >= ext.z ? 0 : (ext.y >= ext.z ? 1 : 2);
        float extent = ax == 0 ? ext.x : ax == 1 ? ext.y : ext.z;
        if (count <= 4 || !(extent > 0.0f)) {
            nodes[index].left = first;
            nodes[index].count = count;
            return index;
        }
        uint32_t mid = first + count / 2;
        auto key = [&](uint32_t p) { V3 c = centroid[p]; return ax == 0 ? c.x : ax == 1 ? c.y : c.z; };
        std::nth_element(prims.begin() + first, prims.begin() + mid, prims.begin() + first + count,
                         [&](uint32_t a, uint32_t b) { return key(a) < key(b) || (key(a) == key(b) && a < b); });
        uint32_t l = build_node(first, mid - first, centroid);
        uint32_t r = build_node(mid, first + count - mid, centroid);
        (void)l;
        nodes[index].left = r;  // left child is index + 1
        nodes[index].count = 0;
        return index;
    }

    // Conservative slab test: [0, tmax] against a box, with a relative slack that covers the
    // rounding of the slab distances and an absolute one for the triangle test's own rounding.
    static bool box_hit(const Node &n, V3 o, V3 inv, float tmax, float &tnear) {
        float t0 = 0.0f, t1 = tmax;
        const float oo[3] = {o.x, o.y, o.z}, ii[3] = {inv.x, inv.y, inv.z};
        for (int a = 0; a < 3; ++a) {
            float pad = (std::fabs(n.lo[a]) + std::fabs(n.hi[a])) * 1e-6f + 1e-6f;
            float lo = (n.lo[a] - pad - oo[a]) * ii[a];
            float hi = (n.hi[a] + pad - oo[a]) * ii[a];
            float a0 = fmin_r(lo, hi), a1 = fmax_r(lo, hi);
            t0 = fmax_r(t0, a0);
            t1 = fmin_r(t1, a1);
        }
        tnear = t0;
        return t0 <= t1 * 1.000002f;
    }
    static V3 safe_inverse(V3 d) {
        auto f = [](float x) { return 1.0f / (x == 0.0f ? std::copysign(1e-30f, x) : x); };
        return V3{f(d.x), f(d.y), f(d.z)};
    }

    bool blocks(const OccluderTriangle &occ, V3 w) const {
        const dl_mesh &mesh = *(*meshes)[occ.mesh];
        if (!mesh.alpha || !mesh.uv0) return true;
        const uint32_t *c = mesh.indices + (size_t)occ.triangle * 3;
        auto uv = [&](uint32_t i) { return V2{mesh.uv0[i * 2], mesh.uv0[i * 2 + 1]}; };
        V2 p = uv(c[0]) * w.x + uv(c[1]) * w.y + uv(c[2]) * w.z;
        return is_opaque(*mesh.alpha, p);
    }
    // hit_distance (occluder.rs:159-165)
    bool hit(uint32_t index, V3 o, V3 d, float max, bool alpha, float &t, V3 &w) const {
        const auto &occ = triangles[index];
        if (!intersect(occ.v, o, d, max, t, w)) return false;
        return !alpha || blocks(occ, w);
    }

    // occluded (occluder.rs:181-189)
    bool occluded(V3 o, V3 dir, float max, bool alpha) const {
        if (triangles.empty()) return false;
        V3 d = dir + V3{0.0f, 0.0f, 0.0f};
        float t;
        V3 w;
        if (brute_force) {
            for (uint32_t i = 0; i < triangles.size(); ++i)
                if (hit(i, o, d, max, alpha, t, w)) return true;
            return false;
        }
        V3 inv = safe_inverse(d);
        float tmax = fmax_r(max, 0.0f);
        uint32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp) {
            const Node &n = nodes[stack[--sp]];
            float tn;
            if (!box_hit(n, o, inv, tmax, tn)) continue;
            if (n.count) {
                for (uint32_t k = n.left; k < n.left + n.count; ++k)
                    if (hit(prims[k], o, d, max, alpha, t, w)) return true;
            } else {
                uint32_t self = (uint32_t)(&n - nodes.data());
                stack[sp++] = n.left;
                stack[sp++] = self + 1;
            }
        }
        return false;
    }

    // closest_hit (occluder.rs:191-220): nearest t, ties to the lowest occluder index.
    bool closest_hit(V3 o, V3 dir, float max, bool alpha, SurfaceHit &out) const {
        if (triangles.empty()) return false;
        V3 d = dir + V3{0.0f, 0.0f, 0.0f};
        bool found = false;
        float best = 0;
        uint32_t best_i = 0;
        V3 best_w{0, 0, 0};
        auto consider = [&](uint32_t i) {
            float t;
            V3 w;
            if (active_mode() == PREC_REFINED) {
                // candidates ordered by their binary64 distance, barycentrics from it too
                if (!intersect(triangles[i].v, o, d, max, t, w)) return;
                retest_count().fetch_add(1, std::memory_order_relaxed);
                if (!intersect_f64(triangles[i].v, o, d, max, t, w)) return;
                if (alpha && !blocks(triangles[i], w)) return;
            } else if (!hit(i, o, d, max, alpha, t, w)) {
                return;
            }
            if (std::isfinite(t) && (!found || t < best || (t == best && i < best_i))) {
                found = true;
                best = t;
                best_i = i;
                best_w = w;
            }
        };
        if (brute_force) {
            for (uint32_t i = 0; i < triangles.size(); ++i) consider(i);
        } else {
            V3 inv = safe_inverse(d);
            float tmax = fmax_r(max, 0.0f);
            uint32_t stack[128];
            int sp = 0;
            stack[sp++] = 0;
            while (sp) {
                const Node &n = nodes[stack[--sp]];
                float tn;
                if (!box_hit(n, o, inv, found ? fmin_r(tmax, best) : tmax, tn)) continue;
                if (n.count) {
                    for (uint32_t k = n.left; k < n.left + n.count; ++k) consider(prims[k]);
                } else {
                    uint32_t self = (uint32_t)(&n - nodes.data());
                    stack[sp++] = n.left;
                    stack[sp++] = self + 1;
                }
            }
        }
        if (!found) return false;
        if (active_mode() != PREC_F32) {
            // the winning test's own barycentrics (a re-test with max = infinity could take the
            // other precision path)
            out = SurfaceHit{best, best_i, best_w};
            return true;
        }
        float t;
        V3 w;
        if (!intersect(triangles[best_i].v, o, d, INFINITY, t, w)) return false;
        out = SurfaceHit{best, best_i, w};
        return true;
    }

    // face_normal (occluder.rs:117-122)
    V3 face_normal(const SurfaceHit &h) const {
        const auto &t = triangles[h.occluder];
        return normalize_or_zero(cross(t.v[1] - t.v[0], t.v[2] - t.v[0]));
    }
    // surface_normal (occluder.rs:126-139)
    V3 surface_normal(const SurfaceHit &h) const {
        const auto &occ = triangles[h.occluder];
        V3 face = face_normal(h);
        const dl_mesh &mesh = *(*meshes)[occ.mesh];
        if (!mesh.normals) return face;
        const uint32_t *c = mesh.indices + (size_t)occ.triangle * 3;
        auto nv = [&](uint32_t i) { return V3{mesh.normals[i * 3], mesh.normals[i * 3 + 1], mesh.normals[i * 3 + 2]}; };
        V3 n = nv(c[0]) * h.w.x + nv(c[1]) * h.w.y + nv(c[2]) * h.w.z;
        bool ok;
        V3 t = try_normalize(n, ok);
        return ok ? t : face;
    }
    V3 albedo(const SurfaceHit &h) const {
        const dl_mesh &mesh = *(*meshes)[triangles[h.occluder].mesh];
        return V3{mesh.albedo[0], mesh.albedo[1], mesh.albedo[2]};
    }
};

}  // namespace oracle
