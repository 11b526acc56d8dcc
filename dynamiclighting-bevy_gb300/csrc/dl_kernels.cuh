// Per-texel device functions of the bake: triangle setup and light association, texel
// generation, burial, and point/area/sun/sky visibility. Each restates the cited reference
// function in f32 with its operation order (dl_math.cuh has the conventions).
#pragma once

#include "dl_device.cuh"

namespace dl {

struct Rect {
    uint32_t min_x, min_y, max_x, max_y;
};

// ---- geometry (src/bake/geometry.rs) ----------------------------------------------------------
// Ericson's closest point on a triangle (geometry.rs:73-108).
__device__ __forceinline__ f3 closest_point(f3 p, f3 a, f3 b, f3 c) {
    f3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    f3 bp = sub(p, b);
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return add(a, scale(ab, d1 / (d1 - d3)));
    f3 cp = sub(p, c);
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return add(a, scale(ac, d2 / (d2 - d6)));
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
        return add(b, scale(sub(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6))));
    float denom = 1.0f / (va + vb + vc);
    return add(add(a, scale(ab, vb * denom)), scale(ac, vc * denom));
}
__device__ __forceinline__ float signed_area(f2 a, f2 b, f2 c) {
    float ax = a.x - c.x, ay = a.y - c.y, bx = b.x - c.x, by = b.y - c.y;
    return (ax * by - ay * bx) * 0.5f;
}
// geometry.rs:125-134
__device__ __forceinline__ bool uv_barycentrics(const f2 t[3], f2 p, f3 &w) {
    float area = signed_area(t[0], t[1], t[2]);
    if (area == 0.0f) return false;
    float a1 = signed_area(t[1], t[2], p) / area;
    float a2 = signed_area(t[2], t[0], p) / area;
    float a3 = signed_area(t[0], t[1], p) / area;
    if (a1 >= 0.0f && a2 >= 0.0f && a3 >= 0.0f) {
        w = f3{a1, a2, a3};
        return true;
    }
    return false;
}
__device__ __forceinline__ uint32_t clamp_texel(float v, uint32_t size) { return f2u(clampf(v, 0.0f, (float)(size - 1))); }
__device__ __forceinline__ void uv_bounds(const f2 uv[3], f2 &mn, f2 &mx) {
    mn = f2{fminf(fminf(uv[0].x, uv[1].x), uv[2].x), fminf(fminf(uv[0].y, uv[1].y), uv[2].y)};
    mx = f2{fmaxf(fmaxf(uv[0].x, uv[1].x), uv[2].x), fmaxf(fmaxf(uv[0].y, uv[1].y), uv[2].y)};
}
// mesh_builder.rs:103-135
__device__ __forceinline__ Rect crop_rect(const f2 uv[3], uint32_t size) {
    f2 mn, mx;
    uv_bounds(uv, mn, mx);
    float s = (float)size;
    return Rect{clamp_texel(floorf(mn.x * s) - 2.0f, size), clamp_texel(floorf(mn.y * s) - 2.0f, size),
                clamp_texel(ceilf(mx.x * s) + 2.0f, size), clamp_texel(ceilf(mx.y * s) + 2.0f, size)};
}
__device__ __forceinline__ Rect center_rect(const f2 uv[3], uint32_t size, float grow) {
    f2 mn, mx;
    uv_bounds(uv, mn, mx);
    float s = (float)size;
    return Rect{clamp_texel(floorf(mn.x * s - 0.5f) - grow, size), clamp_texel(floorf(mn.y * s - 0.5f) - grow, size),
                clamp_texel(ceilf(mx.x * s - 0.5f) + grow, size), clamp_texel(ceilf(mx.y * s - 0.5f) + grow, size)};
}
__device__ __forceinline__ f2 texel_center(uint32_t x, uint32_t y, uint32_t size) {
    return f2{((float)x + 0.5f) / (float)size, ((float)y + 0.5f) / (float)size};
}

// A triangle's corners (PreparedMesh::vertices/normals/uvs, mesh_builder.rs:78-101).
struct TriData {
    f3 v[3], n[3];
    f2 uv[3];
    uint32_t mesh, local, res;
};
__device__ __forceinline__ void load_tri(const DevScene &sc, uint32_t t, TriData &d) {
    uint32_t m = sc.tri_mesh[t];
    d.mesh = m;
    d.local = t - sc.mesh_tri_base[m];
    d.res = sc.mesh_res[m];
    const uint32_t *c = sc.indices + sc.mesh_index_base[m] + (size_t)d.local * 3;
    uint32_t vb = sc.mesh_vertex_base[m];
    bool normals = sc.mesh_flags[m] & kMeshNormals;
    for (int k = 0; k < 3; ++k) {
        size_t vi = (size_t)vb + c[k];
        d.v[k] = f3{sc.positions[vi * 3], sc.positions[vi * 3 + 1], sc.positions[vi * 3 + 2]};
        d.uv[k] = f2{sc.uv1[vi * 2], sc.uv1[vi * 2 + 1]};
        if (normals) d.n[k] = f3{sc.normals[vi * 3], sc.normals[vi * 3 + 1], sc.normals[vi * 3 + 2]};
    }
    if (!normals) {
        f3 f = normalize_or_zero(cross(sub(d.v[1], d.v[0]), sub(d.v[2], d.v[0])));
        d.n[0] = d.n[1] = d.n[2] = f;
    }
}

// BakeLight::may_face (src/bake/light_shape.rs:47-65)
__device__ __forceinline__ bool may_face(const DevLight &l, const f3 v[3], f3 normal) {
    if (l.shape == DL_SHAPE_SKY) return true;
    if (l.shape == DL_SHAPE_SUN) return dot(normal, l.toward) + l.sin_radius > kNdotlTolerance;
    f3 center = divs(add(add(v[0], v[1]), v[2]), 3.0f);
    if (!(l.flags & kLightArea)) return dot(normal, normalize_or_zero(sub(l.position, center))) > kNdotlTolerance;
    bool rect = l.flags & kLightRect;
    bool lit_side = !rect;
    for (int k = 0; k < 3 && !lit_side; ++k) lit_side = dot(l.forward, sub(v[k], l.position)) > 0.0f;
    if (!lit_side) return false;
    f3 hx = scale(l.ax, l.half_x), hy = scale(l.ay, l.half_y), c = l.position;
    f3 corners[4] = {sub(sub(c, hx), hy), sub(add(c, hx), hy), add(add(c, hx), hy), add(sub(c, hx), hy)};
    for (int k = 0; k < 4; ++k)
        if (dot(normal, normalize_or_zero(sub(corners[k], center))) > kNdotlTolerance) return true;
    return false;
}

// associate (src/bake/mesh_bake.rs:141-173): calls `emit(slot)` for every light of the
// triangle in ascending slot order. Local lights come from the light-BVH query, which equals a
// scan of the lights' sphere boxes (light_bvh.rs:191-219); distant lights always follow.
template <class Emit>
__device__ __forceinline__ void associate(const DevScene &sc, const TriData &d, f3 face, Emit emit) {
    bool valid = !is_zero(face);
    bool flat = approx_eq(d.n[0], d.n[1], 1e-5f) && approx_eq(d.n[1], d.n[2], 1e-5f);
    f3 lo = vmin(vmin(vmin(f3{INFINITY, INFINITY, INFINITY}, d.v[0]), d.v[1]), d.v[2]);
    f3 hi = vmax(vmax(vmax(f3{-INFINITY, -INFINITY, -INFINITY}, d.v[0]), d.v[1]), d.v[2]);
    for (uint32_t s = 0; s < sc.light_count; ++s) {
        const DevLight &l = sc.lights[s];
        bool distant = l.flags & kLightDistant;
        if (!distant) {
            bool overlap = l.bounds_lo.x <= hi.x && l.bounds_lo.y <= hi.y && l.bounds_lo.z <= hi.z &&
                           lo.x <= l.bounds_hi.x && lo.y <= l.bounds_hi.y && lo.z <= l.bounds_hi.z;
            if (!overlap) continue;
        }
        if (valid && flat && !(l.flags & kLightBounce) && !may_face(l, d.v, face)) continue;
        if (distant) {
            emit(s);
            continue;
        }
        f3 cp = closest_point(l.position, d.v[0], d.v[1], d.v[2]);
        if (length_sq(sub(cp, l.position)) <= l.radius * l.radius) emit(s);
    }
}

// uv_to_surface (src/bake/texels.rs:24-37) at barycentrics w.
__device__ __forceinline__ void surface_at(const TriData &d, f3 face, f3 w, f3 &pos, f3 &nrm) {
    pos = add(add(scale(d.v[0], w.x), scale(d.v[1], w.y)), scale(d.v[2], w.z));
    bool ok;
    f3 n = try_normalize(add(add(scale(d.n[0], w.x), scale(d.n[1], w.y)), scale(d.n[2], w.z)), ok);
    nrm = ok ? n : face;
}
// nearest_weights (src/bake/texels.rs:125-141)
__device__ __forceinline__ bool nearest_weights(const f2 uv[3], f2 point, f3 &w_out) {
    f3 a{uv[0].x, uv[0].y, 0.0f}, b{uv[1].x, uv[1].y, 0.0f}, c{uv[2].x, uv[2].y, 0.0f};
    f3 n3 = closest_point(f3{point.x, point.y, 0.0f}, a, b, c);
    f3 nearest{n3.x, n3.y, 0.0f};
    float area = cross(sub(b, a), sub(c, a)).z;
    if (area == 0.0f || !isfinite(area)) return false;
    float w0 = cross(sub(b, nearest), sub(c, nearest)).z;
    float w1 = cross(sub(c, nearest), sub(a, nearest)).z;
    float w2 = cross(sub(a, nearest), sub(b, nearest)).z;
    f3 w = f3{fmaxf(w0 / area, 0.0f), fmaxf(w1 / area, 0.0f), fmaxf(w2 / area, 0.0f)};
    float sum = (w.x + w.y) + w.z;
    w_out = divs(w, fmaxf(sum, 1.17549435e-38f));
    return true;
}

// ---- visibility (src/bake/texel_shadow.rs, area.rs, sun.rs, sky.rs) --------------------------
struct Vis {
    bool some;
    uint32_t level;
    uint32_t rays;
};

template <bool COUNT = false>
struct Tracer {
    const DevScene &sc;
    f3 origin;
    bool alpha;
    int *stack;
    int stride;
    Visits *vis;
    __device__ __forceinline__ bool operator()(f3 dir, float dist) const {
        return occluded<COUNT>(sc, origin, dir, dist, alpha, stack, stride, vis);
    }
};

// adaptive_share (area.rs:98-126); `Trace(point, w, unblocked)` is false for a point that sends
// no light, `Point(i)` the i-th spread point.
template <class Trace, class Point>
__device__ __forceinline__ bool adaptive_share(const f2 *probes, int nprobes, uint32_t samples, uint32_t minimum,
                                               Point spread_point, Trace trace, float &fraction) {
    bool any_lit = false, any_blocked = false;
    for (int i = 0; i < nprobes; ++i) {
        float w;
        bool lit;
        if (trace(probes[i], w, lit)) {
            any_lit |= lit;
            any_blocked |= !lit;
        }
    }
    float lit_sum = 0.0f, total = 0.0f;
    for (uint32_t taken = 0; taken < samples; ++taken) {
        if (taken == minimum && any_lit != any_blocked) break;
        float w;
        bool unblocked;
        if (trace(spread_point(taken), w, unblocked)) {
            total += w;
            lit_sum += unblocked ? w : 0.0f;
            any_lit |= unblocked;
            any_blocked |= !unblocked;
        }
    }
    if (any_lit != any_blocked) {
        fraction = any_lit ? 1.0f : 0.0f;
        return true;
    }
    if (total > 0.0f) {
        fraction = lit_sum / total;
        return true;
    }
    return false;
}

// point_texel (texel_shadow.rs:71-90)
template <class TR>
__device__ __forceinline__ Vis point_vis(const DevLight &l, f3 pos, f3 nrm, const TR &tr) {
    f3 to = sub(l.position, pos);
    float dsq = length_sq(to);
    if (dsq > l.radius * l.radius) return Vis{false, 0, 0};
    float d = sqrtf(dsq);
    if (d == 0.0f) return Vis{true, 1, 0};
    f3 dir = divs(to, d);
    if (dot(nrm, dir) <= kNdotlTolerance) return Vis{false, 0, 0};
    return Vis{true, tr(dir, d) ? 0u : 1u, 1};
}

// texel_visibility (area.rs:61-90) with toward (area.rs:130-146)
template <class TR>
__device__ __forceinline__ Vis area_vis(const DevScene &sc, const DevLight &l, f3 pos, f3 nrm, Pcg &rng,
                                        const TR &tr) {
    bool rect = l.flags & kLightRect;
    f3 local = sub(pos, l.position);
    float lx = clampf(dot(local, l.ax), -l.half_x, l.half_x);
    float ly = clampf(dot(local, l.ay), -l.half_y, l.half_y);
    f3 nearest = add(add(l.position, scale(l.ax, lx)), scale(l.ay, ly));
    if (l.reach <= 0.0f || length_sq(sub(pos, nearest)) > l.reach * l.reach) return Vis{false, 0, 0};
    if (rect && dot(l.forward, sub(pos, l.position)) <= 0.0f) return Vis{false, 0, 0};
    uint32_t rays = 0;
    auto trace = [&](f2 uv, float &w, bool &unblocked) {
        float ox = (uv.x * 2.0f - 1.0f) * l.half_x, oy = (uv.y * 2.0f - 1.0f) * l.half_y;
        f3 point = add(add(l.position, scale(l.ax, ox)), scale(l.ay, oy));
        f3 to = sub(point, pos);
        float dsq = length_sq(to);
        if (dsq < 1.0e-12f) return false;
        float dist = sqrtf(dsq);
        f3 dir = divs(to, dist);
        float receiver = dot(nrm, dir) - kNdotlTolerance;
        float emitter = rect ? -dot(l.forward, dir) : 1.0f;
        if (!(receiver > 0.0f && emitter > 0.0f)) return false;
        w = receiver * emitter / dsq;
        rays += 1;
        unblocked = !tr(dir, fmaxf(dist - kEndGap, 0.0f));
        return true;
    };
    f2 off;
    off.x = rng.next_f32();
    off.y = rng.next_f32();
    auto spread_point = [&](uint32_t taken) { return spread(taken, off, rect); };
    const f2 rect_probes[5] = {{0.0f, 0.0f}, {1.0f, 0.0f}, {1.0f, 1.0f}, {0.0f, 1.0f}, {0.5f, 0.5f}};
    const f2 tube_probes[3] = {{0.0f, 0.5f}, {1.0f, 0.5f}, {0.5f, 0.5f}};
    float fraction;
    bool some = adaptive_share(rect ? rect_probes : tube_probes, rect ? 5 : 3, sc.area_samples, sc.area_min_samples,
                               spread_point, trace, fraction);
    return Vis{some, some ? level_of(fraction, l.shadow_bits) : 0u, rays};
}

// sun_visibility (sun.rs:21-56)
template <class TR>
__device__ __forceinline__ Vis sun_vis(const DevScene &sc, const DevLight &l, f3 nrm, Pcg &rng, const TR &tr) {
    if (l.angular_radius <= 0.0f) {
        if (dot(nrm, l.toward) <= kNdotlTolerance) return Vis{false, 0, 0};
        bool lit = !tr(l.toward, INFINITY);
        return Vis{true, lit ? 1u : 0u, 1};
    }
    f3 side, up;
    ortho_pair(l.toward, side, up);
    uint32_t rays = 0;
    auto trace = [&](f2 disk, float &w, bool &unblocked) {
        f3 dir = normalize(add(l.toward, scale(add(scale(side, disk.x), scale(up, disk.y)), l.tan_radius)));
        float receiver = dot(nrm, dir) - kNdotlTolerance;
        if (receiver <= 0.0f) return false;
        rays += 1;
        w = receiver;
        unblocked = !tr(dir, INFINITY);
        return true;
    };
    f2 off;
    off.x = rng.next_f32();
    off.y = rng.next_f32();
    auto spread_point = [&](uint32_t taken) { return concentric(spread(taken, off, true)); };
    const f2 disk_probes[5] = {{0.0f, 0.0f}, {1.0f, 0.0f}, {0.0f, 1.0f}, {-1.0f, 0.0f}, {0.0f, -1.0f}};
    float fraction;
    bool some = adaptive_share(disk_probes, 5, sc.area_samples, sc.area_min_samples, spread_point, trace, fraction);
    return Vis{some, some ? level_of(fraction, l.shadow_bits) : 0u, rays};
}

// sky_visibility (sky.rs:30-44)
template <class TR>
__device__ __forceinline__ Vis sky_vis(const DevScene &sc, const DevLight &l, f3 nrm, Pcg &rng, const TR &tr) {
    f2 off;
    off.x = rng.next_f32();
    off.y = rng.next_f32();
    uint32_t open = 0;
    uint32_t samples = sc.sky_samples;
    for (uint32_t taken = 0; taken < samples; ++taken)
        if (!tr(cosine_direction(nrm, spread(taken, off, true)), INFINITY)) ++open;
    float fraction = (float)open / (float)(samples > 1 ? samples : 1);
    return Vis{true, level_of(fraction, l.shadow_bits), samples};
}

// texel_shadow (texel_shadow.rs:20-67)
template <class TR>
__device__ __forceinline__ Vis texel_shadow(const DevScene &sc, uint32_t slot, uint64_t mesh_id, uint32_t x,
                                            uint32_t y, f3 pos, f3 nrm, const TR &tr) {
    const DevLight &l = sc.lights[slot];
    if (l.shape == DL_SHAPE_POINT) return point_vis(l, pos, nrm, tr);
    Pcg rng = stream5(sc.seed, mesh_id, l.id, x, y);
    if (l.shape == DL_SHAPE_SUN) return sun_vis(sc, l, nrm, rng, tr);
    if (l.shape == DL_SHAPE_SKY) return sky_vis(sc, l, nrm, rng, tr);
    return area_vis(sc, l, pos, nrm, rng, tr);
}

// is_buried (mesh_texels.rs:111-135) with the back-face closest-hit test (:78-84). Returns the
// verdict and adds the rays traced to `rays`.
__device__ __forceinline__ bool is_buried(const DevScene &sc, f3 normal, f3 origin, float turn, int *stack,
                                          int stride, uint32_t &rays) {
    f3 tangent, bitangent;
    ortho_pair(normal, tangent, bitangent);
    uint32_t back = 0, front = 0;
    for (uint32_t i = 0; i < 8; ++i) {
        float ring = (float)((i * 5) % 8) + 0.5f;
        float sin_theta = sqrtf(ring / 8.0f);
        float cos_theta = sqrtf(1.0f - sin_theta * sin_theta);
        float phi = ((float)i + turn) * kTau / 8.0f;
        float sp, cp;
        sincos_f(phi, sp, cp);
        f3 dir = add(scale(add(scale(tangent, cp), scale(bitangent, sp)), sin_theta), scale(normal, cos_theta));
        ++rays;
        Hit h;
        bool backface = false;
        if (traverse<false>(sc, origin, dir, INFINITY, false, stack, stride, h)) {
            // face normal of the hit occluder: cross(b - a, c - a), normalized
            float4 e1 = ldg4(sc.tri_e1 + sc.occ_leaf[h.occluder]), e2 = ldg4(sc.tri_e2 + sc.occ_leaf[h.occluder]);
            f3 fn = normalize_or_zero(cross(f3{e1.x, e1.y, e1.z}, f3{e2.x, e2.y, e2.z}));
            backface = dot(fn, dir) > 0.0f;
        }
        if (backface)
            ++back;
        else
            ++front;
        if (back >= 5) return true;
        if (front > 8 - 5) return false;
    }
    return false;
}

}  // namespace dl
