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

// A shadow-ray tracer from one origin; REFINE selects the refined form's triangle test and
// compensated sums in the visibility functions that use it.
template <bool COUNT = false, bool REFINE = false>
struct Tracer {
    static constexpr bool kRefine = REFINE;
    const DevScene &sc;
    f3 origin;
    bool alpha;
    int *stack;
    int stride;
    Visits *vis;
    __device__ __forceinline__ bool operator()(f3 dir, float dist) const {
        return occluded<COUNT, REFINE>(sc, origin, dir, dist, alpha, stack, stride, vis);
    }
};

// adaptive_share (area.rs:98-126); `Trace(point, w, unblocked)` is false for a point that sends
// no light, `Point(i)` the i-th spread point.
template <bool KAHAN, class Trace, class Point>
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
    FSum<KAHAN> lit_sum, total;
    for (uint32_t taken = 0; taken < samples; ++taken) {
        if (taken == minimum && any_lit != any_blocked) break;
        float w;
        bool unblocked;
        if (trace(spread_point(taken), w, unblocked)) {
            total.add(w);
            lit_sum.add(unblocked ? w : 0.0f);
            any_lit |= unblocked;
            any_blocked |= !unblocked;
        }
    }
    if (any_lit != any_blocked) {
        fraction = any_lit ? 1.0f : 0.0f;
        return true;
    }
    if (total.s > 0.0f) {
        fraction = lit_sum.s / total.s;
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
    bool some = adaptive_share<TR::kRefine>(rect ? rect_probes : tube_probes, rect ? 5 : 3, sc.area_samples,
                                            sc.area_min_samples, spread_point, trace, fraction);
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
    bool some = adaptive_share<TR::kRefine>(disk_probes, 5, sc.area_samples, sc.area_min_samples, spread_point, trace,
                                            fraction);
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
    f3 side, across;
    ortho_pair(nrm, side, across);
    for (uint32_t taken = 0; taken < samples; ++taken)
        if (!tr(cosine_direction_basis(nrm, side, across, spread(taken, off, true)), INFINITY)) ++open;
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
template <bool REFINE = false>
__device__ __forceinline__ bool is_buried(const DevScene &sc, f3 normal, f3 origin, float turn, int *stack,
                                          int stride, uint32_t &rays, Visits *vis = nullptr) {
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
        if (traverse<false, false, REFINE>(sc, origin, dir, INFINITY, false, stack, stride, h, vis)) {
            // face normal of the hit occluder: cross(b - a, c - a), normalized
            const float4 *tp = sc.tris + (size_t)sc.occ_leaf[h.occluder] * 3;
            float4 e1 = ldg4(tp + 1), e2 = ldg4(tp + 2);
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

namespace dl {

// ---- one bounce (src/bake/bounce.rs, sun_bounce.rs, shared/cube.rs) --------------------------

// A photon (bounce.rs:29-39): distance, normal as i8 x 3 and albedo as u8 x 3.
struct Photon {
    float distance;
    uint32_t normal;  // bytes x, y, z (two's complement)
    uint32_t albedo;  // bytes r, g, b
};

// face_uv_to_direction / texel_direction (cube.rs:57-79)
__device__ __forceinline__ f3 cube_texel_direction(uint32_t face, uint32_t x, uint32_t y, uint32_t res) {
    float size = (float)res;
    float sc = ((float)x + 0.5f) / size * 2.0f - 1.0f, tc = ((float)y + 0.5f) / size * 2.0f - 1.0f;
    f3 d;
    switch (face) {
        case 0: d = f3{1.0f, -tc, -sc}; break;
        case 1: d = f3{-1.0f, -tc, sc}; break;
        case 2: d = f3{sc, 1.0f, tc}; break;
        case 3: d = f3{sc, -1.0f, -tc}; break;
        case 4: d = f3{sc, -tc, 1.0f}; break;
        default: d = f3{-sc, -tc, -1.0f}; break;
    }
    return normalize(d);
}
// direction_to_face_uv + direction_to_texel (cube.rs:29-53, 94-105): the flat texel index.
__device__ __forceinline__ uint32_t cube_texel_index(f3 d, uint32_t res) {
    f3 a{fabsf(d.x), fabsf(d.y), fabsf(d.z)};
    uint32_t face;
    float sc, tc, ma;
    if (a.x > a.y && a.x > a.z) {
        if (d.x > 0.0f) { face = 0; sc = -d.z; tc = -d.y; }
        else { face = 1; sc = d.z; tc = -d.y; }
        ma = a.x;
    } else if (a.y > a.z) {
        if (d.y > 0.0f) { face = 2; sc = d.x; tc = d.z; }
        else { face = 3; sc = d.x; tc = -d.z; }
        ma = a.y;
    } else if (d.z > 0.0f) {
        face = 4; sc = d.x; tc = -d.y; ma = a.z;
    } else {
        face = 5; sc = -d.x; tc = -d.y; ma = a.z;
    }
    float u = 0.5f, v = 0.5f;
    if (ma != 0.0f) {
        u = (sc / ma) * 0.5f + 0.5f;
        v = (tc / ma) * 0.5f + 0.5f;
    }
    float max = (float)(res - 1);
    uint32_t x = f2u(clampf(floorf(u * (float)res), 0.0f, max));
    uint32_t y = f2u(clampf(floorf(v * (float)res), 0.0f, max));
    return face * res * res + y * res + x;
}

// Occluder::face_normal / surface_normal / albedo (occluder.rs:117-144) at a closest hit.
__device__ __forceinline__ f3 hit_face_normal(const DevScene &sc, const Hit &h) {
    uint32_t leaf = sc.occ_leaf[h.occluder];
    float4 e1 = ldg4(sc.tris + (size_t)leaf * 3 + 1), e2 = ldg4(sc.tris + (size_t)leaf * 3 + 2);
    return normalize_or_zero(cross(f3{e1.x, e1.y, e1.z}, f3{e2.x, e2.y, e2.z}));
}
__device__ __forceinline__ f3 hit_surface_normal(const DevScene &sc, const Hit &h, f3 face) {
    uint32_t m = sc.occ_mesh[h.occluder];
    if (!(sc.mesh_flags[m] & kMeshNormals)) return face;
    const uint32_t *c = sc.indices + sc.mesh_index_base[m] + (size_t)sc.occ_tri[h.occluder] * 3;
    uint32_t vb = sc.mesh_vertex_base[m];
    float wx = 1.0f - h.u - h.v;
    f3 n{0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 3; ++k) {
        size_t vi = (size_t)vb + c[k];
        f3 nv{sc.normals[vi * 3], sc.normals[vi * 3 + 1], sc.normals[vi * 3 + 2]};
        float w = k == 0 ? wx : k == 1 ? h.u : h.v;
        n = k == 0 ? scale(nv, w) : add(n, scale(nv, w));
    }
    bool ok;
    f3 t = try_normalize(n, ok);
    return ok ? t : face;
}
__device__ __forceinline__ f3 hit_albedo(const DevScene &sc, const Hit &h) {
    const float *a = sc.mesh_albedo + (size_t)sc.occ_mesh[h.occluder] * 3;
    return f3{a[0], a[1], a[2]};
}

// photon (bounce.rs:88-115)
template <bool REFINE = false>
__device__ __forceinline__ Photon make_photon(const DevScene &sc, const DevLight &l, f3 dir, int *stack, int stride,
                                              Visits *vis = nullptr) {
    Hit h;
    if (!traverse<false, false, REFINE>(sc, l.position, dir, l.radius, (l.flags & kLightAlpha) != 0, stack, stride, h,
                                        vis))
        return Photon{l.radius, 0u, 0u};
    f3 face = hit_face_normal(sc, h);
    f3 normal = hit_surface_normal(sc, h, face);
    f3 point = add(l.position, scale(dir, h.t));
    float bias = fmaxf(h.t * 0.001f, 0.001f);
    f3 nudged = add(sub(point, scale(dir, bias)), scale(normal, bias));
    bool lit_side = dot(face, dir) < 0.0f;
    Photon p;
    p.distance = length(sub(nudged, l.position));
    p.normal = 0;
    if (lit_side) {
        uint32_t nx = (uint32_t)(f2i8(roundf(normal.x * 127.0f)) & 0xFF);
        uint32_t ny = (uint32_t)(f2i8(roundf(normal.y * 127.0f)) & 0xFF);
        uint32_t nz = (uint32_t)(f2i8(roundf(normal.z * 127.0f)) & 0xFF);
        p.normal = nx | (ny << 8) | (nz << 16);
    }
    f3 a = hit_albedo(sc, h);
    p.albedo = f2u8(roundf(clampf(a.x, 0.0f, 1.0f) * 255.0f)) | (f2u8(roundf(clampf(a.y, 0.0f, 1.0f) * 255.0f)) << 8) |
               (f2u8(roundf(clampf(a.z, 0.0f, 1.0f) * 255.0f)) << 16);
    return p;
}

// glam's Vec3::slerp as gather_triangle calls it (bounce.rs:270), operation for operation in
// f32 with no fused operations: the angle from acos_approx (the 7-degree polynomial of
// Abramowitz & Stegun 4.4.46 in Horner form, sqrt(1 - |x|) * p(|x|), pi minus it below zero), a
// sine-weighted blend while |cos| < 1 - 3 * 2^-23 with the length interpolated linearly, a turn
// by pi * s about a unit vector orthogonal to `a` when nearly opposite (Quat::from_axis_angle,
// then glam's Quat * Vec3), and the plain lerp when nearly equal.
__device__ __forceinline__ f3 slerp3(f3 a, f3 b, float s) {
    const float la = length(a), lb = length(b);
    const float d = dot(a, b) / (la * lb);
    const float eps = 1.1920928955078125e-7f;  // f32::EPSILON
    if (fabsf(d) < 1.0f - 3.0f * eps) {
        const float angle = acos_approx(d);
        // three sines in a row: one shared out-of-line copy keeps the gather's code small
        const float angle_sin = sin_f_outline(angle);
        const float t1 = sin_f_outline(angle * (1.0f - s)) / angle_sin;
        const float t2 = sin_f_outline(angle * s) / angle_sin * (la / lb);
        return scale(add(scale(a, t1), scale(b, t2)), 1.0f + s * (lb / la - 1.0f));
    }
    if (d < 0.0f) {
        const f3 axis = normalize(fabsf(a.x) > fabsf(a.y) ? f3{-a.z, 0.0f, a.x} : f3{0.0f, a.z, -a.y});
        float sh, ch;
        sincos_f(kPiF * s * 0.5f, sh, ch);
        const float q[4] = {axis.x * sh, axis.y * sh, axis.z * sh, ch};
        return scale(quat_rotate(q, a), 1.0f + s * (lb / la - 1.0f));
    }
    return add(scale(a, 1.0f - s), scale(b, s));
}

__device__ __forceinline__ f3 reflected(const DevScene &sc, f3 albedo) {
    return sc.colored_bounce ? albedo : f3{1.0f, 1.0f, 1.0f};
}

// The gathers below split a texel's samples over a group of lanes: each lane evaluates single
// samples and the group leader adds their contributions in sample order, so the sums are the
// reference's sequential ones (bounce.rs:282, sun_bounce.rs:70).

// One sample's contribution: `add` is false for a sample the reference skips (no sum term).
struct Contribution {
    f3 value;
    bool add;
    uint32_t rays;
};

// gather_triangle's per-texel setup (bounce.rs:252-266): false when the texel is out of reach.
struct LocalGather {
    f3 direction;
    Pcg rng;  // the stream at the lane's first sample
    float step;
};
__device__ __forceinline__ bool local_setup(const DevScene &sc, const DevLight &l, uint64_t mesh_id, uint32_t x,
                                            uint32_t y, f3 pos, uint32_t first, LocalGather &g) {
    f3 to_texel = sub(pos, l.position);
    if (length_sq(to_texel) > l.radius * l.radius) return false;
    g.direction = normalize_or(to_texel, f3{0.0f, 1.0f, 0.0f});
    g.rng = stream5(sc.seed, mesh_id, l.id, x, y);
    g.rng.advance(2ull * first);  // on_unit_sphere takes two draws per sample
    g.step = 0.9f / (float)(l.bounce_samples - 1);
    return true;
}
// Sample i of gather_triangle (bounce.rs:267-289); `g.rng` must stand at sample i.
template <class TR>
__device__ __forceinline__ Contribution local_sample(const DevScene &sc, const DevLight &l, const Photon *cube,
                                                    uint32_t res, f3 normal, LocalGather &g, uint32_t i,
                                                    const TR &tr) {
    Contribution c{f3{0.0f, 0.0f, 0.0f}, false, 0};
    float spread_s = 0.1f + (float)i * g.step;
    f3 random = on_unit_sphere(g.rng);
    f3 sample = normalize_or(slerp3(g.direction, random, spread_s), g.direction);
    Photon ph = cube[cube_texel_index(sample, res)];
    f3 pn{(float)(int8_t)(ph.normal & 0xFF) / 127.0f, (float)(int8_t)((ph.normal >> 8) & 0xFF) / 127.0f,
          (float)(int8_t)((ph.normal >> 16) & 0xFF) / 127.0f};
    pn = normalize_or_zero(pn);
    f3 photon = add(l.position, scale(sample, ph.distance));
    f3 albedo{(float)(ph.albedo & 0xFF) / 255.0f, (float)((ph.albedo >> 8) & 0xFF) / 255.0f,
              (float)((ph.albedo >> 16) & 0xFF) / 255.0f};
    f3 to_photon = sub(photon, tr.origin);
    float distance = length(to_photon);
    if (is_zero(pn) || distance <= 0.0f) return c;
    f3 d = divs(to_photon, distance);
    c.rays = 1;
    if (!tr(d, distance)) {
        float weight = fmaxf(dot(normal, d), 0.0f) * fmaxf(dot(pn, neg(d)), 0.0f);
        c.value = scale(reflected(sc, albedo), weight);
        c.add = true;
    }
    return c;
}

// gather_sun's per-texel setup (sun_bounce.rs:43-52).
struct SunGather {
    f2 off;
    f3 side, across;
};
__device__ __forceinline__ void sun_setup(const DevScene &sc, const DevLight &l, uint64_t mesh_id, uint32_t x,
                                          uint32_t y, f3 normal, SunGather &g) {
    Pcg rng = stream5(sc.seed, mesh_id, l.id, x, y);
    g.off.x = rng.next_f32();
    g.off.y = rng.next_f32();
    ortho_pair(normal, g.side, g.across);
}
// The closest-hit half of sample i of gather_sun (sun_bounce.rs:53-66): `pending` when the hit
// faces the ray and the sun and is lit by it, with the shadow ray's origin `point` and the value
// the sample adds if that ray is open (sun_bounce.rs:67-70). One ray.
struct SunHit {
    f3 value, point;
    bool pending;
};
template <bool COUNT, bool REFINE>
__device__ __forceinline__ SunHit sun_hit(const DevScene &sc, const DevLight &l, f3 origin, f3 normal,
                                          const SunGather &g, uint32_t i, int *stack, int stride, Visits *vis) {
    SunHit r{f3{0.0f, 0.0f, 0.0f}, f3{0.0f, 0.0f, 0.0f}, false};
    bool alpha = (l.flags & kLightAlpha) != 0;
    f3 direction = cosine_direction_basis(normal, g.side, g.across, spread(i, g.off, true));
    Hit h;
    if (!traverse<false, COUNT, REFINE>(sc, origin, direction, INFINITY, alpha, stack, stride, h, vis)) return r;
    f3 face = hit_face_normal(sc, h);
    if (dot(face, direction) >= 0.0f) return r;
    float lit = dot(hit_surface_normal(sc, h, face), l.toward);
    if (lit <= 0.0f || dot(face, l.toward) <= 0.0f) return r;
    r.point = add(add(origin, scale(direction, h.t)), scale(face, kRayOffset));
    r.value = scale(reflected(sc, hit_albedo(sc, h)), lit);
    r.pending = true;
    return r;
}
// Whether the shadow ray of a pending sun-bounce sample is open (sun_bounce.rs:67).
template <bool COUNT, bool REFINE>
__device__ __forceinline__ bool sun_open(const DevScene &sc, const DevLight &l, f3 point, int *stack, int stride,
                                         Visits *vis) {
    return !occluded<COUNT, REFINE>(sc, point, l.toward, INFINITY, (l.flags & kLightAlpha) != 0, stack, stride, vis);
}
// Sample i of gather_sun (sun_bounce.rs:53-71).
template <bool COUNT, bool REFINE>
__device__ __forceinline__ Contribution sun_sample(const DevScene &sc, const DevLight &l, f3 origin, f3 normal,
                                                  const SunGather &g, uint32_t i, int *stack, int stride,
                                                  Visits *vis) {
    Contribution c{f3{0.0f, 0.0f, 0.0f}, false, 1};
    SunHit h = sun_hit<COUNT, REFINE>(sc, l, origin, normal, g, i, stack, stride, vis);
    if (!h.pending) return c;
    c.rays = 2;
    if (sun_open<COUNT, REFINE>(sc, l, h.point, stack, stride, vis)) {
        c.value = h.value;
        c.add = true;
    }
    return c;
}

// quantize (bounce_pack.rs:74-86)
__device__ __forceinline__ uint32_t quantize_bounce(float value, uint32_t bits, Pcg &rng) {
    float max = (float)((1u << bits) - 1);
    float amplitude = bits == 8 ? 0.0f : bits == 6 ? 0.004f : bits == 5 ? 0.008f : 0.02f;
    float color = isnan(value) ? 0.0f : clampf(value, 0.0f, 1.0f);
    if (amplitude > 0.0f && color > 0.001f) color = fminf(color + rng.next_f32() * amplitude, 1.0f);
    return f2u(sqrtf(color) * max);
}

}  // namespace dl
