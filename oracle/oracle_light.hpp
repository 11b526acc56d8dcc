// TEST INFRASTRUCTURE — the parity oracle, not the product.
//
// Lights, low-discrepancy points and per-texel visibility of the reference baker: point,
// area (rectangle/tube), sun and sky, restated in f32 from the cited reference functions.
#pragma once

#include "oracle_scene.hpp"

namespace oracle {

constexpr float NDOTL_TOLERANCE = -0.1f;  // mesh_bake.rs:25
constexpr float RAY_OFFSET = 0.001f;      // mesh_bake.rs:27
constexpr float END_GAP = 1.0e-3f;        // area.rs:33
constexpr uint32_t AREA_SHADOW_BITS = 4;  // area.rs:14
constexpr uint32_t SKY_SHADOW_BITS = 8;   // sky.rs:15

// AreaShape (src/light/area.rs:80-123) at a light's position.
struct AreaShape {
    V3 center, x, y, forward;
    V2 half;
    bool rectangle;
    // area.rs:98-103
    V3 nearest_point(V3 world) const {
        V3 local = world - center;
        float lx = clampf(dot(local, x), -half.x, half.x);
        float ly = clampf(dot(local, y), -half.y, half.y);
        return center + x * lx + y * ly;
    }
    // area.rs:106-109
    V3 point_at(V2 uv) const {
        V2 off{(uv.x * 2.0f - 1.0f) * half.x, (uv.y * 2.0f - 1.0f) * half.y};
        return center + x * off.x + y * off.y;
    }
    // area.rs:112-117
    void corners(V3 out[4]) const {
        V3 hx = x * half.x, hy = y * half.y;
        out[0] = center - hx - hy;
        out[1] = center + hx - hy;
        out[2] = center + hx + hy;
        out[3] = center - hx + hy;
    }
};

// A BakeLight with the derived quantities of src/bake/light_shape.rs and src/light/shape.rs.
struct Light {
    const dl_light *l;
    bool is_distant() const { return l->shape == DL_SHAPE_SUN || l->shape == DL_SHAPE_SKY; }
    bool is_area() const { return l->shape == DL_SHAPE_RECTANGLE || l->shape == DL_SHAPE_TUBE; }
    V3 position() const { return V3{l->position[0], l->position[1], l->position[2]}; }
    // input.rs:176-180
    bool bakes_bounce(const dl_bake_options &o) const {
        return l->illumination == DL_ILLUMINATION_SINGLE_BOUNCE && !o.skip_bounce && l->shape != DL_SHAPE_SKY;
    }
    bool alpha_tested() const { return l->transparency != DL_TRANSPARENCY_DISABLED; }
    // light_shape.rs:33-43
    uint32_t shadow_bits() const {
        switch (l->shape) {
            case DL_SHAPE_POINT: return 1;
            case DL_SHAPE_RECTANGLE:
            case DL_SHAPE_TUBE: return AREA_SHADOW_BITS;
            case DL_SHAPE_SUN: return l->size[0] > 0.0f ? AREA_SHADOW_BITS : 1;
            default: return SKY_SHADOW_BITS;
        }
    }
    // AreaLightShape::half_extents / at (src/light/area.rs:42-57)
    V2 half() const { return V2{l->size[0] * 0.5f, l->size[1] * 0.5f}; }
    AreaShape area_shape() const {
        return AreaShape{position(), quat_rotate(l->rotation, V3{1, 0, 0}), quat_rotate(l->rotation, V3{0, 1, 0}),
                         quat_rotate(l->rotation, V3{0, 0, -1}), half(), l->shape == DL_SHAPE_RECTANGLE};
    }
    // light_shape.rs:22-28
    float shape_reach() const {
        if (!is_area()) return l->radius;
        V2 h = half();
        return l->radius - std::sqrt(h.x * h.x + h.y * h.y);
    }
    // SunDisk::toward / angular_radius (src/light/shape.rs:95-102)
    V3 sun_toward() const { return normalize(quat_rotate(l->rotation, V3{0, 0, 1})); }
    float sun_angular_radius() const { return (l->size[0] * 0.5f) * (PI_F / 180.0f); }
    // may_face (light_shape.rs:47-65)
    bool may_face(const V3 v[3], V3 normal) const {
        V3 center = (v[0] + v[1] + v[2]) / 3.0f;
        auto faces = [&](V3 p) { return dot(normal, normalize_or_zero(p - center)) > NDOTL_TOLERANCE; };
        if (l->shape == DL_SHAPE_SKY) return true;
        if (l->shape == DL_SHAPE_SUN) return dot(normal, sun_toward()) + sin_f(sun_angular_radius()) > NDOTL_TOLERANCE;
        if (!is_area()) return faces(position());
        AreaShape s = area_shape();
        bool lit_side = !s.rectangle;
        for (int k = 0; k < 3 && !lit_side; ++k) lit_side = dot(s.forward, v[k] - s.center) > 0.0f;
        if (!lit_side) return false;
        V3 c[4];
        s.corners(c);
        for (int k = 0; k < 4; ++k)
            if (faces(c[k])) return true;
        return false;
    }
};

// ---- low-discrepancy points (src/bake/spread.rs) -----------------------------------------------
inline uint32_t reverse_bits(uint32_t v) {
    v = ((v >> 1) & 0x55555555u) | ((v & 0x55555555u) << 1);
    v = ((v >> 2) & 0x33333333u) | ((v & 0x33333333u) << 2);
    v = ((v >> 4) & 0x0F0F0F0Fu) | ((v & 0x0F0F0F0Fu) << 4);
    v = ((v >> 8) & 0x00FF00FFu) | ((v & 0x00FF00FFu) << 8);
    return (v >> 16) | (v << 16);
}
// spread.rs:43-53
inline uint32_t sobol_second(uint32_t index) {
    uint32_t value = 0, direction = 1u << 31;
    while (index != 0) {
        if (index & 1u) value ^= direction;
        index >>= 1;
        direction ^= direction >> 1;
    }
    return value;
}
// spread.rs:56-58
inline float unit(uint32_t bits) { return (float)(bits >> 8) / 16777216.0f; }
inline float fract_f(float x) { return x - std::floor(x); }
// spread.rs:16-24
inline V2 spread(uint32_t index, V2 offset, bool rectangle) {
    float across = unit(reverse_bits(index));
    float down = rectangle ? unit(sobol_second(index)) : 0.0f;
    return V2{fract_f(across + offset.x), fract_f(down + offset.y)};
}
// spread.rs:28-39 (Shirley–Chiu concentric map)
inline V2 concentric_disk(V2 square) {
    V2 p{square.x * 2.0f - 1.0f, square.y * 2.0f - 1.0f};
    if (p.x == 0.0f && p.y == 0.0f) return V2{0.0f, 0.0f};
    float radius, angle;
    if (std::fabs(p.x) > std::fabs(p.y)) {
        radius = p.x;
        angle = FRAC_PI_4_F * (p.y / p.x);
    } else {
        radius = p.y;
        angle = 2.0f * FRAC_PI_4_F - FRAC_PI_4_F * (p.x / p.y);
    }
    float s, c;
    sincos_f(angle, s, c);
    return V2{c * radius, s * radius};
}
// sky.rs:20-25 (Malley's method)
inline V3 cosine_direction(V3 normal, V2 square) {
    V2 disk = concentric_disk(square);
    float up = std::sqrt(fmax_r(1.0f - (disk.x * disk.x + disk.y * disk.y), 0.0f));
    V3 side, across;
    any_orthonormal_pair(normal, side, across);
    return normalize(side * disk.x + across * disk.y + normal * up);
}

// ---- visibility (src/bake/area.rs, sun.rs, sky.rs, texel_shadow.rs) -------------------------------
struct Visibility {
    bool some;
    double fraction;  // binary32 values except in the F64 mode
    uint32_t rays;
};
struct Sampling {
    uint32_t samples, minimum;
};

// adaptive_share (area.rs:98-126). `trace(point, weight, unblocked)` returns false for a point
// that sends no light.
template <class P, class SpreadPoint, class Trace>
inline bool adaptive_share(const P *probes, int probe_count, Sampling s, SpreadPoint spread_point, Trace trace,
                           double &fraction) {
    bool any_lit = false, any_blocked = false;
    for (int i = 0; i < probe_count; ++i) {
        float w;
        bool lit;
        if (trace(probes[i], w, lit)) {
            any_lit |= lit;
            any_blocked |= !lit;
        }
    }
    Acc lit_sum, total;
    for (uint32_t taken = 0; taken < s.samples; ++taken) {
        if (taken == s.minimum && any_lit != any_blocked) break;
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
        fraction = any_lit ? 1.0 : 0.0;
        return true;
    }
    if (total.value() > 0.0) {
        fraction = active_mode() == PREC_F64 ? lit_sum.d / total.d : (double)(lit_sum.s / total.s);
        return true;
    }
    return false;
}

static const V2 RECTANGLE_PROBES[5] = {{0.0f, 0.0f}, {1.0f, 0.0f}, {1.0f, 1.0f}, {0.0f, 1.0f}, {0.5f, 0.5f}};
static const V2 TUBE_PROBES[3] = {{0.0f, 0.5f}, {1.0f, 0.5f}, {0.5f, 0.5f}};
static const V2 DISK_PROBES[5] = {{0.0f, 0.0f}, {1.0f, 0.0f}, {0.0f, 1.0f}, {-1.0f, 0.0f}, {0.0f, -1.0f}};

// toward (area.rs:130-146)
inline bool area_toward(const AreaShape &s, V3 pos, V3 normal, V2 uv, V3 &dir, float &dist, float &weight) {
    V3 to = s.point_at(uv) - pos;
    float dsq = length_squared(to);
    if (dsq < 1.0e-12f) return false;
    dist = std::sqrt(dsq);
    dir = to / dist;
    float receiver = dot(normal, dir) - NDOTL_TOLERANCE;
    float emitter = s.rectangle ? -dot(s.forward, dir) : 1.0f;
    if (receiver > 0.0f && emitter > 0.0f) {
        weight = receiver * emitter / dsq;
        return true;
    }
    return false;
}

// texel_visibility (area.rs:61-90). `occluded(dir, distance)`.
template <class Occ>
inline Visibility area_visibility(const AreaShape &s, float reach, V3 pos, V3 normal, Sampling sampling, Rng &rng,
                                  Occ occluded) {
    if (reach <= 0.0f || distance_squared(pos, s.nearest_point(pos)) > reach * reach) return {false, 0, 0};
    if (s.rectangle && dot(s.forward, pos - s.center) <= 0.0f) return {false, 0, 0};
    uint32_t rays = 0;
    auto trace = [&](V2 uv, float &w, bool &unblocked) {
        V3 dir;
        float dist;
        if (!area_toward(s, pos, normal, uv, dir, dist, w)) return false;
        rays += 1;
        unblocked = !occluded(dir, fmax_r(dist - END_GAP, 0.0f));
        return true;
    };
    V2 offset;
    offset.x = rng.next_f32();
    offset.y = rng.next_f32();
    auto spread_point = [&](uint32_t taken) { return spread(taken, offset, s.rectangle); };
    double fraction;
    bool some = s.rectangle ? adaptive_share(RECTANGLE_PROBES, 5, sampling, spread_point, trace, fraction)
                            : adaptive_share(TUBE_PROBES, 3, sampling, spread_point, trace, fraction);
    return {some, some ? fraction : 0.0, rays};
}

// sun_visibility (sun.rs:21-56). `occluded(dir)` traces to infinity.
template <class Occ>
inline Visibility sun_visibility(V3 toward, float radius, float tan_radius, V3 normal, Sampling sampling, Rng &rng,
                                 Occ occluded) {
    if (radius <= 0.0f) {
        if (dot(normal, toward) <= NDOTL_TOLERANCE) return {false, 0, 0};
        bool lit = !occluded(toward);
        return {true, lit ? 1.0f : 0.0f, 1};
    }
    V3 side, up;
    any_orthonormal_pair(toward, side, up);
    uint32_t rays = 0;
    auto trace = [&](V2 disk, float &w, bool &unblocked) {
        V3 dir = normalize(toward + (side * disk.x + up * disk.y) * tan_radius);
        float receiver = dot(normal, dir) - NDOTL_TOLERANCE;
        if (receiver <= 0.0f) return false;
        rays += 1;
        w = receiver;
        unblocked = !occluded(dir);
        return true;
    };
    V2 offset;
    offset.x = rng.next_f32();
    offset.y = rng.next_f32();
    auto spread_point = [&](uint32_t taken) { return concentric_disk(spread(taken, offset, true)); };
    double fraction;
    bool some = adaptive_share(DISK_PROBES, 5, sampling, spread_point, trace, fraction);
    return {some, some ? fraction : 0.0, rays};
}

// sky_visibility (sky.rs:30-44)
template <class Occ>
inline Visibility sky_visibility(V3 normal, uint32_t samples, Rng &rng, Occ occluded) {
    V2 offset;
    offset.x = rng.next_f32();
    offset.y = rng.next_f32();
    uint32_t open = 0;
    for (uint32_t taken = 0; taken < samples; ++taken)
        if (!occluded(cosine_direction(normal, spread(taken, offset, true)))) ++open;
    double fraction = active_mode() == PREC_F64 ? (double)open / (double)std::max(samples, 1u)
                                                   : (double)((float)open / (float)std::max(samples, 1u));
    return {true, fraction, samples};
}

// is_buried (mesh_texels.rs:111-135)
template <class BackFace>
inline bool is_buried(V3 normal, float turn, BackFace back_face) {
    V3 tangent, bitangent;
    any_orthonormal_pair(normal, tangent, bitangent);
    uint32_t back = 0, front = 0;
    for (uint32_t i = 0; i < 8; ++i) {
        float ring = (float)((i * 5) % 8) + 0.5f;
        float sin_theta = std::sqrt(ring / 8.0f);
        float cos_theta = std::sqrt(1.0f - sin_theta * sin_theta);
        float phi = ((float)i + turn) * TAU_F / 8.0f;
        float sp, cp;
        sincos_f(phi, sp, cp);
        V3 dir = (tangent * cp + bitangent * sp) * sin_theta + normal * cos_theta;
        if (back_face(dir))
            ++back;
        else
            ++front;
        if (back >= 5) return true;
        if (front > 8 - 5) return false;
    }
    return false;
}

}  // namespace oracle
