// TEST INFRASTRUCTURE — the parity oracle, not the product.
//
// One-bounce lighting of the reference baker: photon cubes (src/bake/bounce.rs:47-115), the
// cube conventions (src/shared/cube.rs:29-105), the local-light and sun gathers
// (bounce.rs:235-292, src/bake/sun_bounce.rs:24-80), the bounce map filters
// (src/bake/bounce_map.rs:22-151) and bounce packing (src/bake/bounce_pack.rs:18-86).
#pragma once

#include "oracle_light.hpp"

namespace oracle {

// ---- cube conventions (cube.rs) ----------------------------------------------------------------
// cube.rs:29-53
inline void direction_to_face_uv(V3 d, uint32_t &face, V2 &uv) {
    V3 a = vabs(d);
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
    if (ma == 0.0f) {
        uv = V2{0.5f, 0.5f};
        return;
    }
    uv = V2{(sc / ma) * 0.5f + 0.5f, (tc / ma) * 0.5f + 0.5f};
}
// cube.rs:57-70
inline V3 face_uv_to_direction(uint32_t face, V2 uv) {
    float sc = uv.x * 2.0f - 1.0f, tc = uv.y * 2.0f - 1.0f;
    V3 d;
    switch (face) {
        case 0: d = V3{1.0f, -tc, -sc}; break;
        case 1: d = V3{-1.0f, -tc, sc}; break;
        case 2: d = V3{sc, 1.0f, tc}; break;
        case 3: d = V3{sc, -1.0f, -tc}; break;
        case 4: d = V3{sc, -tc, 1.0f}; break;
        default: d = V3{-sc, -tc, -1.0f}; break;
    }
    return normalize(d);
}
// cube.rs:73-79
inline V3 texel_direction(uint32_t face, uint32_t x, uint32_t y, uint32_t res) {
    float size = (float)res;
    return face_uv_to_direction(face, V2{((float)x + 0.5f) / size, ((float)y + 0.5f) / size});
}
// cube.rs:94-105
inline void direction_to_texel(V3 d, uint32_t res, uint32_t &face, uint32_t &x, uint32_t &y) {
    V2 uv;
    direction_to_face_uv(d, face, uv);
    float max = (float)(res == 0 ? 0 : res - 1);
    x = f2u_sat(clampf(std::floor(uv.x * (float)res), 0.0f, max));
    y = f2u_sat(clampf(std::floor(uv.y * (float)res), 0.0f, max));
}

// ---- photon cubes (bounce.rs:29-115) -----------------------------------------------------------
struct Photon {
    float distance;
    int8_t normal[3];
    uint8_t albedo[3];
};
struct PhotonCube {
    uint32_t resolution = 0;
    std::vector<Photon> photons;
    // sample (bounce.rs:73-85)
    void sample(V3 light, V3 dir, V3 &pos, V3 &normal, V3 &albedo) const {
        uint32_t face, x, y;
        direction_to_texel(dir, resolution, face, x, y);
        size_t index = (size_t)face * resolution * resolution + (size_t)y * resolution + x;
        if (index >= photons.size()) {
            pos = light;
            normal = V3{0, 0, 0};
            albedo = V3{0, 0, 0};
            return;
        }
        const Photon &p = photons[index];
        V3 n{(float)p.normal[0] / 127.0f, (float)p.normal[1] / 127.0f, (float)p.normal[2] / 127.0f};
        pos = light + dir * p.distance;
        normal = normalize_or_zero(n);
        albedo = V3{(float)p.albedo[0] / 255.0f, (float)p.albedo[1] / 255.0f, (float)p.albedo[2] / 255.0f};
    }
};
// photon (bounce.rs:88-115)
inline Photon make_photon(const Light &light, const Occluders &occ, V3 dir) {
    BounceScope bounce_stage;
    SurfaceHit hit;
    if (!occ.closest_hit(light.position(), dir, light.l->radius, light.alpha_tested(), hit))
        return Photon{light.l->radius, {0, 0, 0}, {0, 0, 0}};
    V3 normal = occ.surface_normal(hit);
    V3 point = light.position() + dir * hit.distance;
    float bias = fmax_r(hit.distance * 0.001f, 0.001f);
    V3 nudged = point - dir * bias + normal * bias;
    bool lit_side = dot(occ.face_normal(hit), dir) < 0.0f;
    Photon p;
    p.distance = length(nudged - light.position());
    if (lit_side) {
        p.normal[0] = f2i8_sat(std::round(normal.x * 127.0f));
        p.normal[1] = f2i8_sat(std::round(normal.y * 127.0f));
        p.normal[2] = f2i8_sat(std::round(normal.z * 127.0f));
    } else {
        p.normal[0] = p.normal[1] = p.normal[2] = 0;
    }
    V3 a = occ.albedo(hit);
    p.albedo[0] = f2u8_sat(std::round(clampf(a.x, 0.0f, 1.0f) * 255.0f));
    p.albedo[1] = f2u8_sat(std::round(clampf(a.y, 0.0f, 1.0f) * 255.0f));
    p.albedo[2] = f2u8_sat(std::round(clampf(a.z, 0.0f, 1.0f) * 255.0f));
    return p;
}
// PhotonCube::build (bounce.rs:48-70)
inline PhotonCube build_photon_cube(const Light &light, const Occluders &occ, uint32_t res) {
    PhotonCube cube;
    cube.resolution = res;
    cube.photons.resize((size_t)6 * res * res);
    parallel_for((size_t)6 * res, [&](size_t row) {
        uint32_t face = (uint32_t)(row / res), y = (uint32_t)(row % res);
        for (uint32_t x = 0; x < res; ++x)
            cube.photons[(size_t)face * res * res + (size_t)y * res + x] =
                make_photon(light, occ, texel_direction(face, x, y, res));
    });
    return cube;
}

// ---- slerp (glam 0.33 Vec3::slerp, the reference's bounce.rs:270) ------------------------------
// glam is not vendored with the reference; its published slerp is restated here:
//  - the angle comes from glam's acos_approx, not from libm: the 7-degree polynomial of
//    Abramowitz & Stegun 4.4.46 (Hastings), acos|x| = sqrt(1 - |x|) * p(|x|), evaluated in f32
//    by Horner's rule with no fused operations, and pi - that for negative x (the form of
//    DirectXMath's XMScalarACos, which glam follows; the f32 coefficients are the same values);
//  - the sine-weighted blend is taken when |cos| < 1 - 3 * f32::EPSILON, with the result's
//    length interpolated linearly between the two lengths;
//  - nearly opposite vectors turn `a` about a unit vector orthogonal to it by pi * s
//    (Quat::from_axis_angle, then glam's Quat * Vec3), scaled to the interpolated length;
//  - nearly equal vectors (or a NaN cosine) take the plain lerp a * (1 - s) + b * s.
inline float acos_approx(float v) {
    const bool nonnegative = v >= 0.0f;
    const float x = std::fabs(v);
    float omx = 1.0f - x;
    if (omx < 0.0f) omx = 0.0f;
    const float root = std::sqrt(omx);
    float r = -0.0012624911f;
    r = r * x + 0.0066700901f;
    r = r * x - 0.0170881256f;
    r = r * x + 0.0308918810f;
    r = r * x - 0.0501743046f;
    r = r * x + 0.0889789874f;
    r = r * x - 0.2145988016f;
    r = r * x + 1.5707963050f;
    r = r * root;
    return nonnegative ? r : PI_F - r;
}
inline V3 any_orthogonal_vector(V3 v) {
    return std::fabs(v.x) > std::fabs(v.y) ? V3{-v.z, 0.0f, v.x} : V3{0.0f, v.z, -v.y};
}
constexpr float F32_EPSILON = 1.1920928955078125e-7f;  // f32::EPSILON, 2^-23
inline V3 slerp(V3 a, V3 b, float s) {
    const float la = length(a), lb = length(b);
    const float d = dot(a, b) / (la * lb);
    // the interpolated length as a factor of a's: lerp(|a|, |b|, s) / |a|
    if (std::fabs(d) < 1.0f - 3.0f * F32_EPSILON) {
        const float angle = acos_approx(d);
        const float angle_sin = sin_f(angle);
        const float t1 = sin_f(angle * (1.0f - s)) / angle_sin;
        const float t2 = sin_f(angle * s) / angle_sin * (la / lb);
        return (a * t1 + b * t2) * (1.0f + s * (lb / la - 1.0f));
    }
    if (d < 0.0f) {
        const V3 axis = normalize(any_orthogonal_vector(a));
        float sh, ch;
        sincos_f(PI_F * s * 0.5f, sh, ch);
        const V3 v = axis * sh;
        const float q[4] = {v.x, v.y, v.z, ch};
        return quat_rotate(q, a) * (1.0f + s * (lb / la - 1.0f));
    }
    return a * (1.0f - s) + b * s;
}

// ---- bounce map (bounce_map.rs) -----------------------------------------------------------------
constexpr uint32_t WINDOW_MARGIN = 4;  // bounce_map.rs:18
// gaussian_weights (bounce_map.rs:140-151)
inline void gaussian_weights(float out[7]) {
    const float sigma = 5.0f, sigma2 = sigma * sigma;
    float sum = 0.0f;
    for (int i = -3; i <= 3; ++i) {
        float w = (1.0f / std::sqrt(2.0f * PI_F * sigma2)) * exp_f(-(float)(i * i) / (2.0f * sigma2));
        out[i + 3] = w;
        sum += w;
    }
    for (int k = 0; k < 7; ++k) out[k] = out[k] / sum;
}
struct BounceMap {
    uint32_t size;
    Rect rect;
    std::vector<V3> values;
    BounceMap(uint32_t s, Rect crops) : size(s) {
        uint32_t last = s - 1;
        rect = Rect{crops.min_x >= WINDOW_MARGIN ? crops.min_x - WINDOW_MARGIN : 0,
                    crops.min_y >= WINDOW_MARGIN ? crops.min_y - WINDOW_MARGIN : 0,
                    std::min(crops.max_x + WINDOW_MARGIN, last), std::min(crops.max_y + WINDOW_MARGIN, last)};
        values.assign((size_t)rect.width() * rect.height(), V3{0, 0, 0});
    }
    size_t index(uint32_t x, uint32_t y) const {
        return (size_t)(y - rect.min_y) * rect.width() + (x - rect.min_x);
    }
    V3 get(int64_t x, int64_t y) const {
        return rect.contains(x, y) ? values[index((uint32_t)x, (uint32_t)y)] : V3{0, 0, 0};
    }
    void set(uint32_t x, uint32_t y, V3 v) { values[index(x, y)] = v; }
    template <class F>
    std::vector<V3> map_window(F f) const {
        std::vector<V3> out;
        out.reserve(values.size());
        for (uint32_t y = rect.min_y; y <= rect.max_y; ++y)
            for (uint32_t x = rect.min_x; x <= rect.max_x; ++x) out.push_back(f((int64_t)x, (int64_t)y));
        return out;
    }
    // bounce_map.rs:67-87
    void dilate() {
        static const int O[9][2] = {{0, 0}, {-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
        values = map_window([&](int64_t x, int64_t y) {
            for (auto &o : O) {
                V3 v = get(x + o[0], y + o[1]);
                if (max_element(v) > 0.0f) return v;
            }
            return V3{0, 0, 0};
        });
    }
    // bounce_map.rs:92-112
    void blur() {
        float w[7];
        gaussian_weights(w);
        float wsum = 0.0f;
        for (float x : w) wsum += x;
        int64_t last = (int64_t)size - 1;
        for (int vertical = 0; vertical < 2; ++vertical) {
            values = map_window([&](int64_t x, int64_t y) {
                V3 sum{0, 0, 0};
                for (int k = -3; k <= 3; ++k) {
                    V3 s = vertical ? get(x, std::min(std::max(y + k, (int64_t)0), last))
                                    : get(std::min(std::max(x + k, (int64_t)0), last), y);
                    sum = sum + s * w[k + 3];
                }
                return sum / wsum;
            });
        }
    }
    // bounce_map.rs:124-136
    bool crop(Rect c, std::vector<V3> &grid) const {
        uint32_t width = c.width() + 4;
        grid.assign((size_t)width * (c.height() + 4), V3{0, 0, 0});
        bool lit = false;
        for (uint32_t y = c.min_y; y <= c.max_y; ++y)
            for (uint32_t x = c.min_x; x <= c.max_x; ++x) {
                V3 v = get(x, y);
                lit |= max_element(v) > 0.0f;
                grid[(size_t)(y - c.min_y + 2) * width + (x - c.min_x + 2)] = v;
            }
        return lit;
    }
};

// ---- bounce packing (bounce_pack.rs) --------------------------------------------------------
inline float dither_amplitude(uint32_t bits) {
    switch (bits) {
        case 8: return 0.0f;
        case 6: return 0.004f;
        case 5: return 0.008f;
        default: return 0.02f;
    }
}
// quantize (bounce_pack.rs:74-86)
inline uint32_t quantize(float value, uint32_t bits, Rng &rng) {
    float max = (float)((1u << bits) - 1);
    float amplitude = dither_amplitude(bits);
    float color = std::isnan(value) ? 0.0f : clampf(value, 0.0f, 1.0f);
    if (amplitude > 0.0f && color > 0.001f) color = fmin_r(color + rng.next_f32() * amplitude, 1.0f);
    return f2u_sat(std::sqrt(color) * max);
}
// pack_bounce (bounce_pack.rs:28-43)
inline std::vector<uint32_t> pack_bounce(const std::vector<float> &values, uint32_t bits, Rng &rng) {
    size_t per = 32 / bits;
    std::vector<uint32_t> out((values.size() + per - 1) / per, 0);
    for (size_t i = 0; i < values.size(); ++i) out[i / per] |= quantize(values[i], bits, rng) << ((i % per) * bits);
    return out;
}
// pack_bounce_rgb (bounce_pack.rs:47-71)
inline std::vector<uint32_t> pack_bounce_rgb(const std::vector<V3> &values, uint32_t bits, Rng &rng) {
    uint32_t pixel_bits = 3 * bits;
    std::vector<uint32_t> words((values.size() * pixel_bits + 31) / 32, 0);
    for (size_t i = 0; i < values.size(); ++i) {
        uint32_t pixel = 0;
        const float ch[3] = {values[i].x, values[i].y, values[i].z};
        for (uint32_t c = 0; c < 3; ++c) pixel |= quantize(ch[c], bits, rng) << (c * bits);
        size_t offset = i * pixel_bits;
        size_t word = offset / 32;
        uint32_t shift = (uint32_t)(offset % 32);
        words[word] |= pixel << shift;
        if (shift + pixel_bits > 32) words[word + 1] |= pixel >> (32 - shift);
    }
    return words;
}

}  // namespace oracle
