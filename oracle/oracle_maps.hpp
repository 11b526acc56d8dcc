// TEST INFRASTRUCTURE — the parity oracle, not the product.
//
// The bake's maps for moving meshes: distance cubes (src/bake/distance_cubes.rs), sun maps
// (src/bake/sun_map.rs) and sky probes (src/bake/sky_probes.rs), restated in binary32 in the
// reference's operation order. Baked only when dynamic_geometry is not LightingOnly
// (src/bake/baker.rs:114-152).
#pragma once

#include <array>
#include <cstring>

#include "oracle_bounce.hpp"

namespace oracle {

// f32 -> f16 bits, round to nearest even (the `half` crate's f16::from_f32, IEEE 754).
inline uint16_t f16_bits(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u, a = x & 0x7FFFFFFFu;
    if (a > 0x7F800000u) return (uint16_t)(sign | 0x7E00u | ((a >> 13) & 0x3FFu));  // NaN
    if (a >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // 65520 and up round to infinity
    int e = (int)(a >> 23) - 127;
    uint32_t mant = (a & 0x7FFFFFu) | 0x800000u;
    if (e >= -14) {  // normal half
        uint32_t h = ((uint32_t)(e + 15) << 10) | ((a >> 13) & 0x3FFu);
        uint32_t rest = a & 0x1FFFu;
        if (rest > 0x1000u || (rest == 0x1000u && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    if (a == 0) return (uint16_t)sign;
    int shift = -e - 1;  // value / 2^-24 = mant * 2^(e + 1)
    if (shift > 24) return (uint16_t)sign;
    uint32_t q = mant >> shift, rest = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rest > half || (rest == half && (q & 1u))) ++q;
    return (uint16_t)(sign | q);
}
// pack_f16_pair (distance_cubes.rs:23-26)
inline uint32_t pack_f16_pair(float lower, float upper) {
    return (uint32_t)f16_bits(upper) << 16 | (uint32_t)f16_bits(lower);
}

// ---- distance cubes (distance_cubes.rs:29-75) ------------------------------------------------
constexpr uint32_t DISTANCE_CUBE_RESOLUTION = 64;

inline std::vector<uint32_t> bake_distance_cubes(const std::vector<Light> &lights, size_t local,
                                                 const Occluders &occ) {
    const uint32_t res = DISTANCE_CUBE_RESOLUTION, words = res * res / 2;
    std::vector<uint32_t> out((size_t)local * 6 * words);
    parallel_for(local * 6, [&](size_t job) {
        const Light &l = lights[job / 6];
        uint32_t face = (uint32_t)(job % 6);
        V3 p{l.l->position[0], l.l->position[1], l.l->position[2]};
        auto distance = [&](uint32_t texel) {
            SurfaceHit hit;
            if (occ.closest_hit(p, texel_direction(face, texel % res, texel / res, res), l.l->radius,
                                l.alpha_tested(), hit))
                return hit.distance;
            return l.l->radius;
        };
        for (uint32_t w = 0; w < words; ++w) out[job * words + w] = pack_f16_pair(distance(2 * w), distance(2 * w + 1));
    });
    return out;
}

// ---- sun maps (sun_map.rs) -------------------------------------------------------------------
struct SunMapOut {
    float rows[12];
    uint32_t resolution;
    std::vector<uint32_t> texels;
};
// pack_sun_depth (sun_map.rs:77-81)
inline uint32_t unorm16(float d) { return f2u_sat(std::round(clampf(d, 0.0f, 1.0f) * 65535.0f)); }
inline uint32_t pack_sun_depth(float lower, float upper) { return unorm16(upper) << 16 | unorm16(lower); }

// bake_sun_map (sun_map.rs:25-74) with SunFrame (:83-161)
inline SunMapOut bake_sun_map(V3 toward, const Occluders &occ, uint32_t resolution, bool alpha) {
    V3 side, up;
    any_orthonormal_pair(toward, side, up);
    V3 along = -toward;
    auto local = [&](V3 w) { return V3{dot(w, side), dot(w, up), dot(w, along)}; };
    V3 mn{INFINITY, INFINITY, INFINITY}, mx{-INFINITY, -INFINITY, -INFINITY};
    for (const auto &t : occ.triangles)
        for (int k = 0; k < 3; ++k) {
            V3 v = local(t.v[k]);
            mn = vmin(mn, v);
            mx = vmax(mx, v);
        }
    SunMapOut out{};
    if (!(v3_finite(mn) && v3_finite(mx))) {
        out.resolution = 1;
        out.texels = {pack_sun_depth(1.0f, 1.0f)};
        return out;
    }
    V3 size = mx - mn;
    float margin = size.z * 0.01f + 0.05f;
    float extent = fmax_r(size.x, size.y) + 2.0f * margin;
    V3 center = (mn + mx) * 0.5f;
    V3 bmin{center.x - extent * 0.5f, center.y - extent * 0.5f, mn.z - margin};
    float depth = size.z + 2.0f * margin;
    auto row = [&](float *r, V3 axis, float lo, float length) {
        V3 a = axis / length;
        r[0] = a.x;
        r[1] = a.y;
        r[2] = a.z;
        r[3] = -lo / length;
    };
    row(out.rows, side, bmin.x, extent);
    row(out.rows + 4, up, bmin.y, extent);
    row(out.rows + 8, along, bmin.z, depth);
    out.resolution = resolution;
    float texel = extent / (float)resolution;
    std::vector<float> depths((size_t)resolution * resolution);
    parallel_for(resolution, [&](size_t y) {
        for (uint32_t x = 0; x < resolution; ++x) {
            float across = bmin.x + ((float)x + 0.5f) * texel;
            float down = bmin.y + ((float)y + 0.5f) * texel;
            V3 origin = side * across + up * down + along * bmin.z;
            SurfaceHit hit;
            depths[y * resolution + x] = occ.closest_hit(origin, along, depth, alpha, hit) ? hit.distance / depth : 1.0f;
        }
    });
    out.texels.resize((depths.size() + 1) / 2);
    for (size_t w = 0; w < out.texels.size(); ++w)
        out.texels[w] = pack_sun_depth(depths[2 * w], 2 * w + 1 < depths.size() ? depths[2 * w + 1] : 1.0f);
    return out;
}

// ---- sky probes (sky_probes.rs) --------------------------------------------------------------
constexpr uint64_t MAX_SKY_PROBES = 65536;
constexpr uint64_t PROBE_STREAM = 0x736b7970726f6265ull;
constexpr float INSIDE_SHARE = 0.25f;
static const V3 PROBE_AXES[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};

// f32::cbrt: binary64 cube root rounded once
inline float cbrt_f(float x) { return (float)std::cbrt((double)x); }

struct ProbeGrid {
    V3 origin;
    float spacing;
    uint32_t counts[3];
    uint64_t count() const { return (uint64_t)counts[0] * counts[1] * counts[2]; }
    // ProbeGrid::over (sky_probes.rs:45-61)
    static ProbeGrid over(V3 mn, V3 mx, float spacing) {
        V3 extent = vmax(mx - mn, V3{0, 0, 0}) + V3{spacing, spacing, spacing};
        ProbeGrid g{};
        auto counts_at = [&](float s) {
            g.counts[0] = f2u_sat(std::ceil(extent.x / s)) + 1;
            g.counts[1] = f2u_sat(std::ceil(extent.y / s)) + 1;
            g.counts[2] = f2u_sat(std::ceil(extent.z / s)) + 1;
        };
        counts_at(spacing);
        while (g.count() > MAX_SKY_PROBES) {
            float ratio = (float)g.count() / (float)MAX_SKY_PROBES;
            spacing = spacing * fmax_r(cbrt_f(ratio), 1.01f);
            counts_at(spacing);
        }
        V3 span{(float)(g.counts[0] - 1) * spacing, (float)(g.counts[1] - 1) * spacing,
                (float)(g.counts[2] - 1) * spacing};
        g.origin = (mn + mx) * 0.5f - span * 0.5f;
        g.spacing = spacing;
        return g;
    }
    void probe(uint64_t index, uint32_t p[3]) const {
        uint64_t x = counts[0], xy = x * counts[1];
        p[0] = (uint32_t)(index % x);
        p[1] = (uint32_t)(index % xy / x);
        p[2] = (uint32_t)(index / xy);
    }
    V3 position(const uint32_t p[3]) const {
        return origin + V3{(float)p[0] * spacing, (float)p[1] * spacing, (float)p[2] * spacing};
    }
};

struct SkyProbesOut {
    bool present = false;
    V3 origin{0, 0, 0};
    float spacing = 0.0f;
    uint32_t counts[3] = {0, 0, 0};
    std::vector<uint32_t> words;
};

// trace_probe (sky_probes.rs:83-109): the six openness values, false when inside geometry
inline bool trace_probe(const Occluders &occ, V3 position, uint32_t samples, bool alpha, const uint64_t key[4],
                        float open[6]) {
    uint32_t back = 0;
    for (uint32_t axis = 0; axis < 6; ++axis) {
        uint64_t parts[6] = {key[0], PROBE_STREAM, key[1], key[2], key[3], axis};
        Rng rng = stream(parts, 6);
        Visibility v = sky_visibility(PROBE_AXES[axis], samples, rng, [&](V3 dir) {
            SurfaceHit hit;
            bool found = occ.closest_hit(position, dir, INFINITY, alpha, hit) && hit.distance > 0.0f;
            if (found && dot(occ.face_normal(hit), dir) > 0.0f) ++back;
            return found;
        });
        open[axis] = (float)v.fraction;
    }
    float rays = (float)(std::max(samples, 1u) * 6u);
    return (float)back <= INSIDE_SHARE * rays;
}

// fill_inside (sky_probes.rs:114-146)
inline void fill_inside(const ProbeGrid &g, std::vector<std::array<float, 6>> &values, std::vector<uint8_t> &valid) {
    const int cx = (int)g.counts[0], cy = (int)g.counts[1], cz = (int)g.counts[2];
    static const int STEP[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (;;) {
        auto prev_values = values;
        auto prev_valid = valid;
        bool changed = false;
        for (uint64_t index = 0; index < values.size(); ++index) {
            if (prev_valid[index]) continue;
            uint32_t p[3];
            g.probe(index, p);
            float sum[6] = {0, 0, 0, 0, 0, 0};
            float found = 0.0f;
            for (const auto &st : STEP) {
                int nx = (int)p[0] + st[0], ny = (int)p[1] + st[1], nz = (int)p[2] + st[2];
                if (nx < 0 || ny < 0 || nz < 0 || nx >= cx || ny >= cy || nz >= cz) continue;
                uint64_t n = ((uint64_t)nz * cy + ny) * cx + nx;
                if (!prev_valid[n]) continue;
                for (int k = 0; k < 6; ++k) sum[k] = sum[k] + prev_values[n][k];
                found = found + 1.0f;
            }
            if (found > 0.0f) {
                for (int k = 0; k < 6; ++k) values[index][k] = sum[k] / found;
                valid[index] = 1;
                changed = true;
            }
        }
        if (!changed) break;
    }
}

// SkyProbes::pack (format/types.rs:105-112)
inline void pack_probe(const float open[6], uint32_t words[2]) {
    words[0] = words[1] = 0;
    for (int axis = 0; axis < 6; ++axis) {
        uint32_t byte = f2u_sat(std::round(clampf(open[axis], 0.0f, 1.0f) * 255.0f));
        words[axis / 4] |= byte << (8 * (axis % 4));
    }
}

// bake_sky_probes (sky_probes.rs:146-190)
inline SkyProbesOut bake_sky_probes(const Occluders &occ, float spacing, uint32_t samples, bool alpha, uint64_t seed) {
    SkyProbesOut out;
    if (occ.triangles.empty()) return out;
    V3 mn = occ.triangles[0].v[0], mx = mn;
    for (const auto &t : occ.triangles)
        for (int k = 0; k < 3; ++k) {
            mn = vmin(mn, t.v[k]);
            mx = vmax(mx, t.v[k]);
        }
    ProbeGrid g = ProbeGrid::over(mn, mx, spacing);
    uint64_t n = g.count();
    std::vector<std::array<float, 6>> values(n);
    std::vector<uint8_t> valid(n, 0);
    parallel_for(n, [&](size_t index) {
        uint32_t p[3];
        g.probe(index, p);
        uint64_t key[4] = {seed, p[0], p[1], p[2]};
        float open[6];
        if (trace_probe(occ, g.position(p), samples, alpha, key, open)) {
            for (int k = 0; k < 6; ++k) values[index][k] = open[k];
            valid[index] = 1;
        }
    });
    fill_inside(g, values, valid);
    out.present = true;
    out.origin = g.origin;
    out.spacing = g.spacing;
    for (int k = 0; k < 3; ++k) out.counts[k] = g.counts[k];
    out.words.resize(n * 2);
    for (uint64_t i = 0; i < n; ++i) {
        float ones[6] = {1, 1, 1, 1, 1, 1};
        pack_probe(valid[i] ? values[i].data() : ones, &out.words[i * 2]);
    }
    return out;
}

}  // namespace oracle
