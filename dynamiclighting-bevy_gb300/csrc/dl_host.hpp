// Host half of the bake: validation and sorting, the light BVH (which fixes the light slot
// order), per-light constants, per-mesh shadow map sizes, the occluder list and its BVH, and the
// .dynlight payload writer. Everything here is small or runs once per bake; the per-texel work is
// in the CUDA kernels.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dynlight.h"
#include "dl_math.cuh"

namespace dl {

// One light in slot order with the constants every kernel needs (src/bake/light_shape.rs,
// src/light/area.rs:42-123, src/light/shape.rs:95-102), read by the kernels as is.
struct DevLight {
    f3 position;
    float radius;
    uint32_t shape;        // dl_light_shape
    uint32_t flags;        // kLight* bits
    uint32_t shadow_bits;  // 1, 4 or 8
    uint32_t bounce_samples;
    f3 ax, ay, forward;    // area frame (rotation * X, Y, -Z)
    float half_x, half_y;
    float reach;           // shape_reach()
    f3 toward;             // sun: unit vector towards the sun
    float angular_radius;  // sun
    float tan_radius;      // sun
    float sin_radius;      // sun
    float bounce_intensity;
    uint32_t bounce_bits;  // 0: no bounce
    uint64_t id;
    f3 bounds_lo, bounds_hi;  // light_bounds (light_bvh.rs:77-81), local lights only
    uint32_t cube;            // photon cube index of a local bounce light, else ~0
    uint32_t pad;
};
enum : uint32_t {
    kLightDistant = 1,
    kLightAlpha = 2,
    kLightBounce = 4,
    kLightRect = 8,
    kLightArea = 16,
};

// Aila–Laine style BVH2 node: both children's boxes in the parent, 64 bytes.
// c0 = (l0.lo.x, l0.hi.x, l0.lo.y, l0.hi.y), c1 = same for child 1,
// c2 = (l0.lo.z, l0.hi.z, l1.lo.z, l1.hi.z), c3 = (ref0, ref1, 0, 0) as int bits.
// ref >= 0: inner node; ref < 0: leaf ~(first << 3 | count) over triangles [first, first + count);
// ~0 is an empty child.
struct BvhNode {
    float c0[4], c1[4], c2[4];
    int32_t ref[2];
    uint32_t count[2];
};

struct HostScene {
    std::vector<const dl_mesh *> meshes;      // sorted by id
    std::vector<const dl_light *> light_ptrs;  // slot order
    std::vector<DevLight> lights;
    uint32_t local_lights = 0;
    std::vector<dl_light_bvh_node> light_bvh;
    bool bounce_in_scene = false;
    std::vector<uint32_t> resolution;  // per mesh
    std::vector<uint32_t> cube_lights;  // slot of each photon cube's light (bounce.rs:126-151)
    float blur_weights[7];              // gaussian_weights(7, 5) (bounce_map.rs:140-151)
    float blur_weight_sum;
    uint64_t triangles = 0;
    // occluders in the reference's order (sorted mesh order, triangle order, non-degenerate)
    std::vector<uint32_t> occ_mesh, occ_tri;
    // BVH over the occluders, triangles in leaf order
    std::vector<BvhNode> nodes;
    std::vector<float> tris;  // 12 floats per triangle: v0 (w: occluder index bits), e1, e2
    uint32_t bvh_depth = 0;
    uint32_t bvh_node_count = 0;  // inner nodes, from either builder (the device one fills no vectors)
};

// Validates, sorts and prepares (src/bake/baker.rs:32-75). Returns DL_OK or the error status
// with `err` set to the reference's message.
dl_status prepare_scene(const dl_bake_input &in, const dl_bake_options &o, HostScene &s, std::string &err);

// Builds the occluder BVH on the host (binned SAH, leaves of at most 4 triangles, depth capped at
// 60; the rules of dl_bvh_rules.hpp). The bake builds the same tree on the device (dl_bvh.cu)
// unless dl_bake_config.host_bvh asks for this one.
void build_bvh(HostScene &s);

// The first n = 2^m points of the sky's low-discrepancy sequence (src/bake/spread.rs:16-24) form
// a (0, m, 2)-net: one point in each cell of a 2^ceil(m/2) x 2^floor(m/2) grid of the unit square.
// Listed in the Morton order of their cells, any 16 consecutive entries lie in one 4 x 4 block
// of cells, so lanes that trace them together send nearby directions from the same texel. The
// open count of a sky texel does not depend on the order its samples are traced in. Empty
// unless n is a power of two from 16 to 65536.
std::vector<uint16_t> sky_sample_order(uint32_t n);
// The same net's cells for a shifted net: `cells[r]` is the cell (x | y << 8) of the r-th entry of
// sky_sample_order(n) and `samples[y << xbits | x]` the one point of cell (x, y), where the grid
// is 2^xbits x 2^ybits, xbits = ceil(m / 2). A texel whose net is shifted by `off`
// (spread.rs:16-24, a toroidal shift) takes rank r from the cell of rank r moved back by the shift's
// whole cells, floor(off * grid): its shifted point then lies in that cell or the next, so every
// texel's r-th ray leaves in about the same direction. Empty unless n is a power of two from 16 to
// 65536.
struct SampleCells {
    std::vector<uint16_t> cells, samples;
};
SampleCells sample_cells(uint32_t n);

// A sun map's frame and bounds (src/bake/sun_map.rs:25-45,83-161): `empty` when there is no
// static geometry (one texel that nothing is behind).
struct SunMapSetup {
    bool empty = true;
    f3 side, up, along, bmin;
    float extent = 0.0f, depth = 0.0f, texel = 0.0f;
    float rows[12] = {};
    uint32_t resolution = 1;
};
SunMapSetup sun_map_setup(const HostScene &s, uint32_t slot, uint32_t resolution);

// The sky probe grid over the static bounds (src/bake/sky_probes.rs:45-80, 146-162).
struct ProbeGridSetup {
    bool present = false;
    f3 origin;
    float spacing = 0.0f;
    uint32_t counts[3] = {0, 0, 0};
    uint64_t count() const { return (uint64_t)counts[0] * counts[1] * counts[2]; }
};
ProbeGridSetup sky_probe_grid(const HostScene &s, float spacing);
// The probes' words from each (probe, axis)'s open fraction and back-face hits: the inside
// test (sky_probes.rs:104-108), fill_inside (:114-146) and SkyProbes::pack (format/types.rs:105).
std::vector<uint32_t> sky_probe_words(const ProbeGridSetup &g, const float *open, const uint32_t *back,
                                      uint32_t samples);

// The .dynlight payload sections in order (src/bake/format/mod.rs:170-213, lights.rs:27-52,
// maps.rs:16-38) into `w`, which takes little-endian u32/u64/f32 values and word arrays
// (`words(pointer, count)` writes the count as a u64, then the words).
template <class Sink>
void emit_payload(const dl_baked_scene &s, Sink &w) {
    w.u32((s.settings.bounce ? 1u : 0u) | (s.settings.colored_bounce ? 2u : 0u));
    w.u32(s.settings.dynamic_geometry);
    w.f32(s.settings.pixel_density);
    w.u32(s.settings.max_lightmap_size);
    w.u32(s.settings.distance_cube_resolution);
    w.u64(s.light_count);
    for (uint64_t i = 0; i < s.light_count; ++i) {
        const dl_baked_light &l = s.lights[i];
        w.u64(l.id);
        for (int k = 0; k < 3; ++k) w.f32(l.origin[k]);
        w.f32(l.radius);
        w.u32(l.bounce_bits);
        w.u32(l.shape);
        for (int k = 0; k < 4; ++k) w.f32(l.rotation[k]);
        for (int k = 0; k < 2; ++k) w.f32(l.size[k]);
        w.u32(l.shadow_bits_per_texel);
    }
    w.words(reinterpret_cast<const uint32_t *>(s.light_bvh), s.light_bvh_count * 8);
    w.u64(s.mesh_count);
    for (uint64_t i = 0; i < s.mesh_count; ++i) {
        const dl_baked_mesh &m = s.meshes[i];
        w.u64(m.id);
        w.u64(m.content_hash);
        w.u32(m.resolution);
        w.u32(m.occludes ? 1u : 0u);
        w.words(m.triangles, m.word_count);
    }
    w.words(s.distance_cubes, s.distance_cube_words);
    // maps::encode (format/maps.rs:16-38)
    w.u64(s.sun_map_count);
    for (uint64_t i = 0; i < s.sun_map_count; ++i) {
        const dl_sun_map &m = s.sun_maps[i];
        w.u32(m.resolution);
        for (float r : m.rows) w.f32(r);
        w.words(m.texels, m.word_count);
    }
    w.u32(s.sky_probes ? 1u : 0u);
    if (s.sky_probes) {
        const dl_sky_probes &p = *s.sky_probes;
        for (float v : p.origin) w.f32(v);
        w.f32(p.spacing);
        for (uint32_t c : p.counts) w.u32(c);
        w.words(p.words, p.word_count);
    }
    w.u32(s.stats.meshes);
    w.u64(s.stats.triangles);
    w.u64(s.stats.texels);
    w.u64(s.stats.rays);
    w.u64(s.stats.lights_removed);
    w.u64(s.stats.bounce_rays);
    w.u64(s.stats.triangle_words);
}

// The .dynlight payload and its CRC-32.
std::vector<uint8_t> encode_payload(const dl_baked_scene &scene);
uint32_t crc32_ieee(const uint8_t *data, size_t n);
// The raw CRC-32 register (no pre- or post-inversion) after `data`, and after `n` zero bytes: with
// them the CRC of a concatenation follows from its parts' CRCs,
// raw(A B, c) = shift(raw(A, c), |B|) ^ raw(B, 0).
uint32_t crc32_update(uint32_t c, const uint8_t *data, size_t n);
// The slicing tables, 8 x 256 words: table k is the register after byte i and k zero bytes.
const uint32_t *crc32_tables();
uint32_t crc32_shift(uint32_t c, uint64_t n);

}  // namespace dl
