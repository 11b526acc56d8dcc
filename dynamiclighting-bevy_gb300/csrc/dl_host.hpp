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
    std::vector<float> tri_v0, tri_e1, tri_e2;  // 4 floats each (w of v0: occluder index bits)
    uint32_t bvh_depth = 0;
};

// Validates, sorts and prepares (src/bake/baker.rs:32-75). Returns DL_OK or the error status
// with `err` set to the reference's message.
dl_status prepare_scene(const dl_bake_input &in, const dl_bake_options &o, HostScene &s, std::string &err);

// Builds the occluder BVH (binned SAH, leaves of at most 4 triangles, depth capped at 60).
void build_bvh(HostScene &s);

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

// The .dynlight payload (src/bake/format/mod.rs:170-213) and its CRC-32.
std::vector<uint8_t> encode_payload(const dl_baked_scene &scene);
uint32_t crc32_ieee(const uint8_t *data, size_t n);

}  // namespace dl
