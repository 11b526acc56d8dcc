// The light BVH and light slot order that prepare_scene (dl_host.cpp) builds, for a set of point
// lights read from a file: u32 n, then n x (x, y, z, radius) float32, the lights' ids being
// 1..n in file order. Writes u32 node count, the nodes (8 words each, as the .dynlight file holds
// them) and the local lights' slot order as indices into the file's lights. Built and run by
// tests/test_host_light_bvh.py, which compares the output with the oracle's light BVH
// (light_bvh.rs:59-189).
#include <cstdio>
#include <string>
#include <vector>

#include "dl_host.hpp"

using namespace dl;

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    FILE *in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    uint32_t n = 0;
    if (std::fread(&n, 4, 1, in) != 1) return 2;
    std::vector<float> v((size_t)n * 4);
    if (n && std::fread(v.data(), 4, v.size(), in) != v.size()) return 2;
    std::fclose(in);
    std::vector<dl_light> lights(n);
    for (uint32_t i = 0; i < n; ++i) {
        dl_light l{};
        l.id = i + 1;
        for (int k = 0; k < 3; ++k) l.position[k] = v[i * 4 + k];
        l.radius = v[i * 4 + 3];
        l.shape = DL_SHAPE_POINT;
        l.rotation[3] = 1.0f;
        l.bounce_samples = 32;
        l.bounce_intensity = 1.0f;
        l.bounce_compression = -1;
        lights[i] = l;
    }
    dl_bake_input input{nullptr, 0, lights.data(), lights.size()};
    dl_bake_options o{};
    o.pixel_density = 16.0f;
    o.max_lightmap_size = 2048;
    o.bounce_compression = 8;
    o.photon_cube_resolution = 512;
    o.area_light_samples = 16;
    o.area_light_min_samples = 16;
    o.sun_map_resolution = 64;
    o.sky_samples = 16;
    o.sky_probe_spacing = 1.0f;
    HostScene s;
    std::string err;
    if (prepare_scene(input, o, s, err) != DL_OK) {
        std::fprintf(stderr, "prepare failed: %s\n", err.c_str());
        return 1;
    }
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    uint32_t nodes = (uint32_t)s.light_bvh.size();
    std::fwrite(&nodes, 4, 1, out);
    std::fwrite(s.light_bvh.data(), sizeof(dl_light_bvh_node), nodes, out);
    for (uint32_t slot = 0; slot < s.local_lights; ++slot) {
        uint32_t index = (uint32_t)(s.light_ptrs[slot] - lights.data());
        std::fwrite(&index, 4, 1, out);
    }
    std::fclose(out);
    return 0;
}
