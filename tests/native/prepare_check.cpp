// prepare_scene (dl_host.cpp) on a scene large enough for its threaded passes: the occluder list,
// the per-mesh lightmap sizes and the triangle count against a sequential recomputation of the
// same rules (mesh_builder.rs:21-51, occluder.rs:80-97), and the mesh error reported when several
// meshes are invalid (the first in id order, as the sequential validation reports). Built and run
// by tests/test_host_prepare.py.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "dl_host.hpp"

using namespace dl;

struct MeshData {
    std::vector<float> pos, uv;
    std::vector<uint32_t> idx;
};

// A strip of `quads` quads along x, rows of triangles at mesh-dependent heights; every 7th
// triangle degenerate (a repeated vertex), so the occluder list skips it.
static MeshData strip(uint32_t quads, float z, uint32_t seed) {
    MeshData m;
    for (uint32_t q = 0; q <= quads; ++q) {
        float x = (float)q * 0.37f, y = 0.1f * (float)((q * 2654435761u + seed) % 17);
        m.pos.insert(m.pos.end(), {x, y, z, x, y + 0.2f, z + 0.5f});
        m.uv.insert(m.uv.end(), {(float)q / (float)quads, 0.0f, (float)q / (float)quads, 1.0f});
    }
    for (uint32_t q = 0; q < quads; ++q) {
        uint32_t a = 2 * q, b = a + 1, c = a + 2, d = a + 3;
        uint32_t t = (uint32_t)m.idx.size() / 3;
        if (t % 7 == 3) m.idx.insert(m.idx.end(), {a, a, b});
        else m.idx.insert(m.idx.end(), {a, c, b});
        m.idx.insert(m.idx.end(), {b, c, d});
    }
    return m;
}

int main() {
    int failures = 0;
    std::vector<MeshData> data;
    std::vector<dl_mesh> meshes;
    const uint32_t M = 40;
    for (uint32_t i = 0; i < M; ++i) data.push_back(strip(i % 3 == 0 ? 3000 : 40 + i, (float)i, i));
    for (uint32_t i = 0; i < M; ++i) {
        dl_mesh m{};
        m.id = 1000 - 7 * i;  // ids descending: sorting reverses the order
        m.vertex_count = (uint32_t)data[i].pos.size() / 3;
        m.occludes = i % 5 != 4;
        m.index_count = data[i].idx.size();
        m.positions = data[i].pos.data();
        m.indices = data[i].idx.data();
        m.uv1 = data[i].uv.data();
        m.albedo[0] = m.albedo[1] = m.albedo[2] = 0.5f;
        meshes.push_back(m);
    }
    dl_bake_input in{meshes.data(), meshes.size(), nullptr, 0};
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
    dl_status st = prepare_scene(in, o, s, err);
    if (st != DL_OK) {
        std::printf("prepare failed: %s\n", err.c_str());
        return 1;
    }
    // the sequential rules, meshes in id order
    std::vector<uint32_t> occ_mesh, occ_tri, res;
    uint64_t tris = 0;
    for (uint32_t mi = 0; mi < s.meshes.size(); ++mi) {
        const dl_mesh &m = *s.meshes[mi];
        float area = 0.0f;
        for (uint64_t t = 0; t < m.index_count / 3; ++t) {
            f3 v[3];
            for (int k = 0; k < 3; ++k) {
                const float *p = m.positions + (size_t)m.indices[t * 3 + k] * 3;
                v[k] = f3{p[0], p[1], p[2]};
            }
            f3 n = cross(sub(v[1], v[0]), sub(v[2], v[0]));
            area += length(n) * 0.5f;
            if (m.occludes && length_sq(n) > 0.0f) {
                occ_mesh.push_back(mi);
                occ_tri.push_back((uint32_t)t);
            }
        }
        tris += m.index_count / 3;
        float size = ceilf(sqrtf(o.pixel_density * o.pixel_density * area));
        uint32_t r = (uint32_t)fminf(size, (float)o.max_lightmap_size);
        res.push_back(r < 2 ? 2 : r);
    }
    failures += s.occ_mesh != occ_mesh;
    failures += s.occ_tri != occ_tri;
    failures += s.resolution != res;
    failures += s.triangles != tris;
    for (size_t i = 1; i < s.meshes.size(); ++i) failures += s.meshes[i - 1]->id >= s.meshes[i]->id;
    // two invalid meshes: the error names the one that comes first in id order
    std::vector<uint32_t> bad_idx = data[5].idx;
    bad_idx[4] = 1u << 30;
    std::vector<float> bad_pos = data[20].pos;
    bad_pos[1] = NAN;
    meshes[5].indices = bad_idx.data();    // id 965
    meshes[20].positions = bad_pos.data();  // id 860: first in id order
    HostScene s2;
    std::string err2;
    st = prepare_scene(in, o, s2, err2);
    failures += st != DL_INVALID_MESH;
    failures += err2.find("non-finite vertex position") == std::string::npos;
    std::printf("prepare failures %d (%zu occluders, %zu meshes; error: %s)\n", failures, s.occ_mesh.size(),
                s.meshes.size(), err2.c_str());
    return failures ? 1 : 0;
}
