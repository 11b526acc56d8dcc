// Builds the library's occluder BVH over a seeded scene (a heightfield of `grid`^2 vertices plus
// random triangles) and checks it: every occluder in exactly one leaf, every child box padded
// around its subtree's triangles, depth and stack bounds as reported. Prints the build time.
// Built and run by tests/test_bvh_build.py.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "dl_host.hpp"

using namespace dl;

static int failures = 0;
#define CHECK(c, ...)                   \
    do {                                \
        if (!(c)) {                     \
            if (failures < 10) std::printf(__VA_ARGS__); \
            ++failures;                 \
        }                               \
    } while (0)

struct Box {
    float lo[3], hi[3];
};

// Walks the subtree of `ref` inside `box`; marks its triangles; returns the deepest level.
static uint32_t walk(const HostScene &s, int32_t ref, const Box &box, std::vector<int> &seen, uint32_t depth) {
    if (ref < 0) {
        uint32_t packed = (uint32_t)~ref, first = packed >> 3, count = packed & 7u;
        CHECK(count >= 1 && first + count <= seen.size(), "bad leaf %u %u\n", first, count);
        for (uint32_t k = first; k < first + count && k < seen.size(); ++k) {
            ++seen[k];
            const float *v0 = &s.tris[k * 12], *e1 = v0 + 4, *e2 = v0 + 8;
            float p[3][3];
            for (int a = 0; a < 3; ++a) {
                p[0][a] = v0[a];
                p[1][a] = v0[a] + e1[a];
                p[2][a] = v0[a] + e2[a];
            }
            for (int c = 0; c < 3; ++c)
                for (int a = 0; a < 3; ++a)
                    CHECK(p[c][a] >= box.lo[a] && p[c][a] <= box.hi[a], "triangle %u outside its box\n", k);
        }
        return depth;
    }
    const BvhNode &n = s.nodes[(size_t)ref];
    Box b[2] = {{{n.c0[0], n.c0[2], n.c2[0]}, {n.c0[1], n.c0[3], n.c2[1]}},
                {{n.c1[0], n.c1[2], n.c2[2]}, {n.c1[1], n.c1[3], n.c2[3]}}};
    uint32_t d = depth;
    for (int c = 0; c < 2; ++c)
        if (n.ref[c] != -1) d = std::max(d, walk(s, n.ref[c], b[c], seen, depth + 1));
    return d;
}

int main(int argc, char **argv) {
    uint32_t grid = argc > 1 ? (uint32_t)atoi(argv[1]) : 257, extra = argc > 2 ? (uint32_t)atoi(argv[2]) : 20000;
    std::vector<float> pos;
    std::vector<uint32_t> idx;
    for (uint32_t z = 0; z < grid; ++z)
        for (uint32_t x = 0; x < grid; ++x) {
            pos.push_back((float)x);
            pos.push_back(10.0f * std::sin(0.05f * (float)x) * std::cos(0.07f * (float)z));
            pos.push_back((float)z);
        }
    for (uint32_t z = 0; z + 1 < grid; ++z)
        for (uint32_t x = 0; x + 1 < grid; ++x) {
            uint32_t a = z * grid + x, b = a + 1, c = a + grid + 1, d = a + grid;
            idx.insert(idx.end(), {a, d, c, a, c, b});
        }
    uint64_t state = 7;
    auto rnd = [&] { state = splitmix64(state); return (float)((state >> 40) * (1.0 / 16777216.0)); };
    for (uint32_t t = 0; t < extra; ++t) {
        float cx = rnd() * grid, cy = rnd() * 20.0f, cz = rnd() * grid;
        uint32_t base = (uint32_t)(pos.size() / 3);
        for (int k = 0; k < 3; ++k) {
            pos.push_back(cx + rnd() * 2.0f);
            pos.push_back(cy + rnd() * 2.0f);
            pos.push_back(cz + rnd() * 2.0f);
        }
        idx.insert(idx.end(), {base, base + 1, base + 2});
    }
    dl_mesh mesh{};
    mesh.id = 1;
    mesh.vertex_count = (uint32_t)(pos.size() / 3);
    mesh.occludes = 1;
    mesh.index_count = idx.size();
    mesh.positions = pos.data();
    mesh.indices = idx.data();
    HostScene s;
    s.meshes.push_back(&mesh);
    for (uint32_t t = 0; t < idx.size() / 3; ++t) {
        s.occ_mesh.push_back(0);
        s.occ_tri.push_back(t);
    }
    auto t0 = std::chrono::steady_clock::now();
    build_bvh(s);
    double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    size_t n = s.occ_mesh.size();
    std::vector<int> seen(n, 0);
    const BvhNode &root = s.nodes[0];
    Box b[2] = {{{root.c0[0], root.c0[2], root.c2[0]}, {root.c0[1], root.c0[3], root.c2[1]}},
                {{root.c1[0], root.c1[2], root.c2[2]}, {root.c1[1], root.c1[3], root.c2[3]}}};
    uint32_t depth = 1;
    for (int c = 0; c < 2; ++c)
        if (root.ref[c] != -1) depth = std::max(depth, walk(s, root.ref[c], b[c], seen, 2));
    for (size_t k = 0; k < n; ++k) CHECK(seen[k] == 1, "triangle slot %zu in %d leaves\n", k, seen[k]);
    std::vector<int> occ(n, 0);
    for (size_t k = 0; k < n; ++k) {
        uint32_t o;
        std::memcpy(&o, &s.tris[k * 12 + 3], 4);
        CHECK(o < n, "bad occluder index\n");
        if (o < n) ++occ[o];
    }
    for (size_t k = 0; k < n; ++k) CHECK(occ[k] == 1, "occluder %zu stored %d times\n", k, occ[k]);
    CHECK(depth <= s.bvh_depth + 1, "walked depth %u above the reported %u\n", depth, s.bvh_depth);
    std::printf("triangles %zu nodes %zu depth %u build_ms %.1f failures %d\n", n, s.nodes.size(), s.bvh_depth, ms,
                failures);
    return failures ? 1 : 0;
}
