// Host half of the bake (see dl_host.hpp). Compiled with -ffp-contract=off: the f32 formulas
// here (surface areas, light bounds, light frames) must round like the reference's Rust.
#include "dl_host.hpp"
#include "dl_bvh_rules.hpp"

#include <algorithm>
#include <memory>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <future>
#include <numeric>
#include <atomic>
#include <thread>

namespace dl {

namespace {

std::string hex_id(uint64_t id) {
    char b[32];
    std::snprintf(b, sizeof b, "%#018llx", (unsigned long long)id);
    return b;
}

// BakeOptions::validate (src/bake/input.rs:336-373)
bool check_options(const dl_bake_options &o, std::string &err) {
    const char *bad = nullptr;
    if (!(std::isfinite(o.pixel_density) && o.pixel_density > 0.0f)) bad = "pixel density must be positive";
    else if (o.max_lightmap_size < 2) bad = "the maximum shadow map size must be at least 2";
    else if (o.photon_cube_resolution == 0) bad = "the photon cube resolution must be positive";
    else if (o.area_light_samples == 0) bad = "area lights need at least one sample";
    else if (o.sun_map_resolution < 1 || o.sun_map_resolution > 8192) bad = "the sun map resolution must be 1 to 8192";
    else if (o.sky_samples == 0) bad = "skies need at least one sample";
    else if (!(std::isfinite(o.sky_probe_spacing) && o.sky_probe_spacing > 0.0f)) bad = "the sky probe spacing must be positive";
    else if (o.bounce_compression != 8 && o.bounce_compression != 6 && o.bounce_compression != 5 && o.bounce_compression != 4)
        bad = "bounce compression must be 8, 6, 5 or 4 bits";
    else if (o.dynamic_geometry > DL_GEOMETRY_ANGULAR) bad = "unknown dynamic geometry mode";
    if (bad) err = std::string("invalid bake options: ") + bad;
    return bad == nullptr;
}

// BakeMesh::validate (src/bake/input.rs:233-287)
bool check_mesh(const dl_mesh &m, std::string &err) {
    auto bad = [&](const std::string &r) {
        err = "mesh " + hex_id(m.id) + ": " + r;
        return false;
    };
    if (m.index_count % 3) return bad(std::to_string(m.index_count) + " indices is not a multiple of 3");
    if (m.index_count && !m.indices) return bad("missing indices");
    for (uint64_t i = 0; i < m.index_count; ++i)
        if (m.indices[i] >= m.vertex_count)
            return bad("index " + std::to_string(m.indices[i]) + " is out of range for " +
                       std::to_string(m.vertex_count) + " vertices");
    if (m.vertex_count && (!m.positions || !m.uv1)) return bad("missing positions or UV1 coordinates");
    for (uint64_t i = 0; i < (uint64_t)m.vertex_count * 3; ++i)
        if (!std::isfinite(m.positions[i])) return bad("non-finite vertex position");
    if (m.alpha) {
        if (!m.uv0) return bad("an alpha texture needs UV0");
        if ((uint64_t)m.alpha->width * m.alpha->height && !m.alpha->rgba8)
            return bad("alpha texture size doesn't match its data");
    }
    return true;
}

// Runs f(i) for i in [0, n) on the host's threads, taking indices from a shared counter (the
// meshes of a scene differ in size by orders of magnitude). Small inputs run inline.
template <class F>
void for_each_index(uint32_t n, uint64_t work, F f) {
    static const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    unsigned threads = work < 65536 ? 1u : std::min<unsigned>(hw, n);
    if (threads <= 1) {
        for (uint32_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<uint32_t> next{0};
    auto body = [&] {
        for (uint32_t i = next++; i < n; i = next++) f(i);
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; ++t) pool.emplace_back(body);
    body();
    for (auto &th : pool) th.join();
}

bool unit_quat(const float q[4]) {
    for (int i = 0; i < 4; ++i)
        if (!std::isfinite(q[i])) return false;
    float n = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    return std::fabs(n - 1.0f) <= 2e-4f;
}

// BakeLight::validate (src/bake/input.rs:290-323)
bool check_light(const dl_light &l, std::string &err) {
    auto bad = [&](const char *r) {
        err = "light " + hex_id(l.id) + ": " + r;
        return false;
    };
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(l.position[i])) return bad("non-finite position");
    if (l.shape > DL_SHAPE_SKY) return bad("unknown light shape");
    bool distant = l.shape == DL_SHAPE_SUN || l.shape == DL_SHAPE_SKY;
    if (!distant && !(std::isfinite(l.radius) && l.radius > 0.0f)) return bad("radius must be positive and finite");
    if (l.shape == DL_SHAPE_RECTANGLE || l.shape == DL_SHAPE_TUBE) {
        if (!std::isfinite(l.size[0]) || !std::isfinite(l.size[1]) || l.size[0] < 0.0f || l.size[1] < 0.0f)
            return bad("area light size must be finite and not negative");
        if (!unit_quat(l.rotation)) return bad("area light rotation must be a unit quaternion");
    }
    if (l.shape == DL_SHAPE_SUN) {
        if (!unit_quat(l.rotation)) return bad("sun rotation must be a unit quaternion");
        if (!(l.size[0] >= 0.0f && l.size[0] <= 10.0f)) return bad("sun angular diameter must be 0 to 10 degrees");
    }
    if (l.bounce_compression >= 0 && l.bounce_compression != 8 && l.bounce_compression != 6 &&
        l.bounce_compression != 5 && l.bounce_compression != 4)
        return bad("bounce compression must be 8, 6, 5 or 4 bits");
    return true;
}

// ---- light BVH (src/bake/light_bvh.rs:59-189): SAH over light positions, <= 2 per leaf ------
struct Box3 {
    f3 lo{INFINITY, INFINITY, INFINITY}, hi{-INFINITY, -INFINITY, -INFINITY};
    void add(const Box3 &b) {
        lo = vmin(lo, b.lo);
        hi = vmax(hi, b.hi);
    }
    // Aabb::half_area_x2 (src/bake/geometry.rs:49-55)
    float area2() const {
        f3 e = sub(hi, lo);
        if (fminf(fminf(e.x, e.y), e.z) < 0.0f) return 0.0f;
        return 2.0f * (e.x * e.y + e.y * e.z + e.z * e.x);
    }
};
Box3 sphere_box(f3 c, float r) { return Box3{sub(c, f3{r, r, r}), add(c, f3{r, r, r})}; }
float axis_of(f3 v, int a) { return a == 0 ? v.x : a == 1 ? v.y : v.z; }

struct LightBvhBuild {
    const std::vector<f3> &pos;
    const std::vector<float> &rad;
    std::vector<uint32_t> order;
    std::vector<dl_light_bvh_node> nodes;

    void bounds(size_t n) {
        Box3 b;
        for (uint32_t k = nodes[n].left_first; k < nodes[n].left_first + nodes[n].count; ++k)
            b.add(sphere_box(pos[order[k]], rad[order[k]]));
        nodes[n].aabb_min[0] = b.lo.x; nodes[n].aabb_min[1] = b.lo.y; nodes[n].aabb_min[2] = b.lo.z;
        nodes[n].aabb_max[0] = b.hi.x; nodes[n].aabb_max[1] = b.hi.y; nodes[n].aabb_max[2] = b.hi.z;
    }
    float cost(uint32_t first, uint32_t count, int ax, float split) const {
        Box3 l, r;
        uint32_t nl = 0, nr = 0;
        for (uint32_t k = first; k < first + count; ++k) {
            uint32_t i = order[k];
            if (axis_of(pos[i], ax) < split) { ++nl; l.add(sphere_box(pos[i], rad[i])); }
            else { ++nr; r.add(sphere_box(pos[i], rad[i])); }
        }
        if (!nl || !nr) return 3.40282347e+38f;
        return (float)nl * l.area2() + (float)nr * r.area2();
    }
    void split(size_t n) {
        uint32_t first = nodes[n].left_first, count = nodes[n].count;
        if (count <= 2) return;
        Box3 box{f3{nodes[n].aabb_min[0], nodes[n].aabb_min[1], nodes[n].aabb_min[2]},
                 f3{nodes[n].aabb_max[0], nodes[n].aabb_max[1], nodes[n].aabb_max[2]}};
        float parent = (float)count * box.area2();
        bool found = false;
        int bax = 0;
        float bsplit = 0.0f, bcost = 3.40282347e+38f;
        for (int ax = 0; ax < 3; ++ax)
            for (uint32_t k = 0; k < count; ++k) {
                float cand = axis_of(pos[order[first + k]], ax);
                float c = cost(first, count, ax, cand);
                if (c < bcost) { bcost = c; bax = ax; bsplit = cand; found = true; }
            }
        if (!found || bcost >= parent) return;
        int64_t i = first, j = (int64_t)first + count - 1;
        while (i <= j) {
            if (axis_of(pos[order[(size_t)i]], bax) < bsplit) ++i;
            else { std::swap(order[(size_t)i], order[(size_t)j]); --j; }
        }
        uint32_t left_count = (uint32_t)(i - first);
        if (left_count == 0 || left_count == count) return;
        size_t left = nodes.size();
        dl_light_bvh_node a{}, b{};
        a.left_first = first; a.count = left_count;
        b.left_first = (uint32_t)i; b.count = count - left_count;
        nodes.push_back(a);
        nodes.push_back(b);
        nodes[n].left_first = (uint32_t)left;
        nodes[n].count = 0;
        bounds(left);
        bounds(left + 1);
        split(left);
        split(left + 1);
    }
};

}  // namespace

dl_status prepare_scene(const dl_bake_input &in, const dl_bake_options &o, HostScene &s, std::string &err) {
    if (!check_options(o, err)) return DL_INVALID_OPTIONS;
    if ((in.mesh_count && !in.meshes) || (in.light_count && !in.lights)) {
        err = "null mesh or light array";
        return DL_INVALID_ARGUMENT;
    }
    // sorted_meshes / sorted_lights (src/bake/baker.rs:205-233)
    for (uint64_t i = 0; i < in.mesh_count; ++i) s.meshes.push_back(&in.meshes[i]);
    std::stable_sort(s.meshes.begin(), s.meshes.end(), [](auto *a, auto *b) { return a->id < b->id; });
    for (size_t i = 1; i < s.meshes.size(); ++i)
        if (s.meshes[i]->id == s.meshes[i - 1]->id) {
            err = "two meshes share BakeId " + hex_id(s.meshes[i]->id);
            return DL_DUPLICATE_ID;
        }
    {
        // every mesh checked on the host's threads; the first failure in sorted order reports
        uint64_t work = 0;
        for (auto *m : s.meshes) work += m->index_count + m->vertex_count;
        std::vector<std::string> errs(s.meshes.size());
        std::vector<uint8_t> ok(s.meshes.size(), 1);
        for_each_index((uint32_t)s.meshes.size(), work, [&](uint32_t i) { ok[i] = check_mesh(*s.meshes[i], errs[i]); });
        for (size_t i = 0; i < ok.size(); ++i)
            if (!ok[i]) {
                err = errs[i];
                return DL_INVALID_MESH;
            }
    }
    std::vector<const dl_light *> lights;
    for (uint64_t i = 0; i < in.light_count; ++i) lights.push_back(&in.lights[i]);
    std::stable_sort(lights.begin(), lights.end(), [](auto *a, auto *b) { return a->id < b->id; });
    for (size_t i = 1; i < lights.size(); ++i)
        if (lights[i]->id == lights[i - 1]->id) {
            err = "two lights share BakeId " + hex_id(lights[i]->id);
            return DL_DUPLICATE_ID;
        }
    for (auto *l : lights)
        if (!check_light(*l, err)) return DL_INVALID_LIGHT;

    // slot order: light BVH order, then suns, then skies (baker.rs:36-50)
    std::vector<const dl_light *> local, suns, skies;
    for (auto *l : lights)
        (l->shape == DL_SHAPE_SUN ? suns : l->shape == DL_SHAPE_SKY ? skies : local).push_back(l);
    std::vector<f3> pos;
    std::vector<float> rad;
    for (auto *l : local) {
        pos.push_back(f3{l->position[0], l->position[1], l->position[2]});
        rad.push_back(l->radius);
    }
    if (!local.empty()) {
        LightBvhBuild b{pos, rad, {}, {}};
        b.order.resize(local.size());
        std::iota(b.order.begin(), b.order.end(), 0u);
        dl_light_bvh_node root{};
        root.count = (uint32_t)local.size();
        b.nodes.push_back(root);
        b.bounds(0);
        b.split(0);
        s.light_bvh = b.nodes;
        for (uint32_t i : b.order) s.light_ptrs.push_back(local[i]);
    }
    s.local_lights = (uint32_t)s.light_ptrs.size();
    for (auto *l : suns) s.light_ptrs.push_back(l);
    for (auto *l : skies) s.light_ptrs.push_back(l);

    for (auto *lp : s.light_ptrs) {
        const dl_light &l = *lp;
        DevLight d{};
        d.position = f3{l.position[0], l.position[1], l.position[2]};
        d.radius = l.radius;
        d.shape = l.shape;
        d.id = l.id;
        bool distant = l.shape == DL_SHAPE_SUN || l.shape == DL_SHAPE_SKY;
        bool area = l.shape == DL_SHAPE_RECTANGLE || l.shape == DL_SHAPE_TUBE;
        bool bounce = l.illumination == DL_ILLUMINATION_SINGLE_BOUNCE && !o.skip_bounce && l.shape != DL_SHAPE_SKY;
        d.flags = (distant ? kLightDistant : 0) | (l.transparency != DL_TRANSPARENCY_DISABLED ? kLightAlpha : 0) |
                  (bounce ? kLightBounce : 0) | (l.shape == DL_SHAPE_RECTANGLE ? kLightRect : 0) |
                  (area ? kLightArea : 0);
        // shadow_bits_per_texel (light_shape.rs:33-43)
        d.shadow_bits = l.shape == DL_SHAPE_POINT ? 1
                        : area ? 4
                        : l.shape == DL_SHAPE_SUN ? (l.size[0] > 0.0f ? 4 : 1)
                        : 8;
        d.bounce_samples = l.bounce_samples < 2 ? 2 : l.bounce_samples;
        d.bounce_intensity = l.bounce_intensity;
        d.bounce_bits = bounce ? (l.bounce_compression >= 0 ? (uint32_t)l.bounce_compression : o.bounce_compression) : 0;
        if (area) {
            // AreaLightShape::at (src/light/area.rs:48-57) and shape_reach (light_shape.rs:22-28)
            d.ax = quat_rotate(l.rotation, f3{1.0f, 0.0f, 0.0f});
            d.ay = quat_rotate(l.rotation, f3{0.0f, 1.0f, 0.0f});
            d.forward = quat_rotate(l.rotation, f3{0.0f, 0.0f, -1.0f});
            d.half_x = l.size[0] * 0.5f;
            d.half_y = l.size[1] * 0.5f;
            d.reach = l.radius - sqrtf(d.half_x * d.half_x + d.half_y * d.half_y);
        } else {
            d.reach = l.radius;
        }
        if (l.shape == DL_SHAPE_SUN) {
            // SunDisk::toward / angular_radius (src/light/shape.rs:95-102)
            d.toward = normalize(quat_rotate(l.rotation, f3{0.0f, 0.0f, 1.0f}));
            d.angular_radius = (l.size[0] * 0.5f) * (kPiF / 180.0f);
            d.tan_radius = tan_f(d.angular_radius);
            d.sin_radius = sin_f(d.angular_radius);
        }
        Box3 b = sphere_box(d.position, d.radius);
        d.bounds_lo = b.lo;
        d.bounds_hi = b.hi;
        s.lights.push_back(d);
        s.bounce_in_scene |= bounce;
    }
    // photon cubes for local bounce lights, in slot order (bounce.rs:126-151)
    for (uint32_t i = 0; i < s.lights.size(); ++i) {
        DevLight &d = s.lights[i];
        d.cube = 0xFFFFFFFFu;
        if ((d.flags & kLightBounce) && d.shape != DL_SHAPE_SUN) {
            d.cube = (uint32_t)s.cube_lights.size();
            s.cube_lights.push_back(i);
        }
    }
    // gaussian_weights(7, 5.0) (bounce_map.rs:140-151): f32 arithmetic, exp rounded once
    {
        const float sigma2 = 5.0f * 5.0f;
        float sum = 0.0f;
        for (int i = -3; i <= 3; ++i) {
            float w = (1.0f / sqrtf(2.0f * kPiF * sigma2)) * (float)std::exp((double)(-(float)(i * i) / (2.0f * sigma2)));
            s.blur_weights[i + 3] = w;
            sum += w;
        }
        float total = 0.0f;
        for (int k = 0; k < 7; ++k) {
            s.blur_weights[k] = s.blur_weights[k] / sum;
            total += s.blur_weights[k];
        }
        s.blur_weight_sum = total;
    }

    // PreparedMesh resolution (mesh_builder.rs:21-51, geometry.rs:66-70) and the occluders
    // (occluder.rs:80-97): meshes on the host's threads, each mesh's area summed in triangle
    // order and its occluders listed in triangle order, the lists joined in mesh order
    const uint32_t M = (uint32_t)s.meshes.size();
    std::vector<std::vector<uint32_t>> occ(M);
    s.resolution.assign(M, 0);
    uint64_t work = 0;
    for (auto *m : s.meshes) work += m->index_count;
    for_each_index(M, work, [&](uint32_t mi) {
        const dl_mesh &m = *s.meshes[mi];
        float area = 0.0f;
        uint64_t tris = m.index_count / 3;
        for (uint64_t t = 0; t < tris; ++t) {
            f3 v[3];
            for (int k = 0; k < 3; ++k) {
                const float *p = m.positions + (size_t)m.indices[t * 3 + k] * 3;
                v[k] = f3{p[0], p[1], p[2]};
            }
            f3 n = cross(sub(v[1], v[0]), sub(v[2], v[0]));
            area += length(n) * 0.5f;
            if (m.occludes && length_sq(n) > 0.0f && std::isfinite(n.x) && std::isfinite(n.y) && std::isfinite(n.z))
                occ[mi].push_back((uint32_t)t);
        }
        float size = ceilf(sqrtf(o.pixel_density * o.pixel_density * area));
        if (std::isnan(size)) size = 0.0f;
        uint32_t r = f2u(fminf(size, (float)o.max_lightmap_size));
        uint32_t hi = std::max(o.max_lightmap_size, 2u);
        s.resolution[mi] = std::min(std::max(r, 2u), hi);
    });
    size_t total = 0;
    for (uint32_t mi = 0; mi < M; ++mi) {
        s.triangles += s.meshes[mi]->index_count / 3;
        total += occ[mi].size();
    }
    s.occ_mesh.reserve(total);
    s.occ_tri.reserve(total);
    for (uint32_t mi = 0; mi < M; ++mi) {
        s.occ_mesh.insert(s.occ_mesh.end(), occ[mi].size(), mi);
        s.occ_tri.insert(s.occ_tri.end(), occ[mi].begin(), occ[mi].end());
    }
    return DL_OK;
}

// ---- occluder BVH: binned SAH --------------------------------------------------------------------
namespace {

struct Prim {
    float lo[3], hi[3], c[3];
};
struct Ref {
    int32_t ref;
    uint32_t count;
    float lo[3], hi[3];
};
// Subtrees larger than this, near the root, are built on their own threads.
constexpr uint32_t kParallelPrims = 16384;
constexpr uint32_t kParallelDepth = 6;
// Nodes with more primitives than this bin and partition them with several threads.
constexpr uint32_t kWidePrims = 65536;

// Runs f(begin, end) over [first, first + count) split into one chunk per thread.
template <class F>
void par_chunks(uint32_t first, uint32_t count, unsigned threads, F f) {
    if (threads <= 1) {
        f(first, first + count, 0u);
        return;
    }
    std::vector<std::thread> pool;
    uint32_t per = (count + threads - 1) / threads;
    for (unsigned t = 1; t < threads; ++t) {
        uint32_t b = first + std::min(count, t * per), e = first + std::min(count, (t + 1) * per);
        pool.emplace_back([=, &f] { f(b, e, t); });
    }
    f(first, first + std::min(count, per), 0u);
    for (auto &th : pool) th.join();
}

struct Builder {
    std::vector<Prim> prims;
    std::vector<uint32_t> idx;

    // Leaves are referenced as ~(first << 3 | count), count <= 7.
    Ref leaf(uint32_t first, uint32_t count, const float lo[3], const float hi[3]) {
        Ref r{~(int32_t)((first << 3) | count), count, {lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]}};
        return r;
    }

    // Builds the subtree over idx[first, first + count) into `nodes`; `max_depth` collects the
    // deepest level. The two children of a large node near the root build concurrently, the
    // second into its own node array that is then appended with its inner references moved.
    // Bounds of the primitives' boxes and centroids over idx[b, e).
    void bounds(uint32_t b, uint32_t e, float lo[3], float hi[3], float clo[3], float chi[3]) const {
        for (uint32_t k = b; k < e; ++k) {
            const Prim &p = prims[idx[k]];
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], p.lo[a]);
                hi[a] = std::max(hi[a], p.hi[a]);
                clo[a] = std::min(clo[a], p.c[a]);
                chi[a] = std::max(chi[a], p.c[a]);
            }
        }
    }
    // Per-axis bins (boxes and counts) of idx[b, e) for centroid bounds clo .. clo + kBvhBins / k.
    struct Bins : BvhBins {
        void reset() {
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < kBvhBins; ++b) {
                    bc[a][b] = 0;
                    for (int j = 0; j < 3; ++j) { bl[a][b][j] = INFINITY; bh[a][b][j] = -INFINITY; }
                }
        }
        void merge(const Bins &o) {
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < kBvhBins; ++b) {
                    bc[a][b] += o.bc[a][b];
                    for (int j = 0; j < 3; ++j) {
                        bl[a][b][j] = std::min(bl[a][b][j], o.bl[a][b][j]);
                        bh[a][b][j] = std::max(bh[a][b][j], o.bh[a][b][j]);
                    }
                }
        }
    };
    void bin(uint32_t b, uint32_t e, const float clo[3], const float k[3], const bool use[3], Bins &out) const {
        for (uint32_t i = b; i < e; ++i) {
            const Prim &p = prims[idx[i]];
            for (int a = 0; a < 3; ++a) {
                if (!use[a]) continue;
                int bb = bvh_bin(p.c[a], clo[a], k[a]);
                ++out.bc[a][bb];
                for (int j = 0; j < 3; ++j) {
                    out.bl[a][bb][j] = std::min(out.bl[a][bb][j], p.lo[j]);
                    out.bh[a][bb][j] = std::max(out.bh[a][bb][j], p.hi[j]);
                }
            }
        }
    }

    Ref build(std::vector<BvhNode> &nodes, uint32_t first, uint32_t count, uint32_t depth, uint32_t &max_depth) {
        max_depth = std::max(max_depth, depth);
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        // min and max are exact, so the split bounds do not depend on how the work is divided
        // the threads of a level share the machine: subtrees above kParallelPrims already run
        // concurrently, 2^depth of them
        static const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const unsigned wide = count > kWidePrims && depth < 16 ? std::max(1u, hw >> std::min(depth - 1, 15u)) : 1u;
        if (wide > 1) {
            std::vector<std::array<float, 12>> part(wide);
            par_chunks(first, count, wide, [&](uint32_t b, uint32_t e, unsigned t) {
                float l[3] = {INFINITY, INFINITY, INFINITY}, h[3] = {-INFINITY, -INFINITY, -INFINITY};
                float cl[3] = {INFINITY, INFINITY, INFINITY}, ch[3] = {-INFINITY, -INFINITY, -INFINITY};
                bounds(b, e, l, h, cl, ch);
                for (int a = 0; a < 3; ++a) {
                    part[t][a] = l[a]; part[t][3 + a] = h[a]; part[t][6 + a] = cl[a]; part[t][9 + a] = ch[a];
                }
            });
            for (const auto &q : part)
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::min(lo[a], q[a]); hi[a] = std::max(hi[a], q[3 + a]);
                    clo[a] = std::min(clo[a], q[6 + a]); chi[a] = std::max(chi[a], q[9 + a]);
                }
        } else {
            bounds(first, first + count, lo, hi, clo, chi);
        }
        if (bvh_leaf_before_bins(count, depth)) return leaf(first, count, lo, hi);
        // SAH over kBvhBins bins per axis
        float kk[3];
        bool use[3];
        for (int a = 0; a < 3; ++a) {
            float ext = chi[a] - clo[a];
            use[a] = ext > 0.0f;
            kk[a] = use[a] ? (float)kBvhBins / ext : 0.0f;
        }
        Bins bins;
        Bins *all = &bins;
        all->reset();
        if (wide > 1) {
            std::vector<Bins> part(wide);
            par_chunks(first, count, wide, [&](uint32_t b, uint32_t e, unsigned t) {
                part[t].reset();
                bin(b, e, clo, kk, use, part[t]);
            });
            for (auto &q : part) all->merge(q);
        } else {
            bin(first, first + count, clo, kk, use, *all);
        }
        float best_cost;
        int best_axis, best_bin;
        bvh_best_split(*all, use, best_cost, best_axis, best_bin);
        BvhSplit how = bvh_decide(count, depth, lo, hi, best_cost, best_axis);
        if (how == kBvhLeaf) return leaf(first, count, lo, hi);
        uint32_t mid;
        if (how == kBvhByIndex) {
            mid = first + count / 2;  // coincident centroids (or the depth cap): split by index
        } else {
            float k = kk[best_axis];
            auto left = [&](uint32_t i) { return bvh_bin(prims[i].c[best_axis], clo[best_axis], k) <= best_bin; };
            if (wide > 1) {
                // stable partition by chunks: count, place through a scratch array, copy back
                std::vector<uint32_t> lefts(wide, 0), starts(wide, 0);
                par_chunks(first, count, wide, [&](uint32_t b, uint32_t e, unsigned t) {
                    uint32_t n = 0;
                    for (uint32_t i = b; i < e; ++i) n += left(idx[i]) ? 1u : 0u;
                    lefts[t] = n;
                    starts[t] = b;
                });
                uint32_t total_left = 0;
                std::vector<uint32_t> lpos(wide), rpos(wide);
                for (unsigned t = 0; t < wide; ++t) {
                    lpos[t] = total_left;
                    total_left += lefts[t];
                }
                uint32_t r_at = total_left;
                for (unsigned t = 0; t < wide; ++t) {
                    rpos[t] = r_at;
                    uint32_t chunk = (t + 1 < wide ? starts[t + 1] : first + count) - starts[t];
                    r_at += chunk - lefts[t];
                }
                std::vector<uint32_t> tmp(count);
                par_chunks(first, count, wide, [&](uint32_t b, uint32_t e, unsigned t) {
                    uint32_t l = lpos[t], r = rpos[t];
                    for (uint32_t i = b; i < e; ++i) {
                        uint32_t v = idx[i];
                        if (left(v)) tmp[l++] = v;
                        else tmp[r++] = v;
                    }
                });
                std::copy(tmp.begin(), tmp.end(), idx.begin() + first);
                mid = first + total_left;
            } else {
                auto it = std::stable_partition(idx.begin() + first, idx.begin() + first + count, left);
                mid = (uint32_t)(it - idx.begin());
            }
            if (mid == first || mid == first + count) mid = first + count / 2;
        }
        size_t node = nodes.size();
        nodes.push_back(BvhNode{});
        Ref l, r;
        if (count > kParallelPrims && depth < kParallelDepth) {
            std::vector<BvhNode> right;
            uint32_t right_depth = 0;
            std::thread worker([&] { r = build(right, mid, first + count - mid, depth + 1, right_depth); });
            l = build(nodes, first, mid - first, depth + 1, max_depth);
            worker.join();
            int32_t base = (int32_t)nodes.size();
            for (BvhNode nd : right) {
                for (int c = 0; c < 2; ++c)
                    if (nd.ref[c] >= 0) nd.ref[c] += base;
                nodes.push_back(nd);
            }
            if (r.ref >= 0) r.ref += base;
            max_depth = std::max(max_depth, right_depth);
        } else {
            l = build(nodes, first, mid - first, depth + 1, max_depth);
            r = build(nodes, mid, first + count - mid, depth + 1, max_depth);
        }
        BvhNode &n = nodes[node];
        n.c0[0] = l.lo[0]; n.c0[1] = l.hi[0]; n.c0[2] = l.lo[1]; n.c0[3] = l.hi[1];
        n.c1[0] = r.lo[0]; n.c1[1] = r.hi[0]; n.c1[2] = r.lo[1]; n.c1[3] = r.hi[1];
        n.c2[0] = l.lo[2]; n.c2[1] = l.hi[2]; n.c2[2] = r.lo[2]; n.c2[3] = r.hi[2];
        n.ref[0] = l.ref; n.ref[1] = r.ref;
        n.count[0] = 0; n.count[1] = 0;
        Ref me{(int32_t)node, 0, {lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]}};
        return me;
    }
};

}  // namespace

void build_bvh(HostScene &s) {
    size_t n = s.occ_mesh.size();
    s.nodes.clear();
    s.tris.assign(n * 12, 0.0f);
    if (n == 0) return;
    Builder b;
    b.prims.resize(n);
    std::vector<f3> v(n * 3);
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned wide = n > kWidePrims ? hw : 1u;
    par_chunks(0, (uint32_t)n, wide, [&](uint32_t lo_i, uint32_t hi_i, unsigned) {
        for (size_t i = lo_i; i < hi_i; ++i) {
            const dl_mesh &m = *s.meshes[s.occ_mesh[i]];
            Prim &p = b.prims[i];
            for (int k = 0; k < 3; ++k) {
                const float *q = m.positions + (size_t)m.indices[(size_t)s.occ_tri[i] * 3 + k] * 3;
                v[i * 3 + k] = f3{q[0], q[1], q[2]};
            }
            for (int a = 0; a < 3; ++a) {
                float x0 = axis_of(v[i * 3], a), x1 = axis_of(v[i * 3 + 1], a), x2 = axis_of(v[i * 3 + 2], a);
                p.lo[a] = std::min(x0, std::min(x1, x2));
                p.hi[a] = std::max(x0, std::max(x1, x2));
                p.c[a] = (p.lo[a] + p.hi[a]) * 0.5f;
            }
        }
    });
    b.idx.resize(n);
    std::iota(b.idx.begin(), b.idx.end(), 0u);
    std::vector<BvhNode> nodes;
    nodes.reserve(n);
    uint32_t max_depth = 0;
    // nodes in depth-first order, the root first, each left subtree before its right one
    Ref root = b.build(nodes, 0, (uint32_t)n, 1, max_depth);
    if (root.ref < 0) {
        // the whole set is one leaf: the root holds it and an empty second child
        nodes.push_back(BvhNode{});
        BvhNode &r = nodes[0];
        r.c0[0] = root.lo[0]; r.c0[1] = root.hi[0]; r.c0[2] = root.lo[1]; r.c0[3] = root.hi[1];
        r.c2[0] = root.lo[2]; r.c2[1] = root.hi[2];
        r.c1[0] = 1e30f; r.c1[1] = -1e30f; r.c1[2] = 1e30f; r.c1[3] = -1e30f;
        r.c2[2] = 1e30f; r.c2[3] = -1e30f;
        r.ref[0] = root.ref; r.ref[1] = ~0; r.count[0] = 0; r.count[1] = 0;
    }
    for (auto &nd : nodes) {
        float lo[3] = {nd.c0[0], nd.c0[2], nd.c2[0]}, hi[3] = {nd.c0[1], nd.c0[3], nd.c2[1]};
        if (nd.ref[0] != ~0) {
            bvh_pad_box(lo, hi);
            nd.c0[0] = lo[0]; nd.c0[1] = hi[0]; nd.c0[2] = lo[1]; nd.c0[3] = hi[1]; nd.c2[0] = lo[2]; nd.c2[1] = hi[2];
        }
        float lo1[3] = {nd.c1[0], nd.c1[2], nd.c2[2]}, hi1[3] = {nd.c1[1], nd.c1[3], nd.c2[3]};
        if (nd.ref[1] != ~0) {
            bvh_pad_box(lo1, hi1);
            nd.c1[0] = lo1[0]; nd.c1[1] = hi1[0]; nd.c1[2] = lo1[1]; nd.c1[3] = hi1[1]; nd.c2[2] = lo1[2]; nd.c2[3] = hi1[2];
        }
    }
    s.nodes = std::move(nodes);
    s.bvh_depth = max_depth;
    s.bvh_node_count = (uint32_t)s.nodes.size();
    par_chunks(0, (uint32_t)n, wide, [&](uint32_t lo_k, uint32_t hi_k, unsigned) {
        for (size_t k = lo_k; k < hi_k; ++k) {
            uint32_t i = b.idx[k];
            f3 a = v[i * 3], e1 = sub(v[i * 3 + 1], a), e2 = sub(v[i * 3 + 2], a);
            uint32_t bits = i;
            float w;
            std::memcpy(&w, &bits, 4);
            float *p0 = &s.tris[k * 12], *p1 = p0 + 4, *p2 = p0 + 8;
            p0[0] = a.x; p0[1] = a.y; p0[2] = a.z; p0[3] = w;
            p1[0] = e1.x; p1[1] = e1.y; p1[2] = e1.z; p1[3] = 0.0f;
            p2[0] = e2.x; p2[1] = e2.y; p2[2] = e2.z; p2[3] = 0.0f;
        }
    });
}

// ---- payload (src/bake/format/mod.rs:170-213, lights.rs:27-52, maps.rs:16-37) -------------------
namespace {
struct Writer {
    std::vector<uint8_t> b;
    void u32(uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void f32(float f) { uint32_t v; std::memcpy(&v, &f, 4); u32(v); }
    void words(const uint32_t *w, uint64_t n) {
        u64(n);
        size_t at = b.size();
        b.resize(at + n * 4);
        for (uint64_t i = 0; i < n; ++i) {  // little-endian words, whatever the host's order
            uint32_t v = w[i];
            uint8_t *o = &b[at + i * 4];
            o[0] = (uint8_t)v;
            o[1] = (uint8_t)(v >> 8);
            o[2] = (uint8_t)(v >> 16);
            o[3] = (uint8_t)(v >> 24);
        }
    }
};
}  // namespace

std::vector<uint16_t> sky_sample_order(uint32_t n) {
    if (n < 16 || n > 65536 || (n & (n - 1))) return {};
    uint32_t m = 0;
    while ((1u << m) < n) ++m;
    auto spread_bits = [](uint32_t v) {  // bit i of v to bit 2i
        uint32_t r = 0;
        for (int i = 0; i < 16; ++i) r |= ((v >> i) & 1u) << (2 * i);
        return r;
    };
    std::vector<std::pair<uint32_t, uint32_t>> keyed;
    for (uint32_t j = 0; j < n; ++j) {
        uint32_t cx = rev_bits(j) >> (32 - (m + 1) / 2);  // the first coordinate's top bits
        uint32_t cy = sobol2(j) >> (32 - m / 2);           // the second's
        keyed.push_back({spread_bits(cx) | (spread_bits(cy) << 1), j});
    }
    std::sort(keyed.begin(), keyed.end());
    std::vector<uint16_t> order(n);
    for (uint32_t r = 0; r < n; ++r) order[r] = (uint16_t)keyed[r].second;
    return order;
}

SampleCells sample_cells(uint32_t n) {
    SampleCells c;
    std::vector<uint16_t> order = sky_sample_order(n);
    if (order.empty()) return c;
    uint32_t m = 0;
    while ((1u << m) < n) ++m;
    const uint32_t xbits = (m + 1) / 2, ybits = m / 2;
    c.cells.resize(n);
    c.samples.resize(n);
    for (uint32_t r = 0; r < n; ++r) {
        uint32_t j = order[r];
        uint32_t cx = rev_bits(j) >> (32 - xbits), cy = ybits ? sobol2(j) >> (32 - ybits) : 0u;
        c.cells[r] = (uint16_t)(cx | cy << 8);
        c.samples[cy << xbits | cx] = (uint16_t)j;
    }
    return c;
}

// ---- maps for moving meshes: host halves -------------------------------------------------------

// Calls f(vertex) for every corner of every occluder triangle (sun_map.rs:164-170).
template <class F>
static void for_occluder_vertices(const HostScene &s, F f) {
    for (size_t i = 0; i < s.occ_mesh.size(); ++i) {
        const dl_mesh &m = *s.meshes[s.occ_mesh[i]];
        const uint32_t *c = m.indices + (size_t)s.occ_tri[i] * 3;
        for (int k = 0; k < 3; ++k) {
            const float *p = m.positions + (size_t)c[k] * 3;
            f(f3{p[0], p[1], p[2]});
        }
    }
}
static bool finite3(f3 v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }

SunMapSetup sun_map_setup(const HostScene &s, uint32_t slot, uint32_t resolution) {
    SunMapSetup m;
    f3 toward = s.lights[slot].toward;
    ortho_pair(toward, m.side, m.up);
    m.along = neg(toward);
    f3 mn{INFINITY, INFINITY, INFINITY}, mx{-INFINITY, -INFINITY, -INFINITY};
    for_occluder_vertices(s, [&](f3 v) {
        f3 l{dot(v, m.side), dot(v, m.up), dot(v, m.along)};
        mn = vmin(mn, l);
        mx = vmax(mx, l);
    });
    if (!(finite3(mn) && finite3(mx))) return m;  // empty: rows zero, one texel
    m.empty = false;
    f3 size = sub(mx, mn);
    float margin = size.z * 0.01f + 0.05f;  // DEPTH_MARGIN (sun_map.rs:20-22)
    m.extent = fmaxf(size.x, size.y) + 2.0f * margin;
    f3 center = scale(add(mn, mx), 0.5f);
    m.bmin = f3{center.x - m.extent * 0.5f, center.y - m.extent * 0.5f, mn.z - margin};
    m.depth = size.z + 2.0f * margin;
    auto row = [](float *r, f3 axis, float lo, float length) {
        f3 a = divs(axis, length);
        r[0] = a.x;
        r[1] = a.y;
        r[2] = a.z;
        r[3] = -lo / length;
    };
    row(m.rows, m.side, m.bmin.x, m.extent);
    row(m.rows + 4, m.up, m.bmin.y, m.extent);
    row(m.rows + 8, m.along, m.bmin.z, m.depth);
    m.resolution = resolution;
    m.texel = m.extent / (float)resolution;
    return m;
}

ProbeGridSetup sky_probe_grid(const HostScene &s, float spacing) {
    ProbeGridSetup g;
    if (s.occ_mesh.empty()) return g;
    bool first = true;
    f3 mn{0, 0, 0}, mx{0, 0, 0};
    for_occluder_vertices(s, [&](f3 v) {
        if (first) {
            mn = mx = v;
            first = false;
        } else {
            mn = vmin(mn, v);
            mx = vmax(mx, v);
        }
    });
    // ProbeGrid::over (sky_probes.rs:45-61), MAX_SKY_PROBES = 65536 (:18)
    f3 extent = add(vmax(sub(mx, mn), f3{0, 0, 0}), f3{spacing, spacing, spacing});
    auto counts_at = [&](float sp) {
        g.counts[0] = f2u(ceilf(extent.x / sp)) + 1;
        g.counts[1] = f2u(ceilf(extent.y / sp)) + 1;
        g.counts[2] = f2u(ceilf(extent.z / sp)) + 1;
    };
    counts_at(spacing);
    while (g.count() > 65536) {
        float ratio = (float)g.count() / 65536.0f;
        spacing = spacing * fmaxf((float)std::cbrt((double)ratio), 1.01f);  // f32::cbrt, rounded once
        counts_at(spacing);
    }
    f3 span{(float)(g.counts[0] - 1) * spacing, (float)(g.counts[1] - 1) * spacing,
            (float)(g.counts[2] - 1) * spacing};
    g.origin = sub(scale(add(mn, mx), 0.5f), scale(span, 0.5f));
    g.spacing = spacing;
    g.present = true;
    return g;
}

std::vector<uint32_t> sky_probe_words(const ProbeGridSetup &g, const float *open, const uint32_t *back,
                                      uint32_t samples) {
    const uint64_t n = g.count();
    const int cx = (int)g.counts[0], cy = (int)g.counts[1], cz = (int)g.counts[2];
    std::vector<float> values(n * 6);
    std::vector<uint8_t> valid(n);
    const float rays = (float)(std::max(samples, 1u) * 6u);
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t b = 0;
        for (int a = 0; a < 6; ++a) b += back[i * 6 + a];
        valid[i] = (float)b <= 0.25f * rays;  // INSIDE_SHARE (sky_probes.rs:20)
        for (int a = 0; a < 6; ++a) values[i * 6 + a] = open[i * 6 + a];
    }
    static const int STEP[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (;;) {  // fill_inside: layer by layer from the previous pass
        std::vector<float> pv = values;
        std::vector<uint8_t> pok = valid;
        bool changed = false;
        for (uint64_t i = 0; i < n; ++i) {
            if (pok[i]) continue;
            int x = (int)(i % (uint64_t)cx), y = (int)(i % ((uint64_t)cx * cy) / (uint64_t)cx),
                z = (int)(i / ((uint64_t)cx * cy));
            float sum[6] = {0, 0, 0, 0, 0, 0}, found = 0.0f;
            for (const auto &st : STEP) {
                int nx = x + st[0], ny = y + st[1], nz = z + st[2];
                if (nx < 0 || ny < 0 || nz < 0 || nx >= cx || ny >= cy || nz >= cz) continue;
                uint64_t j = ((uint64_t)nz * cy + ny) * cx + nx;
                if (!pok[j]) continue;
                for (int a = 0; a < 6; ++a) sum[a] = sum[a] + pv[j * 6 + a];
                found = found + 1.0f;
            }
            if (found > 0.0f) {
                for (int a = 0; a < 6; ++a) values[i * 6 + a] = sum[a] / found;
                valid[i] = 1;
                changed = true;
            }
        }
        if (!changed) break;
    }
    std::vector<uint32_t> words(n * 2, 0);
    for (uint64_t i = 0; i < n; ++i)
        for (int a = 0; a < 6; ++a) {
            float v = valid[i] ? values[i * 6 + a] : 1.0f;
            uint32_t byte = f2u(roundf(clampf(v, 0.0f, 1.0f) * 255.0f));
            words[i * 2 + a / 4] |= byte << (8 * (a % 4));
        }
    return words;
}

std::vector<uint8_t> encode_payload(const dl_baked_scene &s) {
    Writer w;
    emit_payload(s, w);
    return w.b;
}

// CRC-32 (IEEE 802.3, reflected polynomial 0xEDB88320), table-driven.
// CRC-32 tables for slicing by 8 (Intel's slicing-by-8, Kounavis & Berry 2008): t[0] is the
// byte-at-a-time table of the reflected polynomial 0xEDB88320, t[k] advances k more zero bytes.
struct Crc32Tables {
    uint32_t t[8][256];
    Crc32Tables() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[0][i] = c;
        }
        for (uint32_t i = 0; i < 256; ++i)
            for (int k = 1; k < 8; ++k) t[k][i] = t[0][t[k - 1][i] & 0xFF] ^ (t[k - 1][i] >> 8);
    }
};
const Crc32Tables &crc_tables() {
    static const Crc32Tables tables;
    return tables;
}
const uint32_t *crc32_tables() { return &crc_tables().t[0][0]; }

uint32_t crc32_update(uint32_t c, const uint8_t *data, size_t n) {
    const auto &t = crc_tables().t;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint32_t lo = c ^ ((uint32_t)data[i] | (uint32_t)data[i + 1] << 8 | (uint32_t)data[i + 2] << 16 |
                           (uint32_t)data[i + 3] << 24);
        uint32_t hi = (uint32_t)data[i + 4] | (uint32_t)data[i + 5] << 8 | (uint32_t)data[i + 6] << 16 |
                      (uint32_t)data[i + 7] << 24;
        c = t[7][lo & 0xFF] ^ t[6][(lo >> 8) & 0xFF] ^ t[5][(lo >> 16) & 0xFF] ^ t[4][lo >> 24] ^ t[3][hi & 0xFF] ^
            t[2][(hi >> 8) & 0xFF] ^ t[1][(hi >> 16) & 0xFF] ^ t[0][hi >> 24];
    }
    for (; i < n; ++i) c = t[0][(c ^ data[i]) & 0xFF] ^ (c >> 8);
    return c;
}

uint32_t crc32_ieee(const uint8_t *data, size_t n) { return crc32_update(0xFFFFFFFFu, data, n) ^ 0xFFFFFFFFu; }

// The CRC register after `n` more zero bytes: multiplication by x^(8n) modulo the polynomial,
// by squaring the one-zero-byte operator (the technique of zlib's crc32_combine).
namespace {
uint32_t gf2_times(const uint32_t m[32], uint32_t v) {
    uint32_t r = 0;
    for (int i = 0; v; ++i, v >>= 1)
        if (v & 1) r ^= m[i];
    return r;
}
void gf2_square(uint32_t out[32], const uint32_t m[32]) {
    for (int i = 0; i < 32; ++i) out[i] = gf2_times(m, m[i]);
}
}  // namespace
uint32_t crc32_shift(uint32_t c, uint64_t n) {
    uint32_t odd[32], even[32];
    odd[0] = 0xEDB88320u;  // the operator for one zero bit
    for (int i = 1; i < 32; ++i) odd[i] = 1u << (i - 1);
    gf2_square(even, odd);  // two zero bits
    gf2_square(odd, even);  // four zero bits
    while (n) {
        gf2_square(even, odd);  // 8, 32, 128, ... zero bits: one byte, then 4, 16, ... bytes
        if (n & 1) c = gf2_times(even, c);
        n >>= 1;
        if (!n) break;
        gf2_square(odd, even);  // 2, 8, 32, ... bytes
        if (n & 1) c = gf2_times(odd, c);
        n >>= 1;
    }
    return c;
}

}  // namespace dl
