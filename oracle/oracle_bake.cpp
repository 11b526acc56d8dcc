// TEST INFRASTRUCTURE — the parity oracle, not the product. Only tests/, the smoke check and
// the benchmark's CPU-baseline leg load the library built from this file.
//
// A CPU restatement of the reference baker's bake() (src/bake/baker.rs:27-203) and its
// per-mesh pipeline (src/bake/mesh_bake.rs:73-267, mesh_texels.rs, shadows.rs, seams.rs,
// bounce.rs, triangle_words.rs), in f32 with the reference's operation order. It is
// multithreaded over triangles like the reference's rayon pool; every cross-thread reduction is
// an OR, a max or an integer sum, so results do not depend on the thread count.
//
// Parity with the (unbuildable here) Rust reference is pinned by the reference's own
// known-answer vectors (tests/test_oracle_golden.py) and left unpinned where the reference
// calls glam/libm internals (see oracle_math.hpp).

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>

#include "oracle_maps.hpp"

namespace oracle {

struct Error {
    dl_status status;
    std::string message;
};

// ---- validation (src/bake/input.rs:233-373) -----------------------------------------------------
static bool validate_options(const dl_bake_options &o, Error &e) {
    auto bad = [&](const char *m) { e = Error{DL_INVALID_OPTIONS, m}; return false; };
    if (!(std::isfinite(o.pixel_density) && o.pixel_density > 0.0f)) return bad("pixel density must be positive");
    if (o.max_lightmap_size < 2) return bad("the maximum shadow map size must be at least 2");
    if (o.photon_cube_resolution == 0) return bad("the photon cube resolution must be positive");
    if (o.area_light_samples == 0) return bad("area lights need at least one sample");
    if (o.sun_map_resolution < 1 || o.sun_map_resolution > 8192) return bad("the sun map resolution must be 1 to 8192");
    if (o.sky_samples == 0) return bad("skies need at least one sample");
    if (!(std::isfinite(o.sky_probe_spacing) && o.sky_probe_spacing > 0.0f)) return bad("the sky probe spacing must be positive");
    if (!(o.bounce_compression == 8 || o.bounce_compression == 6 || o.bounce_compression == 5 || o.bounce_compression == 4))
        return bad("bounce compression must be 8, 6, 5 or 4 bits");
    if (o.dynamic_geometry > DL_GEOMETRY_ANGULAR) return bad("unknown dynamic geometry mode");
    return true;
}
static bool validate_mesh(const dl_mesh &m, Error &e) {
    auto bad = [&](const std::string &r) {
        char id[32];
        std::snprintf(id, sizeof id, "%#018llx", (unsigned long long)m.id);
        e = Error{DL_INVALID_MESH, std::string("mesh ") + id + ": " + r};
        return false;
    };
    if (m.index_count % 3) return bad("index count is not a multiple of 3");
    for (uint64_t i = 0; i < m.index_count; ++i)
        if (m.indices[i] >= m.vertex_count) return bad("index out of range");
    if (m.vertex_count && !m.uv1) return bad("missing UV1");
    if (m.vertex_count && !m.positions) return bad("missing positions");
    for (uint64_t i = 0; i < (uint64_t)m.vertex_count * 3; ++i)
        if (!std::isfinite(m.positions[i])) return bad("non-finite vertex position");
    if (m.alpha) {
        if (!m.uv0) return bad("an alpha texture needs UV0");
        if (m.alpha->width && m.alpha->height && !m.alpha->rgba8) return bad("alpha texture size doesn't match its data");
    }
    return true;
}
static bool quat_ok(const float q[4]) {
    for (int i = 0; i < 4; ++i)
        if (!std::isfinite(q[i])) return false;
    float n = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    return std::fabs(n - 1.0f) <= 2e-4f;  // glam is_normalized: |len² − 1| <= 2e-4
}
static bool validate_light(const dl_light &l, Error &e) {
    auto bad = [&](const char *r) {
        char id[32];
        std::snprintf(id, sizeof id, "%#018llx", (unsigned long long)l.id);
        e = Error{DL_INVALID_LIGHT, std::string("light ") + id + ": " + r};
        return false;
    };
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(l.position[i])) return bad("non-finite position");
    bool distant = l.shape == DL_SHAPE_SUN || l.shape == DL_SHAPE_SKY;
    if (!distant && !(std::isfinite(l.radius) && l.radius > 0.0f)) return bad("radius must be positive and finite");
    if (l.shape > DL_SHAPE_SKY) return bad("unknown shape");
    if (l.shape == DL_SHAPE_RECTANGLE || l.shape == DL_SHAPE_TUBE) {
        if (!std::isfinite(l.size[0]) || !std::isfinite(l.size[1]) || l.size[0] < 0.0f || l.size[1] < 0.0f)
            return bad("area light size must be finite and not negative");
        if (!quat_ok(l.rotation)) return bad("area light rotation must be a unit quaternion");
    }
    if (l.shape == DL_SHAPE_SUN) {
        if (!quat_ok(l.rotation)) return bad("sun rotation must be a unit quaternion");
        if (!(l.size[0] >= 0.0f && l.size[0] <= 10.0f)) return bad("sun angular diameter must be 0 to 10 degrees");
    }
    return true;
}

// ---- PreparedMesh (src/bake/mesh_builder.rs:21-101) ---------------------------------------------
struct Prepared {
    const dl_mesh *mesh;
    uint32_t resolution;
    std::vector<V2> uv1;
    uint32_t tris() const { return (uint32_t)(mesh->index_count / 3); }
    V3 pos(uint32_t i) const { return V3{mesh->positions[i * 3], mesh->positions[i * 3 + 1], mesh->positions[i * 3 + 2]}; }
    void vertices(uint32_t t, V3 v[3]) const {
        for (int k = 0; k < 3; ++k) v[k] = pos(mesh->indices[(size_t)t * 3 + k]);
    }
    void normals(uint32_t t, V3 n[3]) const {
        if (!mesh->normals) {
            V3 v[3];
            vertices(t, v);
            V3 f = normalize_or_zero(cross(v[1] - v[0], v[2] - v[0]));
            n[0] = n[1] = n[2] = f;
            return;
        }
        for (int k = 0; k < 3; ++k) {
            uint32_t i = mesh->indices[(size_t)t * 3 + k];
            n[k] = V3{mesh->normals[i * 3], mesh->normals[i * 3 + 1], mesh->normals[i * 3 + 2]};
        }
    }
    void uvs(uint32_t t, V2 uv[3]) const {
        for (int k = 0; k < 3; ++k) uv[k] = uv1[mesh->indices[(size_t)t * 3 + k]];
    }
};
static Prepared prepare(const dl_mesh *m, const dl_bake_options &o) {
    Prepared p;
    p.mesh = m;
    float area = 0.0f;
    for (uint32_t t = 0; t < m->index_count / 3; ++t) {
        V3 v[3];
        for (int k = 0; k < 3; ++k) {
            uint32_t i = m->indices[(size_t)t * 3 + k];
            v[k] = V3{m->positions[i * 3], m->positions[i * 3 + 1], m->positions[i * 3 + 2]};
        }
        area += triangle_area(v[0], v[1], v[2]);
    }
    p.uv1.resize(m->vertex_count);
    for (uint32_t i = 0; i < m->vertex_count; ++i) {
        V2 uv{m->uv1[i * 2], m->uv1[i * 2 + 1]};
        p.uv1[i] = (std::isfinite(uv.x) && std::isfinite(uv.y)) ? uv : V2{0.0f, 0.0f};
    }
    p.resolution = lightmap_size(area, o.pixel_density, o.max_lightmap_size);
    return p;
}

// ---- scene (mesh_bake.rs:30-43) --------------------------------------------------------------
struct Scene {
    const dl_bake_options *options;
    std::vector<Light> lights;  // BVH order, then suns by id, then skies
    size_t local_lights;
    LightBvh light_bvh;
    Occluders occluders;
    bool bounce_in_scene;
    std::vector<int> bounce_kind;  // per slot: 0 none, 1 photons, 2 sun
    std::vector<PhotonCube> cubes; // per slot (empty unless photons)
    std::vector<V3> sun_toward;    // per slot
    std::vector<float> tan_radius; // per slot (suns)
    const dl_progress *progress;
    bool cancelled() const { return progress && progress->cancel; }
};

struct Setup {
    std::vector<uint32_t> lights;
    V3 face_normal;
    Rect crop;
};

// associate (mesh_bake.rs:141-173)
static Setup associate(const Scene &sc, const Prepared &p, uint32_t t) {
    V3 v[3], n[3];
    p.vertices(t, v);
    p.normals(t, n);
    Setup s;
    s.face_normal = normalize_or_zero(cross(v[1] - v[0], v[2] - v[0]));
    bool valid = !is_zero(s.face_normal);
    bool flat = approx_eq(n[0], n[1], 1e-5f) && approx_eq(n[1], n[2], 1e-5f);
    std::vector<uint32_t> cand;
    Aabb box = Aabb::empty().grow(v[0]).grow(v[1]).grow(v[2]);
    sc.light_bvh.query(box, cand);
    for (size_t s2 = sc.local_lights; s2 < sc.lights.size(); ++s2) cand.push_back((uint32_t)s2);
    for (uint32_t slot : cand) {
        const Light &l = sc.lights[slot];
        if (valid && flat && !l.bakes_bounce(*sc.options) && !l.may_face(v, s.face_normal)) continue;
        if (l.is_distant() || sphere_intersects_triangle(l.position(), l.l->radius, v[0], v[1], v[2]))
            s.lights.push_back(slot);
    }
    V2 uv[3];
    p.uvs(t, uv);
    s.crop = crop_rect(uv, p.resolution);
    return s;
}

// MeshTexels (mesh_texels.rs:41-125)
struct MeshTexels {
    BitGrid owned;
    std::vector<std::vector<bool>> buried;
    uint64_t burial_rays = 0;
};
static void centered(const Prepared &p, uint32_t t, V3 face, std::vector<SurfaceTexel> &out) {
    V3 v[3], n[3];
    V2 uv[3];
    p.vertices(t, v);
    p.normals(t, n);
    p.uvs(t, uv);
    triangle_texels(v, n, uv, face, p.resolution, out);
}
static void traced(const Prepared &p, uint32_t t, V3 face, const BitGrid &owned, std::vector<SurfaceTexel> &out) {
    centered(p, t, face, out);
    V3 v[3], n[3];
    V2 uv[3];
    p.vertices(t, v);
    p.normals(t, n);
    p.uvs(t, uv);
    touched_texels(v, n, uv, face, p.resolution, [&](uint32_t x, uint32_t y) { return owned.get(x, y); }, out);
}
static MeshTexels mesh_texels(const Scene &sc, const Prepared &p, const std::vector<Setup> &setups) {
    MeshTexels mt;
    uint32_t size = p.resolution;
    mt.owned = BitGrid(size, size);
    parallel_for(setups.size(), [&](size_t t) {
        if (is_zero(setups[t].face_normal)) return;
        std::vector<SurfaceTexel> c;
        centered(p, (uint32_t)t, setups[t].face_normal, c);
        for (auto &tx : c) mt.owned.set_atomic(tx.x, tx.y);
    });
    mt.buried.resize(setups.size());
    std::atomic<uint64_t> rays{0};
    const uint64_t seed = sc.options->seed, mesh_id = p.mesh->id;
    parallel_for(setups.size(), [&](size_t t) {
        V3 normal = setups[t].face_normal;
        if (is_zero(normal)) return;
        std::vector<SurfaceTexel> texels;
        traced(p, (uint32_t)t, normal, mt.owned, texels);
        std::vector<bool> b(texels.size());
        uint64_t local_rays = 0;
        for (size_t k = 0; k < texels.size(); ++k) {
            V3 origin = texels[k].position + normal * RAY_OFFSET;
            uint64_t parts[6] = {seed, mesh_id, 0x627572696564ull, (uint64_t)t, texels[k].x, texels[k].y};
            Rng rng = stream(parts, 6);
            auto back_face = [&](V3 dir) {
                ++local_rays;
                SurfaceHit hit;
                if (!sc.occluders.closest_hit(origin, dir, INFINITY, false, hit)) return false;
                return dot(sc.occluders.face_normal(hit), dir) > 0.0f;
            };
            b[k] = is_buried(normal, rng.next_f32(), back_face);
        }
        mt.buried[t] = std::move(b);
        rays += local_rays;
    });
    mt.burial_rays = rays;
    return mt;
}
// MeshTexels::of (mesh_texels.rs:92-105)
static void texels_of(const MeshTexels &mt, const Prepared &p, uint32_t t, V3 face, std::vector<SurfaceTexel> &out) {
    std::vector<SurfaceTexel> all;
    traced(p, t, face, mt.owned, all);
    const auto &b = mt.buried[t];
    for (size_t k = 0; k < all.size(); ++k)
        if (!(k < b.size() && b[k])) out.push_back(all[k]);
}

// light_regions (mesh_bake.rs:175-192)
struct Regions {
    std::vector<uint32_t> slot;
    std::vector<std::pair<uint32_t, Rect>> rects;
};
static Regions light_regions(const std::vector<Setup> &setups, size_t light_count) {
    std::vector<bool> has(light_count, false);
    std::vector<Rect> rect(light_count);
    for (const auto &s : setups)
        for (uint32_t l : s.lights) {
            rect[l] = has[l] ? rect[l].unite(s.crop) : s.crop;
            has[l] = true;
        }
    Regions r;
    r.slot.assign(light_count, 0xFFFFFFFFu);
    for (size_t l = 0; l < light_count; ++l)
        if (has[l]) {
            r.slot[l] = (uint32_t)r.rects.size();
            r.rects.push_back({(uint32_t)l, rect[l]});
        }
    return r;
}

// texel_shadow (texel_shadow.rs:20-67) and point_texel (:71-90)
static Visibility texel_shadow(const Scene &sc, const Prepared &p, uint32_t slot, const SurfaceTexel &tx, V3 origin) {
    const Light &light = sc.lights[slot];
    bool alpha = light.alpha_tested();
    auto occluded = [&](V3 dir, float dist) { return sc.occluders.occluded(origin, dir, dist, alpha); };
    Sampling sampling{sc.options->area_light_samples, sc.options->area_light_min_samples};
    uint64_t parts[5] = {sc.options->seed, p.mesh->id, light.l->id, tx.x, tx.y};
    switch (light.l->shape) {
        case DL_SHAPE_POINT: {
            V3 to = light.position() - tx.position;
            float dsq = length_squared(to);
            if (dsq > light.l->radius * light.l->radius) return {false, 0, 0};
            float d = std::sqrt(dsq);
            if (d == 0.0f) return {true, 1.0f, 0};
            V3 dir = to / d;
            if (dot(tx.normal, dir) <= NDOTL_TOLERANCE) return {false, 0, 0};
            return {true, occluded(dir, d) ? 0.0f : 1.0f, 1};
        }
        case DL_SHAPE_RECTANGLE:
        case DL_SHAPE_TUBE: {
            Rng rng = stream(parts, 5);
            return area_visibility(light.area_shape(), light.shape_reach(), tx.position, tx.normal, sampling, rng,
                                   occluded);
        }
        case DL_SHAPE_SUN: {
            Rng rng = stream(parts, 5);
            return sun_visibility(sc.sun_toward[slot], light.sun_angular_radius(), sc.tan_radius[slot], tx.normal,
                                  sampling, rng, [&](V3 dir) { return occluded(dir, INFINITY); });
        }
        default: {
            Rng rng = stream(parts, 5);
            return sky_visibility(tx.normal, sc.options->sky_samples, rng,
                                  [&](V3 dir) { return occluded(dir, INFINITY); });
        }
    }
}

struct Traced {
    BitGrid visited;
    std::vector<ShadowRegion> bits;
    uint64_t texels = 0, rays = 0;
};
// trace (mesh_bake.rs:203-267)
static Traced trace(const Scene &sc, const Prepared &p, const std::vector<Setup> &setups, const Regions &regions,
                    const MeshTexels &mt) {
    Traced tr;
    uint32_t size = p.resolution;
    tr.visited = BitGrid(size, size);
    for (auto &r : regions.rects)
        tr.bits.push_back(ShadowRegion{r.second, ShadowGrid(r.second.width(), r.second.height(),
                                                            sc.lights[r.first].shadow_bits())});
    std::atomic<uint64_t> texels{0}, rays{0};
    parallel_for(setups.size(), [&](size_t t) {
        const Setup &s = setups[t];
        if (is_zero(s.face_normal) || sc.cancelled()) return;
        std::vector<SurfaceTexel> tx;
        texels_of(mt, p, (uint32_t)t, s.face_normal, tx);
        V3 offset = s.face_normal * RAY_OFFSET;
        uint64_t r = 0;
        for (uint32_t slot : s.lights) {
            uint32_t index = regions.slot[slot];
            ShadowRegion &grid = tr.bits[index];
            Rect rect = regions.rects[index].second;
            uint32_t bits = sc.lights[slot].shadow_bits();
            for (const auto &texel : tx) {
                V3 origin = texel.position + offset;
                Visibility v = texel_shadow(sc, p, slot, texel, origin);
                if (!v.some) continue;
                r += v.rays;
                tr.visited.set_atomic(texel.x, texel.y);
                grid.grid.raise_atomic(texel.x - rect.min_x, texel.y - rect.min_y, level_of(v.fraction, bits));
            }
        }
        texels += tx.size();
        rays += r;
    });
    tr.texels = texels;
    tr.rays = rays;
    return tr;
}

// ---- bounce per mesh (bounce.rs:155-292, sun_bounce.rs:24-80) ----------------------------------
struct GatheredTexel {
    uint32_t x, y;
    V3 value;
};
static V3 reflected(const Scene &sc, V3 albedo) { return sc.options->colored_bounce ? albedo : V3{1, 1, 1}; }

static uint64_t gather_triangle(const Scene &sc, const std::vector<SurfaceTexel> &texels, const Setup &s,
                                const Prepared &p, uint32_t slot, std::vector<GatheredTexel> &out) {
    BounceScope bounce_stage;
    if (is_zero(s.face_normal)) return 0;
    const Light &light = sc.lights[slot];
    const PhotonCube &cube = sc.cubes[slot];
    uint32_t samples = std::max(light.l->bounce_samples, 2u);
    float spread_step = 0.9f / (float)(samples - 1);
    bool alpha = light.alpha_tested();
    V3 normal = s.face_normal;
    V3 lp = light.position();
    uint64_t rays = 0;
    for (const auto &tx : texels) {
        V3 to_texel = tx.position - lp;
        if (length_squared(to_texel) > light.l->radius * light.l->radius) continue;
        V3 direction = normalize_or(to_texel, V3{0, 1, 0});
        V3 origin = tx.position + normal * RAY_OFFSET;
        uint64_t parts[5] = {sc.options->seed, p.mesh->id, light.l->id, tx.x, tx.y};
        Rng rng = stream(parts, 5);
        Acc3 sum;
        for (uint32_t i = 0; i < samples; ++i) {
            float spread_s = 0.1f + (float)i * spread_step;
            V3 random = on_unit_sphere(rng);
            V3 sample = normalize_or(slerp(direction, random, spread_s), direction);
            V3 photon, pn, albedo;
            cube.sample(lp, sample, photon, pn, albedo);
            V3 to_photon = photon - origin;
            float distance = length(to_photon);
            if (is_zero(pn) || distance <= 0.0f) continue;
            V3 d = to_photon / distance;
            ++rays;
            if (!sc.occluders.occluded(origin, d, distance, alpha)) {
                float weight = fmax_r(dot(normal, d), 0.0f) * fmax_r(dot(pn, -d), 0.0f);
                sum.add(reflected(sc, albedo) * weight);
            }
        }
        out.push_back(GatheredTexel{tx.x, tx.y, sum.mean(light.l->bounce_intensity, samples)});
    }
    return rays;
}

static uint64_t gather_sun(const Scene &sc, const std::vector<SurfaceTexel> &texels, const Setup &s,
                           const Prepared &p, uint32_t slot, std::vector<GatheredTexel> &out) {
    BounceScope bounce_stage;
    if (is_zero(s.face_normal)) return 0;
    const Light &light = sc.lights[slot];
    V3 toward = sc.sun_toward[slot];
    uint32_t samples = std::max(light.l->bounce_samples, 2u);
    bool alpha = light.alpha_tested();
    V3 normal = s.face_normal;
    const Occluders &occ = sc.occluders;
    uint64_t rays = 0;
    for (const auto &tx : texels) {
        V3 origin = tx.position + normal * RAY_OFFSET;
        uint64_t parts[5] = {sc.options->seed, p.mesh->id, light.l->id, tx.x, tx.y};
        Rng rng = stream(parts, 5);
        V2 offset;
        offset.x = rng.next_f32();
        offset.y = rng.next_f32();
        Acc3 sum;
        for (uint32_t i = 0; i < samples; ++i) {
            V3 direction = cosine_direction(normal, spread(i, offset, true));
            ++rays;
            SurfaceHit hit;
            if (!occ.closest_hit(origin, direction, INFINITY, alpha, hit)) continue;
            V3 face = occ.face_normal(hit);
            if (dot(face, direction) >= 0.0f) continue;
            float lit = dot(occ.surface_normal(hit), toward);
            if (lit <= 0.0f || dot(face, toward) <= 0.0f) continue;
            V3 point = origin + direction * hit.distance + face * RAY_OFFSET;
            ++rays;
            if (!occ.occluded(point, toward, INFINITY, alpha)) sum.add(reflected(sc, occ.albedo(hit)) * lit);
        }
        out.push_back(GatheredTexel{tx.x, tx.y, sum.mean(light.l->bounce_intensity, samples)});
    }
    return rays;
}

// A test hook: the bounce map of one (mesh id, light slot) before and after its filters.
struct BounceCapture {
    bool on = false;
    uint64_t mesh_id = 0;
    uint32_t slot = 0;
    bool taken = false;
    Rect rect{};
    uint32_t size = 0;
    std::vector<V3> pre, post;
};
static BounceCapture g_capture;
// All filtered bounce maps of the next bake, when armed (for precision reports).
struct CapturedMap {
    uint64_t mesh_id;
    uint32_t slot;
    Rect rect;
    std::vector<V3> post;
};
static struct {
    bool on = false;
    std::mutex lock;
    std::vector<CapturedMap> maps;
} g_capture_all;

// bake_mesh_bounce (bounce.rs:155-217): result[t][k] = padded bounce grid or empty.
static uint64_t mesh_bounce(const Scene &sc, const Prepared &p, const std::vector<Setup> &setups,
                            const MeshTexels &mt, std::vector<std::vector<std::vector<V3>>> &result,
                            std::vector<std::vector<bool>> &has) {
    result.assign(setups.size(), {});
    has.assign(setups.size(), {});
    for (size_t t = 0; t < setups.size(); ++t) {
        result[t].resize(setups[t].lights.size());
        has[t].assign(setups[t].lights.size(), false);
    }
    if (!sc.bounce_in_scene) return 0;
    uint64_t rays = 0;
    for (uint32_t slot = 0; slot < sc.lights.size(); ++slot) {
        if (sc.bounce_kind[slot] == 0) continue;
        if (sc.cancelled()) break;
        std::vector<std::pair<uint32_t, uint32_t>> receivers;
        for (uint32_t t = 0; t < setups.size(); ++t) {
            const auto &ls = setups[t].lights;
            for (uint32_t k = 0; k < ls.size(); ++k)
                if (ls[k] == slot) {
                    receivers.push_back({t, k});
                    break;
                }
        }
        if (receivers.empty()) continue;
        Rect crops = setups[receivers[0].first].crop;
        for (auto &r : receivers) crops = crops.unite(setups[r.first].crop);
        std::vector<std::vector<GatheredTexel>> gathered(receivers.size());
        std::vector<uint64_t> counts(receivers.size(), 0);
        parallel_for(receivers.size(), [&](size_t i) {
            uint32_t t = receivers[i].first;
            std::vector<SurfaceTexel> tx;
            if (!is_zero(setups[t].face_normal)) texels_of(mt, p, t, setups[t].face_normal, tx);
            counts[i] = sc.bounce_kind[slot] == 1 ? gather_triangle(sc, tx, setups[t], p, slot, gathered[i])
                                                  : gather_sun(sc, tx, setups[t], p, slot, gathered[i]);
        });
        BounceMap map(p.resolution, crops);
        for (size_t i = 0; i < receivers.size(); ++i) {
            rays += counts[i];
            for (auto &g : gathered[i]) map.set(g.x, g.y, g.value);
        }
        bool capture = g_capture.on && g_capture.mesh_id == p.mesh->id && g_capture.slot == slot;
        if (capture) {
            g_capture.taken = true;
            g_capture.rect = map.rect;
            g_capture.size = map.size;
            g_capture.pre = map.values;
        }
        map.dilate();
        map.blur();
        if (capture) g_capture.post = map.values;
        if (g_capture_all.on) {
            std::lock_guard<std::mutex> guard(g_capture_all.lock);
            g_capture_all.maps.push_back(CapturedMap{p.mesh->id, slot, map.rect, map.values});
        }
        for (auto &r : receivers) has[r.first][r.second] = map.crop(setups[r.first].crop, result[r.first][r.second]);
    }
    return rays;
}

// ---- seams, crop (seams.rs:15-71, shadows.rs:136-159) -----------------------------------------
static void pad_seams(ShadowRegion &region, const BitGrid &visited) {
    Rect rect = region.rect;
    auto vis = [&](int64_t x, int64_t y) { return visited.get_or_false(x, y); };
    static const int D[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
    for (uint32_t y = rect.min_y; y <= rect.max_y; ++y)
        for (uint32_t x = rect.min_x; x <= rect.max_x; ++x) {
            int64_t X = x, Y = y;
            if (vis(X, Y)) continue;
            uint8_t lv = 0;
            for (auto &d : D) {
                int64_t nx = X + d[0], ny = Y + d[1];
                if (vis(nx, ny))
                    lv = std::max(lv, region.get(nx, ny));
                else if (vis(X + 2 * d[0], Y + 2 * d[1]))
                    lv = std::max(lv, region.get(X + 2 * d[0], Y + 2 * d[1]));
            }
            region.grid.set(x - rect.min_x, y - rect.min_y, lv);
        }
}
static uint8_t dilated(const ShadowGrid &copy, uint32_t x, uint32_t y) {
    uint8_t m = 0;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) m = std::max(m, copy.get_or_zero((int64_t)x + dx, (int64_t)y + dy));
    return m;
}
static void dilate_row(ShadowGrid &g, const ShadowGrid &c, uint32_t y) {
    for (uint32_t x = 0; x < g.width; ++x) g.set(x, y, dilated(c, x, y));
}
static void dilate_column(ShadowGrid &g, const ShadowGrid &c, uint32_t x) {
    for (uint32_t y = 0; y < g.height; ++y) g.set(x, y, dilated(c, x, y));
}
static void dilate_shadows(ShadowGrid &g) {
    uint32_t w = g.width, h = g.height;
    ShadowGrid copy = g;
    if (h >= 2) dilate_row(g, copy, 1);
    if (h >= 4) dilate_row(g, copy, h - 2);
    if (w >= 2) dilate_column(g, copy, 1);
    if (w >= 4) dilate_column(g, copy, w - 2);
    copy = g;
    if (h >= 1) dilate_row(g, copy, 0);
    if (h >= 3) dilate_row(g, copy, h - 1);
    if (w >= 1) dilate_column(g, copy, 0);
    if (w >= 3) dilate_column(g, copy, w - 1);
}
static ShadowGrid crop_shadows(const ShadowRegion &region, Rect crop) {
    ShadowGrid g(crop.width() + 4, crop.height() + 4, region.grid.bits);
    for (uint32_t y = crop.min_y; y <= crop.max_y; ++y)
        for (uint32_t x = crop.min_x; x <= crop.max_x; ++x)
            g.set(x - crop.min_x + 2, y - crop.min_y + 2, region.get(x, y));
    dilate_shadows(g);
    return g;
}
static bool any_light(const ShadowRegion &region, Rect rect) {
    Rect r = region.rect;
    uint32_t min_x = std::max(rect.min_x, r.min_x), max_x = std::min(rect.max_x, r.max_x);
    uint32_t min_y = std::max(rect.min_y, r.min_y), max_y = std::min(rect.max_y, r.max_y);
    if (min_x > max_x || min_y > max_y) return false;
    for (uint32_t y = min_y; y <= max_y; ++y)
        for (uint32_t x = min_x; x <= max_x; ++x)
            if (region.grid.get(x - r.min_x, y - r.min_y) != 0) return true;
    return false;
}

// ---- triangle words (triangle_words.rs:47-89) ---------------------------------------------------
struct RecordLight {
    uint32_t light;
    bool has_shadow, has_bounce;
    std::vector<uint32_t> shadow, bounce;
};
struct Record {
    Rect crop;
    std::vector<RecordLight> lights;
};
static std::vector<uint32_t> serialize_triangles(const std::vector<Record> &tris, bool bounce_layout) {
    uint32_t stride = bounce_layout ? 3 : 2;
    std::vector<uint32_t> words;
    for (const auto &t : tris) {
        words.push_back(0);
        words.push_back(t.crop.min_x - 2u);
        words.push_back(t.crop.min_y - 2u);
        words.push_back(t.crop.width() + 4);
    }
    std::vector<size_t> light_data;
    for (size_t i = 0; i < tris.size(); ++i) {
        uint32_t offset = (uint32_t)words.size();
        words[i * 4] = offset;
        light_data.push_back(offset);
        words.push_back((uint32_t)tris[i].lights.size());
        for (const auto &l : tris[i].lights) {
            words.push_back(l.light);
            words.push_back(0);
            if (bounce_layout) words.push_back(0);
        }
    }
    for (size_t i = 0; i < tris.size(); ++i)
        for (size_t k = 0; k < tris[i].lights.size(); ++k) {
            size_t entry = light_data[i] + 1 + k * stride;
            const auto &l = tris[i].lights[k];
            if (l.has_shadow) {
                words[entry + 1] = (uint32_t)words.size();
                words.insert(words.end(), l.shadow.begin(), l.shadow.end());
            }
            if (bounce_layout && l.has_bounce) {
                words[entry + 2] = (uint32_t)words.size();
                words.insert(words.end(), l.bounce.begin(), l.bounce.end());
            }
        }
    return words;
}

// ---- bake_mesh (mesh_bake.rs:73-113) ---------------------------------------------------------
struct MeshOut {
    dl_baked_mesh mesh;
    std::vector<uint32_t> words;
    uint64_t texels, rays, bounce_rays, lights_removed, burial_rays;
};
static MeshOut bake_mesh(const Scene &sc, const Prepared &p) {
    std::vector<Setup> setups(p.tris());
    parallel_for(setups.size(), [&](size_t t) { setups[t] = associate(sc, p, (uint32_t)t); });
    Regions regions = light_regions(setups, sc.lights.size());
    MeshTexels mt = mesh_texels(sc, p, setups);
    Traced tr = trace(sc, p, setups, regions, mt);
    std::vector<std::vector<std::vector<V3>>> bounce;
    std::vector<std::vector<bool>> has_bounce;
    uint64_t bounce_rays = mesh_bounce(sc, p, setups, mt, bounce, has_bounce);

    // LightEntries::optimize (shadows.rs:54-73)
    uint64_t removed = 0;
    std::vector<std::vector<uint32_t>> kept(setups.size());
    for (uint32_t t = 0; t < setups.size(); ++t) {
        V2 uv[3];
        p.uvs(t, uv);
        Rect rect = optimize_rect(uv, p.resolution);
        for (uint32_t k = 0; k < setups[t].lights.size(); ++k) {
            uint32_t l = setups[t].lights[k];
            if (has_bounce[t][k] || any_light(tr.bits[regions.slot[l]], rect))
                kept[t].push_back(k);
            else
                ++removed;
        }
    }
    std::vector<bool> used(sc.lights.size(), false);
    for (uint32_t t = 0; t < setups.size(); ++t)
        for (uint32_t k : kept[t]) used[setups[t].lights[k]] = true;
    parallel_for(regions.rects.size(), [&](size_t i) {
        if (used[regions.rects[i].first]) pad_seams(tr.bits[i], tr.visited);
    });

    // into_records (shadows.rs:87-132)
    std::vector<Record> records(setups.size());
    parallel_for(setups.size(), [&](size_t t) {
        Record &rec = records[t];
        rec.crop = setups[t].crop;
        for (uint32_t k : kept[t]) {
            uint32_t l = setups[t].lights[k];
            const Light &light = sc.lights[l];
            RecordLight rl;
            rl.light = l;
            rl.has_shadow = true;
            rl.shadow = crop_shadows(tr.bits[regions.slot[l]], rec.crop).into_words();
            rl.has_bounce = has_bounce[t][k];
            if (rl.has_bounce) {
                uint32_t bits = light.l->bounce_compression >= 0 ? (uint32_t)light.l->bounce_compression
                                                                  : sc.options->bounce_compression;
                uint64_t parts[4] = {sc.options->seed, p.mesh->id, light.l->id, (uint64_t)t};
                Rng rng = stream(parts, 4);
                if (sc.options->colored_bounce) {
                    rl.bounce = pack_bounce_rgb(bounce[t][k], bits, rng);
                } else {
                    std::vector<float> v;
                    v.reserve(bounce[t][k].size());
                    for (auto &x : bounce[t][k]) v.push_back(x.x);
                    rl.bounce = pack_bounce(v, bits, rng);
                }
            }
            rec.lights.push_back(std::move(rl));
        }
    });
    MeshOut out;
    out.words = serialize_triangles(records, sc.bounce_in_scene);
    out.mesh = dl_baked_mesh{p.mesh->id, p.mesh->content_hash, p.resolution, p.mesh->occludes ? 1u : 0u, nullptr, 0};
    out.texels = tr.texels;
    out.rays = tr.rays;
    out.bounce_rays = bounce_rays;
    out.lights_removed = removed;
    out.burial_rays = mt.burial_rays;
    return out;
}

// ---- bake (baker.rs:27-203) -------------------------------------------------------------------
struct Result {
    dl_baked_scene scene;
    std::vector<dl_baked_light> lights;
    std::vector<dl_light_bvh_node> bvh;
    std::vector<dl_baked_mesh> meshes;
    std::vector<std::vector<uint32_t>> words;
    std::vector<uint32_t> distance_cubes;
    std::vector<SunMapOut> sun_map_data;
    std::vector<dl_sun_map> sun_maps;
    SkyProbesOut probes;
    dl_sky_probes sky_probes{};
    uint64_t burial_rays = 0, photon_rays = 0;
};

// BakeProgress::begin and advance (src/bake/progress.rs:91-100) on the caller's counters, which
// the bake writes and the caller reads from another thread.
static void progress_begin(const dl_progress *p, uint32_t stage, uint64_t total) {
    if (!p) return;
    auto *w = const_cast<dl_progress *>(p);
    w->done = 0;
    w->total = total;
    w->stage = stage;
}
static void progress_advance(const dl_progress *p, uint64_t items) {
    if (p) const_cast<dl_progress *>(p)->done = p->done + items;
}

static bool bake(const dl_bake_input &in, const dl_bake_options &o, const dl_progress *progress, bool brute,
                 Result &res, Error &err) {
    if (!validate_options(o, err)) return false;
    progress_begin(progress, 0, 0);  // BakeStage::Preparing (baker.rs:33)
    // sorted_meshes / sorted_lights (baker.rs:205-233)
    std::vector<const dl_mesh *> meshes;
    for (uint64_t i = 0; i < in.mesh_count; ++i) meshes.push_back(&in.meshes[i]);
    std::stable_sort(meshes.begin(), meshes.end(), [](const dl_mesh *a, const dl_mesh *b) { return a->id < b->id; });
    for (size_t i = 1; i < meshes.size(); ++i)
        if (meshes[i]->id == meshes[i - 1]->id) {
            err = Error{DL_DUPLICATE_ID, "two meshes share a BakeId"};
            return false;
        }
    for (auto *m : meshes)
        if (!validate_mesh(*m, err)) return false;
    std::vector<const dl_light *> lights;
    for (uint64_t i = 0; i < in.light_count; ++i) lights.push_back(&in.lights[i]);
    std::stable_sort(lights.begin(), lights.end(), [](const dl_light *a, const dl_light *b) { return a->id < b->id; });
    for (size_t i = 1; i < lights.size(); ++i)
        if (lights[i]->id == lights[i - 1]->id) {
            err = Error{DL_DUPLICATE_ID, "two lights share a BakeId"};
            return false;
        }
    for (auto *l : lights)
        if (!validate_light(*l, err)) return false;
    std::vector<const dl_light *> local, suns, skies;
    for (auto *l : lights) {
        if (l->shape == DL_SHAPE_SUN) suns.push_back(l);
        else if (l->shape == DL_SHAPE_SKY) skies.push_back(l);
        else local.push_back(l);
    }
    std::vector<V3> pos;
    std::vector<float> rad;
    for (auto *l : local) {
        pos.push_back(V3{l->position[0], l->position[1], l->position[2]});
        rad.push_back(l->radius);
    }
    Scene sc;
    sc.options = &o;
    sc.progress = progress;
    sc.light_bvh = build_light_bvh(pos, rad);
    for (size_t i : sc.light_bvh.order) sc.lights.push_back(Light{local[i]});
    sc.local_lights = local.size();
    for (auto *l : suns) sc.lights.push_back(Light{l});
    for (auto *l : skies) sc.lights.push_back(Light{l});
    sc.bounce_in_scene = false;
    for (auto &l : sc.lights) sc.bounce_in_scene |= l.bakes_bounce(o);
    sc.occluders.brute_force = brute;
    sc.occluders.build(meshes);
    if (progress && progress->cancel) {
        err = Error{DL_CANCELLED, "the bake was cancelled"};
        return false;
    }
    size_t L = sc.lights.size();
    sc.bounce_kind.assign(L, 0);
    sc.cubes.resize(L);
    sc.sun_toward.assign(L, V3{0, 0, 0});
    sc.tan_radius.assign(L, 0.0f);
    for (size_t s = 0; s < L; ++s) {
        const Light &l = sc.lights[s];
        if (l.l->shape == DL_SHAPE_SUN) {
            sc.sun_toward[s] = l.sun_toward();
            sc.tan_radius[s] = tan_f(l.sun_angular_radius());
        }
    }
    uint64_t bounce_lights = 0;
    for (auto &l : sc.lights) bounce_lights += l.bakes_bounce(o) ? 1 : 0;
    progress_begin(progress, 1, bounce_lights);  // BakeStage::PhotonCubes (baker.rs:56-57)
    for (size_t s = 0; s < L; ++s) {
        const Light &l = sc.lights[s];
        if (!l.bakes_bounce(o) || sc.cancelled()) continue;
        if (l.l->shape == DL_SHAPE_SUN) {
            sc.bounce_kind[s] = 2;
        } else {
            sc.bounce_kind[s] = 1;
            sc.cubes[s] = build_photon_cube(l, sc.occluders, o.photon_cube_resolution);
            res.photon_rays += (uint64_t)6 * o.photon_cube_resolution * o.photon_cube_resolution;
        }
        progress_advance(progress, 1);
    }
    if (sc.cancelled()) {
        err = Error{DL_CANCELLED, "the bake was cancelled"};
        return false;
    }
    std::vector<Prepared> prepared;
    for (auto *m : meshes) prepared.push_back(prepare(m, o));
    std::vector<MeshOut> outs;
    progress_begin(progress, 2, prepared.size());  // BakeStage::Meshes (baker.rs:84-89)
    for (auto &p : prepared) {
        outs.push_back(bake_mesh(sc, p));
        progress_advance(progress, 1);
        if (sc.cancelled()) {
            err = Error{DL_CANCELLED, "the bake was cancelled"};
            return false;
        }
    }
    dl_bake_stats stats{};
    stats.meshes = (uint32_t)outs.size();
    for (auto &p : prepared) stats.triangles += p.tris();
    for (auto &out : outs) {
        stats.texels += out.texels;
        stats.rays += out.rays;
        stats.bounce_rays += out.bounce_rays;
        stats.lights_removed += out.lights_removed;
        stats.triangle_words += out.words.size();
        res.burial_rays += out.burial_rays;
    }
    for (auto &l : sc.lights) {
        dl_baked_light b{};
        b.id = l.l->id;
        for (int i = 0; i < 3; ++i) b.origin[i] = l.l->position[i];
        b.radius = l.l->radius;
        b.shape = l.l->shape;
        bool has_rot = l.l->shape != DL_SHAPE_POINT && l.l->shape != DL_SHAPE_SKY;
        b.rotation[0] = has_rot ? l.l->rotation[0] : 0.0f;
        b.rotation[1] = has_rot ? l.l->rotation[1] : 0.0f;
        b.rotation[2] = has_rot ? l.l->rotation[2] : 0.0f;
        b.rotation[3] = has_rot ? l.l->rotation[3] : 1.0f;
        b.size[0] = has_rot ? l.l->size[0] : 0.0f;
        b.size[1] = (l.l->shape == DL_SHAPE_RECTANGLE || l.l->shape == DL_SHAPE_TUBE) ? l.l->size[1] : 0.0f;
        b.bounce_bits = l.bakes_bounce(o) ? (l.l->bounce_compression >= 0 ? (uint32_t)l.l->bounce_compression
                                                                           : o.bounce_compression)
                                          : 0;
        b.shadow_bits_per_texel = l.shadow_bits();
        res.lights.push_back(b);
    }
    res.bvh = sc.light_bvh.nodes;
    // distance cubes, sun maps, sky probes (baker.rs:114-152)
    {
        const bool maps = o.dynamic_geometry != DL_GEOMETRY_LIGHTING_ONLY;
        uint64_t n_suns = 0, n_skies = 0;
        for (size_t s = sc.local_lights; s < sc.lights.size(); ++s) {
            n_suns += sc.lights[s].l->shape == DL_SHAPE_SUN ? 1 : 0;
            n_skies += sc.lights[s].l->shape == DL_SHAPE_SKY ? 1 : 0;
        }
        // BakeStage::DistanceCubes (baker.rs:117-120)
        progress_begin(progress, 3, (uint64_t)sc.local_lights * 6 + (maps ? n_suns : 0) + (maps && n_skies ? 1 : 0));
    }
    if (o.dynamic_geometry != DL_GEOMETRY_LIGHTING_ONLY) {
        res.distance_cubes = bake_distance_cubes(sc.lights, sc.local_lights, sc.occluders);
        bool any_sky = false, sky_alpha = false;
        for (size_t s = sc.local_lights; s < sc.lights.size(); ++s) {
            const Light &l = sc.lights[s];
            if (l.l->shape == DL_SHAPE_SUN)
                res.sun_map_data.push_back(bake_sun_map(sc.sun_toward[s], sc.occluders, o.sun_map_resolution,
                                                        l.alpha_tested()));
            if (l.l->shape == DL_SHAPE_SKY) {
                any_sky = true;
                sky_alpha |= l.alpha_tested();
            }
        }
        if (any_sky) res.probes = bake_sky_probes(sc.occluders, o.sky_probe_spacing, o.sky_samples, sky_alpha, o.seed);
        if (sc.cancelled()) {
            err = Error{DL_CANCELLED, "the bake was cancelled"};
            return false;
        }
    }
    for (auto &m : res.sun_map_data) {
        dl_sun_map d{};
        for (int k = 0; k < 12; ++k) d.rows[k] = m.rows[k];
        d.resolution = m.resolution;
        d.word_count = m.texels.size();
        d.texels = m.texels.data();
        res.sun_maps.push_back(d);
    }
    if (res.probes.present) {
        dl_sky_probes &p = res.sky_probes;
        p.origin[0] = res.probes.origin.x;
        p.origin[1] = res.probes.origin.y;
        p.origin[2] = res.probes.origin.z;
        p.spacing = res.probes.spacing;
        for (int k = 0; k < 3; ++k) p.counts[k] = res.probes.counts[k];
        p.word_count = res.probes.words.size();
        p.words = res.probes.words.data();
    }
    for (auto &out : outs) {
        res.words.push_back(std::move(out.words));
        res.meshes.push_back(out.mesh);
    }
    for (size_t i = 0; i < res.meshes.size(); ++i) {
        res.meshes[i].triangles = res.words[i].data();
        res.meshes[i].word_count = res.words[i].size();
    }
    dl_baked_scene &s = res.scene;
    s = dl_baked_scene{};
    s.settings.bounce = sc.bounce_in_scene;
    s.settings.colored_bounce = sc.bounce_in_scene && o.colored_bounce;
    s.settings.dynamic_geometry = o.dynamic_geometry;
    s.settings.pixel_density = o.pixel_density;
    s.settings.max_lightmap_size = o.max_lightmap_size;
    s.settings.distance_cube_resolution = 64;
    s.light_count = res.lights.size();
    s.lights = res.lights.data();
    s.light_bvh_count = res.bvh.size();
    s.light_bvh = res.bvh.data();
    s.mesh_count = res.meshes.size();
    s.meshes = res.meshes.data();
    s.distance_cube_words = res.distance_cubes.size();
    s.distance_cubes = res.distance_cubes.data();
    s.sun_map_count = res.sun_maps.size();
    s.sun_maps = res.sun_maps.data();
    s.sky_probes = res.probes.present ? &res.sky_probes : nullptr;
    s.stats = stats;
    progress_begin(progress, 4, 0);  // BakeStage::Done (baker.rs:201)
    return true;
}

}  // namespace oracle

using namespace oracle;

// ---- C API for the tests ---------------------------------------------------------------------
extern "C" {

struct oracle_result;
static thread_local std::string g_error;

const char *oracle_last_error(void) { return g_error.c_str(); }

// Bakes with `threads` worker threads (0: all cores). `brute_force` tests every occluder per ray.
// `mode` is a Precision (0 the reference's binary32, 1 the refined form with re-test margin
// `eps`, 2 the FP64 oracle, 3 the bounce-refined form: binary32 but in the bounce stages, which
// run refined); `retests` gets the refined form's binary64 re-tests.
int oracle_bake_ex(const dl_bake_input *in, const dl_bake_options *o, const dl_progress *progress, uint32_t threads,
                   uint32_t brute_force, uint32_t mode, float eps, dl_baked_scene **out, uint64_t *burial_rays,
                   uint64_t *photon_rays, uint64_t *retests) {
    if (mode > PREC_REFINED_BOUNCE || !(eps >= 0.0f)) {
        g_error = "invalid precision mode";
        *out = nullptr;
        return DL_INVALID_OPTIONS;
    }
    thread_count() = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
    precision().mode = mode == PREC_REFINED_BOUNCE ? PREC_F32 : (Precision)mode;
    precision().bounce = mode == PREC_REFINED_BOUNCE ? PREC_REFINED : (Precision)mode;
    precision().eps = eps;
    precision().eps2 = eps * eps;
    retest_count().store(0);
    auto *res = new Result();
    Error err{DL_OK, ""};
    bool ok = bake(*in, *o, progress, brute_force != 0, *res, err);
    precision() = PrecisionMode{};
    if (retests) *retests = retest_count().load();
    if (!ok) {
        g_error = err.message;
        delete res;
        *out = nullptr;
        return err.status;
    }
    if (burial_rays) *burial_rays = res->burial_rays;
    if (photon_rays) *photon_rays = res->photon_rays;
    // dl_baked_scene is the first member, so the scene pointer is the result pointer.
    *out = &res->scene;
    return DL_OK;
}
int oracle_bake(const dl_bake_input *in, const dl_bake_options *o, const dl_progress *progress, uint32_t threads,
                uint32_t brute_force, dl_baked_scene **out, uint64_t *burial_rays, uint64_t *photon_rays) {
    return oracle_bake_ex(in, o, progress, threads, brute_force, PREC_F32, 0.0f, out, burial_rays, photon_rays,
                          nullptr);
}
void oracle_free(dl_baked_scene *s) { delete reinterpret_cast<Result *>(s); }

// Arms (on = 1) or clears the capture of every filtered bounce map of the next bakes.
void oracle_capture_all_bounce(uint32_t on) {
    std::lock_guard<std::mutex> guard(g_capture_all.lock);
    g_capture_all.on = on != 0;
    g_capture_all.maps.clear();
}
uint32_t oracle_captured_map_count(void) { return (uint32_t)g_capture_all.maps.size(); }
// Map i: its mesh id, light slot, window (min_x, min_y, max_x, max_y) and up to `cap` RGB
// texels row-major over the window; returns the window's texel count.
uint32_t oracle_captured_map(uint32_t i, uint64_t *mesh_id, uint32_t *slot, uint32_t rect[4], float *rgb,
                             uint32_t cap) {
    if (i >= g_capture_all.maps.size()) return 0;
    const CapturedMap &m = g_capture_all.maps[i];
    *mesh_id = m.mesh_id;
    *slot = m.slot;
    rect[0] = m.rect.min_x; rect[1] = m.rect.min_y; rect[2] = m.rect.max_x; rect[3] = m.rect.max_y;
    uint32_t n = (uint32_t)m.post.size();
    for (uint32_t k = 0; k < n && k < cap; ++k) {
        rgb[k * 3] = m.post[k].x;
        rgb[k * 3 + 1] = m.post[k].y;
        rgb[k * 3 + 2] = m.post[k].z;
    }
    return n;
}

// Arms the bounce-map capture of (mesh id, light slot) for the next oracle_bake.
void oracle_capture_bounce(uint64_t mesh_id, uint32_t slot) {
    g_capture = BounceCapture{};
    g_capture.on = true;
    g_capture.mesh_id = mesh_id;
    g_capture.slot = slot;
}
// The captured window (rect min_x, min_y, max_x, max_y; map size) and its texels before and after
// the filters, RGB floats; returns the texel count (0 when nothing was captured).
uint32_t oracle_captured_bounce(uint32_t rect[4], uint32_t *size, float *pre, float *post, uint32_t cap) {
    if (!g_capture.taken) return 0;
    rect[0] = g_capture.rect.min_x; rect[1] = g_capture.rect.min_y;
    rect[2] = g_capture.rect.max_x; rect[3] = g_capture.rect.max_y;
    *size = g_capture.size;
    uint32_t n = (uint32_t)g_capture.pre.size();
    for (uint32_t i = 0; i < n && i < cap; ++i) {
        pre[i * 3] = g_capture.pre[i].x; pre[i * 3 + 1] = g_capture.pre[i].y; pre[i * 3 + 2] = g_capture.pre[i].z;
        post[i * 3] = g_capture.post[i].x; post[i * 3 + 1] = g_capture.post[i].y; post[i * 3 + 2] = g_capture.post[i].z;
    }
    g_capture.on = false;
    return n;
}

// ---- known-answer hooks (one per reference unit test family) ----------------------------------
uint32_t oracle_lightmap_size(float area, float density, uint32_t max_size) {
    return lightmap_size(area, density, max_size);
}
void oracle_rects(const float uv[6], uint32_t size, uint32_t out[12]) {
    V2 u[3] = {{uv[0], uv[1]}, {uv[2], uv[3]}, {uv[4], uv[5]}};
    Rect r[3] = {crop_rect(u, size), trace_rect(u, size), optimize_rect(u, size)};
    for (int i = 0; i < 3; ++i) {
        out[i * 4] = r[i].min_x; out[i * 4 + 1] = r[i].min_y; out[i * 4 + 2] = r[i].max_x; out[i * 4 + 3] = r[i].max_y;
    }
}
// mode 0: centered texels; mode 1: touched texels with `owned` (size*size bytes, may be NULL).
uint32_t oracle_texels(uint32_t mode, const float v[9], const float n[9], const float uv[6], const float face[3],
                       uint32_t size, const uint8_t *owned, uint32_t cap, uint32_t *xy, float *pos, float *nrm) {
    V3 vv[3], nn[3];
    V2 u[3];
    for (int k = 0; k < 3; ++k) {
        vv[k] = V3{v[k * 3], v[k * 3 + 1], v[k * 3 + 2]};
        nn[k] = V3{n[k * 3], n[k * 3 + 1], n[k * 3 + 2]};
        u[k] = V2{uv[k * 2], uv[k * 2 + 1]};
    }
    V3 f{face[0], face[1], face[2]};
    std::vector<SurfaceTexel> out;
    if (mode == 0)
        triangle_texels(vv, nn, u, f, size, out);
    else
        touched_texels(vv, nn, u, f, size, [&](uint32_t x, uint32_t y) { return owned && owned[(size_t)y * size + x]; }, out);
    uint32_t count = (uint32_t)std::min<size_t>(out.size(), cap);
    for (uint32_t i = 0; i < count; ++i) {
        xy[i * 2] = out[i].x; xy[i * 2 + 1] = out[i].y;
        pos[i * 3] = out[i].position.x; pos[i * 3 + 1] = out[i].position.y; pos[i * 3 + 2] = out[i].position.z;
        nrm[i * 3] = out[i].normal.x; nrm[i * 3 + 1] = out[i].normal.y; nrm[i * 3 + 2] = out[i].normal.z;
    }
    return (uint32_t)out.size();
}
typedef int (*oracle_dir_fn)(const float *dir, float distance);
// is_buried with a callback answering "back face?" per direction; returns buried, fills rays.
int oracle_is_buried(const float normal[3], float turn, oracle_dir_fn back_face, uint32_t *rays) {
    uint32_t count = 0;
    bool b = is_buried(V3{normal[0], normal[1], normal[2]}, turn, [&](V3 d) {
        ++count;
        float a[3] = {d.x, d.y, d.z};
        return back_face(a, 0.0f) != 0;
    });
    *rays = count;
    return b;
}
uint8_t oracle_level(float fraction, uint32_t bits) { return level(fraction, bits); }
// Packs `levels` (w*h) into words as ShadowGrid::into_words does; returns the word count.
uint32_t oracle_pack_levels(const uint8_t *levels, uint32_t w, uint32_t h, uint32_t bits, uint32_t *words) {
    ShadowGrid g(w, h, bits);
    for (uint32_t i = 0; i < w * h; ++i) g.levels[i] = bits == 1 ? (levels[i] != 0) : levels[i];
    auto out = g.into_words();
    std::memcpy(words, out.data(), out.size() * 4);
    return (uint32_t)out.size();
}
// pad_seams on a region covering rect (levels w*h) of a map whose visited bits are `visited`
// (map_w*map_h bytes).
void oracle_pad_seams(uint8_t *levels, const uint32_t rect[4], uint32_t bits, const uint8_t *visited, uint32_t map_w,
                      uint32_t map_h) {
    ShadowRegion r{Rect{rect[0], rect[1], rect[2], rect[3]}, ShadowGrid(rect[2] - rect[0] + 1, rect[3] - rect[1] + 1, bits)};
    for (size_t i = 0; i < r.grid.levels.size(); ++i) r.grid.levels[i] = levels[i];
    BitGrid vis(map_w, map_h);
    for (uint32_t y = 0; y < map_h; ++y)
        for (uint32_t x = 0; x < map_w; ++x)
            if (visited[(size_t)y * map_w + x]) vis.set(x, y, true);
    pad_seams(r, vis);
    for (size_t i = 0; i < r.grid.levels.size(); ++i) levels[i] = r.grid.levels[i];
}
void oracle_dilate(uint8_t *levels, uint32_t w, uint32_t h, uint32_t bits) {
    ShadowGrid g(w, h, bits);
    for (size_t i = 0; i < g.levels.size(); ++i) g.levels[i] = levels[i];
    dilate_shadows(g);
    for (size_t i = 0; i < g.levels.size(); ++i) levels[i] = g.levels[i];
}
// Serializes records given as flat arrays: per triangle its crop (4 u32) and light count; per
// light entry: light, shadow word count (or 0xFFFFFFFF for none), bounce word count (or none),
// then the words. Returns the word count written into `out` (capacity `cap`).
uint32_t oracle_serialize(uint32_t triangles, const uint32_t *crops, const uint32_t *light_counts,
                          const uint32_t *entries, const uint32_t *payload, uint32_t bounce_layout, uint32_t cap,
                          uint32_t *out) {
    std::vector<Record> recs(triangles);
    size_t e = 0, w = 0;
    for (uint32_t t = 0; t < triangles; ++t) {
        recs[t].crop = Rect{crops[t * 4], crops[t * 4 + 1], crops[t * 4 + 2], crops[t * 4 + 3]};
        for (uint32_t k = 0; k < light_counts[t]; ++k, ++e) {
            RecordLight rl;
            rl.light = entries[e * 3];
            uint32_t ns = entries[e * 3 + 1], nb = entries[e * 3 + 2];
            rl.has_shadow = ns != 0xFFFFFFFFu;
            rl.has_bounce = nb != 0xFFFFFFFFu;
            if (rl.has_shadow) { rl.shadow.assign(payload + w, payload + w + ns); w += ns; }
            if (rl.has_bounce) { rl.bounce.assign(payload + w, payload + w + nb); w += nb; }
            recs[t].lights.push_back(rl);
        }
    }
    auto words = serialize_triangles(recs, bounce_layout != 0);
    uint32_t n = (uint32_t)std::min<size_t>(words.size(), cap);
    std::memcpy(out, words.data(), n * 4);
    return (uint32_t)words.size();
}
void oracle_spread(uint32_t index, float ox, float oy, uint32_t rectangle, float out[2]) {
    V2 p = spread(index, V2{ox, oy}, rectangle != 0);
    out[0] = p.x; out[1] = p.y;
}
void oracle_concentric_disk(float sx, float sy, float out[2]) {
    V2 p = concentric_disk(V2{sx, sy});
    out[0] = p.x; out[1] = p.y;
}
void oracle_cosine_direction(const float n[3], float sx, float sy, float out[3]) {
    V3 d = cosine_direction(V3{n[0], n[1], n[2]}, V2{sx, sy});
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}
uint64_t oracle_seed(const uint64_t *parts, uint32_t n) { return key_seed(parts, (int)n); }
void oracle_stream_u32(const uint64_t *parts, uint32_t n, uint32_t count, uint32_t *out) {
    Rng r = stream(parts, (int)n);
    for (uint32_t i = 0; i < count; ++i) out[i] = r.next_u32();
}
void oracle_sincos(float x, float out[2]) { sincos_f(x, out[0], out[1]); }
float oracle_acos_approx(float x) { return acos_approx(x); }
float oracle_tan(float x) { return tan_f(x); }
int oracle_intersect(const float v[9], const float o[3], const float d[3], float max, float *t, float w[3]) {
    V3 vv[3] = {{v[0], v[1], v[2]}, {v[3], v[4], v[5]}, {v[6], v[7], v[8]}};
    V3 ww;
    bool hit = intersect(vv, V3{o[0], o[1], o[2]}, V3{d[0], d[1], d[2]}, max, *t, ww);
    if (hit) { w[0] = ww.x; w[1] = ww.y; w[2] = ww.z; }
    return hit;
}
// n ray/triangle tests in precision `mode` (re-test margin `eps`): triangle i is v[9i..9i+9],
// ray i o[3i..], d[3i..] with length max[i]; hit[i] gets 1/0 and t[i] the distance of a hit.
// Returns the refined mode's binary64 re-tests.
uint64_t oracle_intersect_batch(uint32_t mode, float eps, uint32_t n, const float *v, const float *o, const float *d,
                                const float *max, uint8_t *hit, float *t) {
    precision().mode = (Precision)std::min<uint32_t>(mode, PREC_F64);
    precision().eps = eps;
    precision().eps2 = eps * eps;
    retest_count().store(0);
    for (uint32_t i = 0; i < n; ++i) {
        const float *a = v + (size_t)i * 9;
        V3 vv[3] = {{a[0], a[1], a[2]}, {a[3], a[4], a[5]}, {a[6], a[7], a[8]}};
        V3 w;
        float ti = 0.0f;
        hit[i] = intersect(vv, V3{o[i * 3], o[i * 3 + 1], o[i * 3 + 2]}, V3{d[i * 3], d[i * 3 + 1], d[i * 3 + 2]},
                           max[i], ti, w);
        t[i] = hit[i] ? ti : 0.0f;
    }
    precision() = PrecisionMode{};
    return retest_count().load();
}
// f32 -> f16 bits of the distance cubes' packing.
uint16_t oracle_f16_bits(float f) { return f16_bits(f); }
// ProbeGrid::over (sky_probes.rs:45-61): origin, spacing and counts of the probe grid.
void oracle_probe_grid(const float mn[3], const float mx[3], float spacing, float origin[3], float *out_spacing,
                       uint32_t counts[3]) {
    ProbeGrid g = ProbeGrid::over(V3{mn[0], mn[1], mn[2]}, V3{mx[0], mx[1], mx[2]}, spacing);
    origin[0] = g.origin.x;
    origin[1] = g.origin.y;
    origin[2] = g.origin.z;
    *out_spacing = g.spacing;
    for (int k = 0; k < 3; ++k) counts[k] = g.counts[k];
}
// fill_inside (sky_probes.rs:114-146) on a grid of `counts`: values 6 per probe, valid 0/1, in place.
void oracle_fill_inside(const uint32_t counts[3], float *values, uint8_t *valid) {
    ProbeGrid g{};
    for (int k = 0; k < 3; ++k) g.counts[k] = counts[k];
    uint64_t n = g.count();
    std::vector<std::array<float, 6>> v(n);
    std::vector<uint8_t> ok(valid, valid + n);
    for (uint64_t i = 0; i < n; ++i)
        for (int k = 0; k < 6; ++k) v[i][k] = values[i * 6 + k];
    fill_inside(g, v, ok);
    for (uint64_t i = 0; i < n; ++i) {
        valid[i] = ok[i];
        for (int k = 0; k < 6; ++k) values[i * 6 + k] = v[i][k];
    }
}
// Area-light visibility of one texel with a callback `blocked(dir, distance)`; the shape is the
// light's rotation and size at `center`. Returns 1 with fraction/rays, or 0 for None.
int oracle_area_visibility(uint32_t rectangle, const float rotation[4], const float size[2], const float center[3],
                           float reach, const float pos[3], const float normal[3], uint32_t samples, uint32_t minimum,
                           const uint64_t *parts, uint32_t nparts, oracle_dir_fn blocked, float *fraction,
                           uint32_t *rays) {
    dl_light l{};
    l.shape = rectangle ? DL_SHAPE_RECTANGLE : DL_SHAPE_TUBE;
    for (int i = 0; i < 4; ++i) l.rotation[i] = rotation[i];
    l.size[0] = size[0]; l.size[1] = size[1];
    for (int i = 0; i < 3; ++i) l.position[i] = center[i];
    AreaShape s = Light{&l}.area_shape();
    Rng rng = stream(parts, (int)nparts);
    Visibility v = area_visibility(s, reach, V3{pos[0], pos[1], pos[2]}, V3{normal[0], normal[1], normal[2]},
                                   Sampling{samples, minimum}, rng, [&](V3 d, float dist) {
                                       float a[3] = {d.x, d.y, d.z};
                                       return blocked(a, dist) != 0;
                                   });
    *fraction = v.fraction;
    *rays = v.rays;
    return v.some;
}
int oracle_sun_visibility(const float rotation[4], float diameter, const float normal[3], uint32_t samples,
                          uint32_t minimum, const uint64_t *parts, uint32_t nparts, oracle_dir_fn blocked,
                          float *fraction, uint32_t *rays) {
    dl_light l{};
    l.shape = DL_SHAPE_SUN;
    for (int i = 0; i < 4; ++i) l.rotation[i] = rotation[i];
    l.size[0] = diameter;
    Light light{&l};
    Rng rng = stream(parts, (int)nparts);
    float radius = light.sun_angular_radius();
    Visibility v = sun_visibility(light.sun_toward(), radius, tan_f(radius), V3{normal[0], normal[1], normal[2]},
                                  Sampling{samples, minimum}, rng, [&](V3 d) {
                                      float a[3] = {d.x, d.y, d.z};
                                      return blocked(a, INFINITY) != 0;
                                  });
    *fraction = v.fraction;
    *rays = v.rays;
    return v.some;
}
float oracle_sky_visibility(const float normal[3], uint32_t samples, const uint64_t *parts, uint32_t nparts,
                            oracle_dir_fn blocked) {
    Rng rng = stream(parts, (int)nparts);
    return sky_visibility(V3{normal[0], normal[1], normal[2]}, samples, rng, [&](V3 d) {
               float a[3] = {d.x, d.y, d.z};
               return blocked(a, INFINITY) != 0;
           }).fraction;
}
void oracle_any_orthonormal_pair(const float n[3], float out[6]) {
    V3 a, b;
    any_orthonormal_pair(V3{n[0], n[1], n[2]}, a, b);
    out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = b.x; out[4] = b.y; out[5] = b.z;
}
void oracle_quat_rotate(const float q[4], const float v[3], float out[3]) {
    V3 r = quat_rotate(q, V3{v[0], v[1], v[2]});
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
// Light BVH over spheres: fills nodes (capacity 2n) and order; returns the node count.
uint32_t oracle_light_bvh(const float *positions, const float *radii, uint32_t n, dl_light_bvh_node *nodes,
                          uint32_t *order) {
    std::vector<V3> p;
    std::vector<float> r;
    for (uint32_t i = 0; i < n; ++i) {
        p.push_back(V3{positions[i * 3], positions[i * 3 + 1], positions[i * 3 + 2]});
        r.push_back(radii[i]);
    }
    LightBvh b = build_light_bvh(p, r);
    for (size_t i = 0; i < b.nodes.size(); ++i) nodes[i] = b.nodes[i];
    for (size_t i = 0; i < b.order.size(); ++i) order[i] = (uint32_t)b.order[i];
    return (uint32_t)b.nodes.size();
}
void oracle_gaussian_weights(float out[7]) { gaussian_weights(out); }
// pack_bounce (rgb = 0: one channel of `values`, else 3 channels per pixel).
uint32_t oracle_pack_bounce(const float *values, uint32_t count, uint32_t rgb, uint32_t bits, const uint64_t *parts,
                            uint32_t nparts, uint32_t *words) {
    Rng rng = parts ? stream(parts, (int)nparts) : rng_new(splitmix64(0 ^ splitmix64(0)), 0);
    std::vector<uint32_t> out;
    if (rgb) {
        std::vector<V3> v;
        for (uint32_t i = 0; i < count; ++i) v.push_back(V3{values[i * 3], values[i * 3 + 1], values[i * 3 + 2]});
        out = pack_bounce_rgb(v, bits, rng);
    } else {
        out = pack_bounce(std::vector<float>(values, values + count), bits, rng);
    }
    std::memcpy(words, out.data(), out.size() * 4);
    return (uint32_t)out.size();
}
// BounceMap: set `count` texels (x, y, r, g, b), dilate, blur, then write the window over
// `crops` (min_x, min_y, max_x, max_y) into out (window w*h*3 floats); returns the window rect.
void oracle_bounce_map(uint32_t size, const uint32_t crops[4], const float *texels, uint32_t count, float *out,
                       uint32_t window[4]) {
    BounceMap m(size, Rect{crops[0], crops[1], crops[2], crops[3]});
    for (uint32_t i = 0; i < count; ++i)
        m.set((uint32_t)texels[i * 5], (uint32_t)texels[i * 5 + 1], V3{texels[i * 5 + 2], texels[i * 5 + 3], texels[i * 5 + 4]});
    m.dilate();
    m.blur();
    for (size_t i = 0; i < m.values.size(); ++i) {
        out[i * 3] = m.values[i].x; out[i * 3 + 1] = m.values[i].y; out[i * 3 + 2] = m.values[i].z;
    }
    window[0] = m.rect.min_x; window[1] = m.rect.min_y; window[2] = m.rect.max_x; window[3] = m.rect.max_y;
}
void oracle_cube_texel(const float d[3], uint32_t res, uint32_t out[3]) {
    direction_to_texel(V3{d[0], d[1], d[2]}, res, out[0], out[1], out[2]);
}
void oracle_cube_direction(uint32_t face, uint32_t x, uint32_t y, uint32_t res, float out[3]) {
    V3 d = texel_direction(face, x, y, res);
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}
void oracle_slerp(const float a[3], const float b[3], float s, float out[3]) {
    V3 r = slerp(V3{a[0], a[1], a[2]}, V3{b[0], b[1], b[2]}, s);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

// ---- random streams (effects/rng.rs:27-93, random.rs:8-28) ----
// `count` values of EffectRng::new(seed, stream).
void oracle_rng_u32(uint64_t seed, uint64_t stream_id, uint32_t count, uint32_t *out) {
    Rng r = rng_new(seed, stream_id);
    for (uint32_t i = 0; i < count; ++i) out[i] = r.next_u32();
}
// `count` points of on_unit_sphere from the keyed stream of `parts`.
void oracle_sphere_points(const uint64_t *parts, int n, uint32_t count, float *out) {
    Rng r = stream(parts, n);
    for (uint32_t i = 0; i < count; ++i) {
        V3 p = on_unit_sphere(r);
        out[i * 3] = p.x; out[i * 3 + 1] = p.y; out[i * 3 + 2] = p.z;
    }
}

// ---- geometry.rs helpers (geometry.rs:19-140) ----
static V3 v3_at(const float *p) { return V3{p[0], p[1], p[2]}; }
void oracle_closest_point(const float p[3], const float tri[9], float out[3]) {
    V3 r = closest_point_on_triangle(v3_at(p), v3_at(tri), v3_at(tri + 3), v3_at(tri + 6));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
int oracle_sphere_triangle(const float center[3], float radius, const float tri[9]) {
    return sphere_intersects_triangle(v3_at(center), radius, v3_at(tri), v3_at(tri + 3), v3_at(tri + 6)) ? 1 : 0;
}
// 1 and the weights when `p` lies in the UV triangle `t` (either winding), else 0.
int oracle_uv_barycentrics(const float t[6], const float p[2], float out[3]) {
    V2 tt[3] = {V2{t[0], t[1]}, V2{t[2], t[3]}, V2{t[4], t[5]}};
    V3 w{0, 0, 0};
    bool inside = uv_barycentrics(tt, V2{p[0], p[1]}, w);
    out[0] = w.x; out[1] = w.y; out[2] = w.z;
    return inside ? 1 : 0;
}
// half_area_x2 of a box; empty != 0 takes Aabb::EMPTY instead of (mn, mx).
float oracle_box_half_area_x2(const float mn[3], const float mx[3], int empty) {
    return (empty ? Aabb::empty() : Aabb{v3_at(mn), v3_at(mx)}).half_area_x2();
}
// Whether the box of two corner points overlaps the box around a sphere.
int oracle_box_sphere_overlap(const float a[3], const float b[3], const float center[3], float radius) {
    Aabb box = Aabb::empty().grow(v3_at(a)).grow(v3_at(b));
    return box.intersects(Aabb::from_sphere(v3_at(center), radius)) ? 1 : 0;
}
float oracle_triangle_area(const float tri[9]) { return triangle_area(v3_at(tri), v3_at(tri + 3), v3_at(tri + 6)); }
int oracle_approx_eq(const float a[3], const float b[3], float eps) { return approx_eq(v3_at(a), v3_at(b), eps) ? 1 : 0; }

// ---- light_shape.rs helpers (light_shape.rs:22-65) ----
float oracle_light_reach(const dl_light *l) { return Light{l}.shape_reach(); }
uint32_t oracle_light_shadow_bits(const dl_light *l) { return Light{l}.shadow_bits(); }
int oracle_light_may_face(const dl_light *l, const float tri[9], const float normal[3]) {
    V3 v[3] = {v3_at(tri), v3_at(tri + 3), v3_at(tri + 6)};
    return Light{l}.may_face(v, v3_at(normal)) ? 1 : 0;
}

// ---- shadows.rs helpers (shadows.rs:136-160): a region of `w` x `h` levels over `rect` ----
static ShadowRegion region_of(const uint8_t *levels, uint32_t w, uint32_t h, uint32_t bits, const uint32_t rect[4]) {
    ShadowRegion r{Rect{rect[0], rect[1], rect[2], rect[3]}, ShadowGrid(w, h, bits)};
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) r.grid.set(x, y, levels[(size_t)y * w + x]);
    return r;
}
// The padded, dilated grid of `crop`: (crop width + 4) x (crop height + 4) levels into `out`.
void oracle_crop_shadows(const uint8_t *levels, uint32_t w, uint32_t h, uint32_t bits, const uint32_t rect[4],
                         const uint32_t crop[4], uint8_t *out) {
    ShadowGrid g = crop_shadows(region_of(levels, w, h, bits, rect), Rect{crop[0], crop[1], crop[2], crop[3]});
    std::memcpy(out, g.levels.data(), g.levels.size());
}
int oracle_any_light(const uint8_t *levels, uint32_t w, uint32_t h, uint32_t bits, const uint32_t rect[4],
                     const uint32_t query[4]) {
    return any_light(region_of(levels, w, h, bits, rect), Rect{query[0], query[1], query[2], query[3]}) ? 1 : 0;
}

}  // extern "C"
