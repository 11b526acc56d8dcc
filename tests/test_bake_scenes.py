"""The reference's scene-level bake tests, restated over the word reader (`mirror.py`) with the
reference's own thresholds: analytic shadow footprints under point lights
(src/bake/tests/footprint.rs), parallel sun shadows and penumbrae (sun.rs), sky view factors and
probes (sky.rs), meshes that cast no shadow and decals (shadowless.rs), texels inside boxes, thin
strips and buried islands (coverage.rs), local bounce (bounce.rs), sun and colored bounce
(colored_bounce.rs), determinism and output order (determinism.rs), the word layout (layout.rs),
area light penumbrae against brute force (tests/area_light_bake.rs, without its ECS app), and
the public bake API's file round trip and shader-side reads (tests/bake_api.rs).

Every test runs on two bakers: the oracle on the CPU, and the CUDA library's batched form under
the gpu marker. Passing on the oracle pins the restatement to the reference's analytic answers;
passing on the GPU shows the product meets them too (it also equals the oracle word for word)."""
import math

import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import scenes
from dynlight_gb300.mirror import TriangleView, probe_openness
from oracle import oracle

from . import fixtures as fx
from .golden.cases import digest

Y = np.float32([0, 1, 0])


@pytest.fixture(params=["oracle", pytest.param("cuda", marks=pytest.mark.gpu)])
def baker(request):
    """bake(inp, opts) on the oracle (CPU) or through the CUDA library."""
    if request.param == "oracle":
        return lambda inp, opts, progress=None: oracle.bake(inp, opts, progress=progress)[0]
    return lambda inp, opts, progress=None: dl.bake(inp, opts, progress)


def mesh_of(baked, mesh_id):
    return next(m for m in baked.meshes if m.id == mesh_id)


def view(baked, mesh_id, triangle):
    return TriangleView.load(mesh_of(baked, mesh_id).triangles, triangle, baked.settings["bounce"])


def slab(point, direction, lo, hi, t_max):
    """Whether the ray point + t * direction, 0 <= t <= t_max, passes through the box."""
    t0, t1 = 0.0, t_max
    for a in range(3):
        o, d = float(point[a]), float(direction[a])
        if abs(d) < 1e-9:
            if o < lo[a] or o > hi[a]:
                return False
            continue
        u, v = (lo[a] - o) / d, (hi[a] - o) / d
        t0, t1 = max(t0, min(u, v)), min(t1, max(u, v))
    return t0 <= t1


def neighbours(position, texel):
    return [np.float32(position) + np.float32([dx, 0, dz]) * np.float32(texel)
            for dx in (-1.0, 0.0, 1.0) for dz in (-1.0, 0.0, 1.0)]


# ---- footprint.rs: a box between a floor and a point light -----------------------------------

BOX_MIN, BOX_MAX = (-0.5, 0.5, -0.5), (0.5, 1.0, 0.5)


def footprint_scene(light):
    return dl.BakeInput([fx.floor(1, (0, 0, 0), 2.0), fx.cuboid(2, BOX_MIN, BOX_MAX)],
                        [fx.point_light(10, light, 10.0)])


def check_floor(baked, light):
    """footprint.rs:57-99: every floor texel against the segment-to-light slab test, skipping
    texels whose 3x3 neighbourhood straddles the shadow edge; (ambiguous, lit, shadowed)."""
    floor = fx.floor(1, (0, 0, 0), 2.0)
    size = mesh_of(baked, 1).resolution
    texel = 4.0 / size
    light = np.float32(light)
    ambiguous = lit = shadowed = 0
    for t in range(2):
        v = view(baked, 1, t)
        entry = v.entry_for(0)
        for x, y, p in fx.triangle_texels(floor, t, size, face=Y):
            expected = not slab(p, light - p, BOX_MIN, BOX_MAX, 1.0)
            if any((not slab(q, light - q, BOX_MIN, BOX_MAX, 1.0)) != expected for q in neighbours(p, texel)):
                ambiguous += 1
                continue
            actual = entry is not None and v.shadow_bit(entry, x, y) is True
            assert actual == expected, (x, y, p)
            lit, shadowed = lit + expected, shadowed + (not expected)
    return ambiguous, lit, shadowed


def test_shadow_under_a_box_matches_the_projection(baker):
    light = (0.0, 3.0, 0.0)
    baked = baker(footprint_scene(light), fx.options(pixel_density=16.0))
    assert baked.meshes[0].resolution == 64
    ambiguous, lit, shadowed = check_floor(baked, light)
    side = 1.5 * 16.0  # the box's top face projected from the light: a 1.5 m square
    assert (side - 2) ** 2 < shadowed <= side * side
    assert lit > 3000 and ambiguous < 4 * 26 * 3


def test_off_center_light_casts_a_skewed_shadow(baker):
    light = (1.2, 2.5, -0.7)
    _, lit, shadowed = check_floor(baker(footprint_scene(light), fx.options(pixel_density=16.0)), light)
    assert shadowed > 300 and lit > 3000


def test_texels_beyond_the_radius_get_no_light(baker):
    inp = footprint_scene((0.0, 0.5, 0.0))
    inp.meshes = inp.meshes[:1]
    inp.lights[0].radius = 1.0
    baked = baker(inp, fx.options(pixel_density=16.0))
    for t in range(2):
        v = view(baked, 1, t)
        assert v.shadow_bit(v.light(0), 56, 56) is False  # 1.53 m out, past the 1 m radius
        assert v.shadow_bit(v.light(0), 31, 31) is True   # right under the light


def test_walls_facing_away_lose_the_light(baker):
    inp = dl.BakeInput([fx.floor(1, (0, 0, 0), 1.0), fx.floor(3, (0, 5, 0), 1.0)],
                       [fx.point_light(10, (0.0, 3.0, 0.0), 10.0)])
    baked = baker(inp, fx.options(pixel_density=16.0))
    assert view(baked, 1, 0).light_count == 1
    assert view(baked, 3, 0).light_count == 0
    assert baked.stats["lights_removed"] == 0


# ---- sun.rs -----------------------------------------------------------------------------------

def bake_sun(baker, toward, degrees, lo, hi):
    inp = dl.BakeInput([fx.floor(1, (0, 0, 0), 2.0), fx.cuboid(2, lo, hi)], [fx.sun_light(10, toward, degrees)])
    return baker(inp, fx.options(pixel_density=16.0, sun_map_resolution=64))


def floor_values(baked, floor, mesh_id=1, slot=0):
    """[(position, value or None)] over the floor's texels for baked light `slot`."""
    bits = baked.lights[slot].shadow_bits_per_texel
    size = mesh_of(baked, mesh_id).resolution
    out = []
    for t in range(2):
        v = view(baked, mesh_id, t)
        entry = v.entry_for(slot)
        for x, y, p in fx.triangle_texels(floor, t, size, face=Y):
            out.append((p, None if entry is None else v.shadow_value(entry, x, y, bits)))
    return out


def test_hard_sun_shadows_are_the_parallel_projection(baker):
    lo, hi = (-0.5, 0.5, -0.5), (0.5, 1.0, 0.5)
    toward = np.float32([0.4, 1.0, -0.3])
    toward = toward / np.float32(np.linalg.norm(toward))
    baked = bake_sun(baker, toward, 0.0, lo, hi)
    assert baked.lights[0].shadow_bits_per_texel == 1
    texel = 4.0 / baked.meshes[0].resolution
    lit = shadowed = 0
    for p, value in floor_values(baked, fx.floor(1, (0, 0, 0), 2.0)):
        expected = not slab(p, toward, lo, hi, math.inf)
        if any(slab(q, toward, lo, hi, math.inf) == expected for q in neighbours(p, texel)):
            continue
        assert value is not None, "every floor texel sees the sun"
        assert (value == 1.0) == expected, p
        lit, shadowed = lit + expected, shadowed + (not expected)
    # the box along the sun covers 1.35 m^2 = 345 texels, less the skipped edge texels
    assert 200 < shadowed < 346 and lit > 3000


def penumbra_texels(baker, degrees, height):
    lo = (-0.5, height, -0.5)
    baked = bake_sun(baker, (0, 1, 0), degrees, lo, (0.5, height + 0.2, 0.5))
    return sum(1 for _, v in floor_values(baked, fx.floor(1, (0, 0, 0), 2.0)) if v is not None and 0.0 < v < 1.0)


def test_penumbras_widen_with_the_disk_and_the_blocker_height(baker):
    assert penumbra_texels(baker, 0.0, 1.0) == 0, "a sun without a disk is hard"
    narrow, wide, high = (penumbra_texels(baker, 4.0, 1.0), penumbra_texels(baker, 10.0, 1.0),
                          penumbra_texels(baker, 10.0, 1.6))
    assert 0 < narrow < wide < high
    assert wide < 4 * 18 * 4  # each edge of the 1 m square spread over under 3 texels


def test_suns_skip_the_light_bvh_and_distance_cubes(baker):
    inp = dl.BakeInput([fx.floor(1, (0, 0, 0), 2.0), fx.floor(3, (0, 3, 0), 0.5)],
                       [fx.sun_light(5, (0.2, 1.0, 0.1), 0.53), fx.point_light(9, (0.0, 1.0, 0.0), 2.0)])
    baked = baker(inp, fx.options(pixel_density=16.0, sun_map_resolution=64, dynamic_geometry=dl.ANGULAR))
    assert [l.id for l in baked.lights] == [9, 5], "suns come last whatever their id"
    assert baked.light_bvh[0][7] == 1, "the BVH holds the point light only"
    assert baked.distance_cubes.size == 12_288 and len(baked.sun_maps) == 1
    assert baked.lights[1].bounce_bits == 0 and not baked.settings["bounce"]
    roof = view(baked, 3, 0)
    assert [e.light_index for e in roof.entries()] == [1]


def test_lighting_only_bakes_no_sun_maps(baker):
    baked = bake_sun(baker, (0, 1, 0), 0.53, (1, 1, 1), (1.5, 1.5, 1.5))
    assert baked.sun_maps == [] and baked.distance_cubes.size == 0


# ---- sky.rs -----------------------------------------------------------------------------------

def bake_sky(baker, meshes, **kw):
    return baker(dl.BakeInput(meshes, [fx.sky_light(10)]), fx.options(pixel_density=8.0, **kw))


def test_roofed_floors_see_almost_no_sky_and_open_floors_all_of_it(baker):
    roofed, open_, enclosed = (fx.floor(1, (0, 0, 0), 2.0), fx.floor(2, (0, 30, 0), 1.0),
                               fx.floor(3, (0, 10, 0), 0.25))
    meshes = [roofed, open_, enclosed, fx.cuboid(4, (-1.5, 0.1, -1.5), (1.5, 0.2, 1.5)),
              fx.cuboid(5, (-1.0, 9.0, -1.0), (1.0, 11.0, 1.0))]
    baked = bake_sky(baker, meshes, sky_samples=64)
    assert baked.lights[0].shadow_bits_per_texel == 8
    under = [v for p, v in floor_values(baked, roofed, 1) if abs(p[0]) < 0.5 and abs(p[2]) < 0.5]
    assert under and all(v is not None for v in under), "some sky reaches under the roof"
    assert all(v < 0.035 for v in under) and sum(under) / len(under) < 0.015
    assert all(v == 1.0 for _, v in floor_values(baked, open_, 2))
    assert all(v is None for _, v in floor_values(baked, enclosed, 3)), "dropped"
    assert baked.stats["lights_removed"] >= 2


def test_a_long_wall_hides_the_analytic_share_of_the_sky(baker):
    # beside an endless wall of height h a floor point d away sees 1/2 (1 + d / sqrt(d^2 + h^2))
    ground = fx.floor(1, (-2.0, 0.0, 0.0), 2.0)
    baked = bake_sky(baker, [ground, fx.cuboid(2, (0.0, 0.0, -20.0), (0.1, 1.0, 20.0))], sky_samples=256)
    columns = {}
    for p, value in floor_values(baked, ground):
        d = -float(p[0])
        if abs(p[2]) > 1.5 or d < 0.2:
            continue
        expected = 0.5 * (1.0 + d / math.sqrt(d * d + 1.0))
        assert value is not None and abs(value - expected) < 0.06, (d, value, expected)
        c = columns.setdefault(int(d * 1000.0), [0.0, 0.0, 0])
        c[0], c[1], c[2] = c[0] + value, c[1] + expected, c[2] + 1
    assert len(columns) > 20
    for d, (value, expected, n) in columns.items():
        assert abs(value / n - expected / n) < 0.02, d


def test_sky_probes_see_the_roof_and_fill_from_above_under_the_floor(baker):
    meshes = [fx.floor(1, (0, 0, 0), 3.0), fx.cuboid(2, (-1.0, 1.4, -1.0), (1.0, 1.6, 1.0))]
    baked = bake_sky(baker, meshes, dynamic_geometry=dl.ANGULAR, sky_probe_spacing=1.0, sky_samples=1024)
    p = baked.sky_probes
    assert p is not None and tuple(p.counts) == (8, 4, 8)
    assert np.array_equal(np.float32(p.origin), np.float32([-3.5, -0.7, -3.5]))
    assert all(probe_openness(p, x, 3, z)[2] == 1.0 for x in range(8) for z in range(8)), "above everything"
    # 0.3 m over the floor, 1.1 m under the roof: the roof's four parts fill a view factor of 0.411
    _, _, up, down, _, _ = probe_openness(p, 3, 1, 3)
    assert abs(up - 0.589) < 0.01 and down < 0.05
    assert probe_openness(p, 3, 0, 3) == probe_openness(p, 3, 1, 3), "filled from the probe above"
    assert bake_sky(baker, meshes, sky_samples=16).sky_probes is None
    assert bake_sky(baker, [], dynamic_geometry=dl.ANGULAR, sky_probe_spacing=1.0,
                    sky_samples=1024).sky_probes is None, "nothing to shade"


# ---- shadowless.rs ----------------------------------------------------------------------------

def shadowless_scene(occludes):
    point = fx.point_light(10, (0.0, 3.0, 0.0), 8.0, illumination=dl.SINGLE_BOUNCE, bounce=dl.BakeBounce(samples=8))
    area = fx.area_light(11, (1.0, 2.5, 0.5), 8.0, scenes.rotation_x(-math.pi / 2), (0.5, 0.5))
    meshes = [fx.floor(1, (0, 0, 0), 2.0)]
    if occludes is not None:
        block = fx.cuboid(2, (-0.5, 0.5, -0.5), (0.5, 1.0, 0.5))
        block.occludes = occludes
        meshes.append(block)
    return dl.BakeInput(meshes, [point, area, fx.sun_light(12, (0.3, 1.0, 0.2), 1.0), fx.sky_light(13)])


SHADOWLESS_OPTIONS = dict(pixel_density=8.0, dynamic_geometry=dl.ANGULAR, photon_cube_resolution=32,
                          sun_map_resolution=64, sky_samples=64)


def test_meshes_that_cast_no_shadows_are_traced_through(baker):
    open_, silent, solid = (baker(shadowless_scene(o), fx.options(**SHADOWLESS_OPTIONS)) for o in (None, False, True))
    a, b, c = mesh_of(silent, 1), mesh_of(open_, 1), mesh_of(solid, 1)
    assert a.resolution == b.resolution and np.array_equal(a.triangles, b.triangles), "the floor, bounce included"
    assert not np.array_equal(c.triangles, b.triangles)
    assert np.array_equal(silent.distance_cubes, open_.distance_cubes)
    assert not np.array_equal(solid.distance_cubes, open_.distance_cubes)
    assert all(np.array_equal(x.texels, y.texels) for x, y in zip(silent.sun_maps, open_.sun_maps))
    assert not all(np.array_equal(x.texels, y.texels) for x, y in zip(solid.sun_maps, open_.sun_maps))
    assert open_.sky_probes is not None and silent.maps_equal(open_)
    assert not mesh_of(silent, 2).occludes and mesh_of(solid, 2).occludes


def test_meshes_that_cast_no_shadows_still_receive_light(baker):
    silent = baker(shadowless_scene(False), fx.options(**SHADOWLESS_OPTIONS))
    assert view(silent, 2, 4).light_count > 0  # the top face, under the point light


@pytest.mark.parametrize("gap", [0.01, 0.001, 0.0002])
def test_decals_just_above_a_surface_are_lit(baker, gap):
    inp = dl.BakeInput([fx.floor(1, (0, 0, 0), 2.0), fx.floor(2, (0, gap, 0), 0.25)],
                       [fx.point_light(10, (0.7, 2.0, 0.3), 8.0)])
    baked = baker(inp, fx.options(pixel_density=32.0))
    lit, dark = count_bits(baked, 2, range(2))
    assert lit > 0 and dark == 0, (gap, lit, dark)


def count_bits(baked, mesh_id, triangles, inside=None):
    """(lit, dark) one-bit texels of light entry 0 over the whole map of each triangle, limited
    to texels where inside(x, y) holds when given."""
    size = mesh_of(baked, mesh_id).resolution
    lit = dark = 0
    for t in triangles:
        v = view(baked, mesh_id, t)
        e = v.light(0)
        for y in range(size):
            for x in range(size):
                if inside is not None and not inside(x, y):
                    continue
                b = v.shadow_bit(e, x, y)
                lit, dark = lit + (b is True), dark + (b is False)
    return lit, dark


# ---- coverage.rs ------------------------------------------------------------------------------

def floor_through_box(baker, bottom):
    inp = dl.BakeInput([fx.floor(1, (0, 0, 0), 1.0), fx.cuboid(2, (-0.25, bottom, -0.25), (0.25, 0.25, 0.25))],
                       [fx.point_light(10, (3.0, 1.5, 0.0), 8.0)])
    baked = baker(inp, fx.options(pixel_density=16.0))
    size = mesh_of(baked, 1).resolution
    texel = np.float32(2.0) / np.float32(size)

    def inside(x, y):
        # floor texel centers at the box's +X side within 1.5 texels inside the box
        at = ((np.float32([x, y]) + np.float32(0.5)) / np.float32(size)) * np.float32(2.0) - np.float32(1.0)
        return at[0] < 0.25 and at[0] > np.float32(0.25) - np.float32(1.5) * texel and abs(at[1]) < np.float32(0.25 * 0.6)
    return count_bits(baked, 1, range(2), inside)


@pytest.mark.parametrize("bottom", [-0.25, 0.0])
def test_texels_inside_a_box_take_their_visible_neighbours_light(baker, bottom):
    lit, dark = floor_through_box(baker, bottom)
    assert lit > 0 and dark == 0, (lit, dark)


def test_strips_narrower_than_a_texel_are_lit(baker):
    # six 0.1 m strips whose UV islands are 0.4 texels wide and 3 texels apart
    strips, density = 6, 32.0
    size = oracle.lib().oracle_lightmap_size(C_float(strips * 0.1), C_float(density), 2048)
    pos, uv1, idx = [], [], []
    for k in range(strips):
        x = np.float32(k) * np.float32(0.1) - np.float32(0.3)
        u = (np.float32(3.0) * np.float32(k) + np.float32(0.55)) / np.float32(size)
        du = np.float32(0.4) / np.float32(size)
        base = len(pos)
        for a, b in [(0.0, -0.5), (0.1, -0.5), (0.1, 0.5), (0.0, 0.5)]:
            pos.append([x + np.float32(a), 0.0, b])
            uv1.append([u + np.float32(a) * np.float32(10.0) * du, np.float32(0.5) + np.float32(b) * np.float32(0.9)])
        idx += [base, base + 2, base + 1, base, base + 3, base + 2]
    pos, uv1 = np.float32(pos), np.float32(uv1)
    mesh = dl.BakeMesh(id=1, positions=pos, indices=np.uint32(idx), uv1=uv1, normals=np.tile(Y, (len(pos), 1)))
    baked = baker(dl.BakeInput([mesh], [fx.point_light(10, (0.2, 1.5, 0.1), 8.0)]), fx.options(pixel_density=density))
    assert baked.meshes[0].resolution == size
    for t in range(2 * strips):
        v = view(baked, 1, t)
        assert v.light_count == 1, t
        c = uv1[idx[3 * t]] + uv1[idx[3 * t + 1]] + uv1[idx[3 * t + 2]]
        tx, ty = np.floor(c / np.float32(3.0) * np.float32(size))
        assert v.shadow_bit(v.light(0), int(tx), int(ty)) is True, t


def test_a_buried_island_leaves_an_overlapping_one_lit(baker):
    # one mesh whose UV islands overlap: a lit floor and a quad shut inside a box below it
    top, hidden = fx.floor(1, (0, 0, 0), 0.5), fx.floor(1, (0, -0.75, 0), 0.25)
    both = dl.BakeMesh(id=1, positions=np.concatenate([top.positions, hidden.positions]),
                       indices=np.concatenate([top.indices, hidden.indices + 4]).astype(np.uint32),
                       uv1=np.concatenate([top.uv1, hidden.uv1]), normals=np.concatenate([top.normals, hidden.normals]))
    inp = dl.BakeInput([both, fx.cuboid(2, (-0.4, -1.0, -0.4), (0.4, -0.5, 0.4))],
                       [fx.point_light(10, (0.1, 1.5, 0.2), 8.0)])
    lit, dark = count_bits(baker(inp, fx.options(pixel_density=16.0)), 1, range(2))
    assert lit > 0 and dark == 0, (lit, dark)


def C_float(x):
    import ctypes
    return ctypes.c_float(x)


# ---- bounce.rs --------------------------------------------------------------------------------

def bounce_box_input(floor_albedo=(1.0, 1.0, 1.0)):
    light = fx.point_light(10, (0.0, 1.5, 0.0), 5.0, illumination=dl.SINGLE_BOUNCE, bounce=dl.BakeBounce(samples=12))
    ground = fx.floor(1, (0, 0, 0), 3.0)
    ground.albedo = floor_albedo
    return dl.BakeInput([ground, fx.cuboid(2, (1.0, 0.0, -0.5), (1.5, 1.0, 0.5))], [light])


def bounce_options(skip_bounce=False, compression=6, colored=False):
    return fx.options(pixel_density=8.0, photon_cube_resolution=48, skip_bounce=skip_bounce,
                      bounce_compression=compression, colored_bounce=colored)


def bounce_values(baked, mesh, triangle, bits, slot=0, require=False):
    """Decoded (squared) bounce over the triangle's texels for light `slot`: RGB triples, white
    ones repeated when the bake is not colored; None when the triangle has no entry."""
    v = TriangleView.load(mesh_of(baked, mesh.id).triangles, triangle, baked.settings["bounce"])
    entry = v.entry_for(slot)
    if entry is None:
        assert not require, "the light reaches the triangle"
        return None
    texels = fx.triangle_texels(mesh, triangle, mesh_of(baked, mesh.id).resolution)
    assert texels
    if entry.bounce_offset == 0:
        return [(0.0, 0.0, 0.0)] * len(texels)
    out = []
    for x, y, _ in texels:
        if baked.settings["colored_bounce"]:
            s = v.bounce_texel_rgb(entry, x, y, bits)
        else:
            s = (v.bounce_texel(entry, x, y, bits),) * 3
        out.append(tuple(float(np.float32(c) * np.float32(c)) for c in s))
    return out


def test_the_floor_bounces_onto_the_far_side_of_the_box(baker):
    inp = bounce_box_input()
    baked = baker(inp, bounce_options())
    assert baked.settings["bounce"] and baked.lights[0].bounce_bits == 6 and baked.stats["bounce_rays"] > 0
    cube, floor = inp.meshes[1], inp.meshes[0]
    for t in range(2):  # cuboid face 0 (+X) faces away from the light: bounce alone reaches it
        entry = view(baked, 2, t).entry_for(0)
        assert entry is not None and entry.bounce_offset != 0
        values = [c[0] for c in bounce_values(baked, cube, t, 6)]
        assert sum(1 for c in values if c > 0) * 2 > len(values)
        assert all(0.0 <= c <= 1.0 for c in values)
    assert any(c[0] > 0 for c in bounce_values(baked, cube, 2, 6)), "the -X face receives bounce too"
    floor_values_ = [c[0] for t in range(2) for c in (bounce_values(baked, floor, t, 6) or [])]
    assert any(c > 0 for c in floor_values_), "the floor gets light bounced off the box"


def test_preview_skips_bounce(baker):
    baked = baker(bounce_box_input(), bounce_options(skip_bounce=True))
    assert not baked.settings["bounce"] and baked.lights[0].bounce_bits == 0 and baked.stats["bounce_rays"] == 0
    for t in range(2):
        assert view(baked, 2, t).light_count == 0, "no direct light reaches the far side"


# ---- colored_bounce.rs ------------------------------------------------------------------------

RED = (0.8, 0.1, 0.0)


def sun_wall_input(floor_albedo):
    sun = fx.sun_light(10, (0, 1, 0), 0.0, illumination=dl.SINGLE_BOUNCE, bounce=dl.BakeBounce(samples=64))
    ground = fx.floor(1, (0, 0, 0), 10.0)
    ground.albedo = floor_albedo
    return dl.BakeInput([ground, fx.cuboid(2, (-0.02, 0.0, -0.5), (0.0, 1.0, 0.5))], [sun])


def mean(values):
    return np.mean(np.float64(values), axis=0)


def wall_bounce(baked, inp):
    return [c for t in range(2) for c in bounce_values(baked, inp.meshes[1], t, 8, require=True)]


def test_a_sunlit_floor_bounces_onto_a_wall_by_its_view_factor(baker):
    inp = sun_wall_input((1.0, 1.0, 1.0))
    baked = baker(inp, bounce_options(compression=8))
    assert baked.settings["bounce"] and not baked.settings["colored_bounce"]
    assert baked.lights[0].bounce_bits == 8
    values = wall_bounce(baked, inp)
    # h up a wall, a floor reaching 10 m out fills about 1/2 (1 - h / sqrt(h^2 + L^2)) = 0.48
    assert 0.40 <= mean(values)[0] < 0.50
    assert all(c[0] > 0.3 for c in values), "every texel sees the floor"
    ground = bounce_values(baked, inp.meshes[0], 0, 8, require=True)
    assert mean(ground)[0] < 0.01


def test_colored_sun_bounce_takes_the_floor_color(baker):
    red_in = sun_wall_input(RED)
    colored = mean(wall_bounce(baker(red_in, bounce_options(compression=8, colored=True)), red_in))
    white_in = sun_wall_input((1.0, 1.0, 1.0))
    white = mean(wall_bounce(baker(white_in, bounce_options(compression=8)), white_in))
    assert np.all(np.abs(colored - np.float64(RED) * white[0]) <= 0.01), (colored, white)


def test_photons_carry_the_color_of_what_they_hit(baker):
    inp = bounce_box_input(RED)
    baked = baker(inp, bounce_options(compression=8, colored=True))
    values = [c for t in range(2) for c in bounce_values(baked, inp.meshes[1], t, 8, require=True)]
    lit = [c for c in values if c[0] > 0.0]
    assert len(lit) * 2 > len(values)
    for r, g, b in lit:  # blue stays 0; green follows red at an eighth, within a step
        assert b == 0.0 and abs(g - r / 8.0) < 0.01


def test_white_bounce_ignores_colors(baker):
    opts = bounce_options(compression=8)
    assert digest(baker(sun_wall_input(RED), opts)) == digest(baker(sun_wall_input((1.0, 1.0, 1.0)), opts))


@pytest.mark.parametrize("scene", ["bounce", "colored"])
def test_bounce_bakes_are_identical_on_any_thread_count(scene):
    # bounce.rs:113-126 and colored_bounce.rs:171-184 (the oracle's thread pool)
    if scene == "bounce":
        inp, opts = bounce_box_input(), bounce_options()
    else:
        inp, opts = sun_wall_input(RED), bounce_options(compression=8, colored=True)
    single = digest(oracle.bake(inp, opts, threads=1)[0])
    assert single == digest(oracle.bake(inp, opts, threads=3)[0]) == digest(oracle.bake(inp, opts, threads=8)[0])


# ---- determinism.rs ---------------------------------------------------------------------------

def determinism_options():
    return fx.options(pixel_density=12.0, dynamic_geometry=dl.ANGULAR, sun_map_resolution=64, sky_samples=16,
                      sky_probe_spacing=0.75)


def test_bakes_are_identical_on_any_thread_count():
    inp, _ = fx.determinism_room()
    opts = determinism_options()
    single = digest(oracle.bake(inp, opts, threads=1)[0])
    for threads in (1, 4, 7):
        assert digest(oracle.bake(inp, opts, threads=threads)[0]) == single, threads


def test_input_order_does_not_matter(baker):
    inp, _ = fx.determinism_room()
    shuffled = dl.BakeInput(list(reversed(inp.meshes)), inp.lights[2:] + inp.lights[:2])
    assert digest(baker(inp, determinism_options())) == digest(baker(shuffled, determinism_options()))


def test_outputs_are_sorted_and_lights_follow_the_bvh(baker):
    inp, _ = fx.determinism_room()
    baked = baker(inp, determinism_options())
    assert [m.id for m in baked.meshes] == [3, 4, 5, 9]
    assert len(baked.lights) == 10
    assert [l.id for l in baked.lights[7:]] == [15, 25, 12], "suns by id, then the sky"
    kinds = [l.shape for l in baked.lights]
    assert sum(k not in (dl.SUN, dl.SKY) for k in kinds) == 7
    assert (sum(k == dl.SUN for k in kinds), sum(k in (dl.SUN, dl.SKY) for k in kinds)) == (2, 3)
    assert baked.lights[9].shadow_bits_per_texel == 8 and baked.sky_probes is not None
    for node in baked.light_bvh:  # every leaf's lights lie inside it
        lo, first, hi, count = node[0:3].view(np.float32), int(node[3]), node[4:7].view(np.float32), int(node[7])
        for light in baked.lights[first:first + count]:
            o, r = np.float32(light.origin), np.float32(light.radius)
            assert np.all(lo <= o - r + np.float32(1e-5)) and np.all(hi >= o + r - np.float32(1e-5))
    assert baked.distance_cubes.size == 7 * 12_288, "no cubes for suns"
    assert len(baked.sun_maps) == 2
    assert sum(l.shadow_bits_per_texel == 4 for l in baked.lights) == 3, "panel, tube and the wide sun"
    assert baked.stats["rays"] > 0 and baked.stats["texels"] > 0 and baked.stats["meshes"] == 4


# ---- layout.rs --------------------------------------------------------------------------------

def mesh_area(mesh):
    """The mesh's surface area summed in binary32 in index order, each triangle's half cross
    product length with the dot product as (x*x + y*y) + z*z (src/bake/mesh_builder.rs:22-27,
    src/bake/geometry.rs:59-61)."""
    area = np.float32(0.0)
    p = mesh.positions.astype(np.float32)
    for a, b, c in mesh.indices.reshape(-1, 3):
        e1, e2 = p[b] - p[a], p[c] - p[a]
        n = (e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0])
        area = area + np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]) * np.float32(0.5)
    return float(area)


def test_baked_words_are_well_formed(baker):
    meshes = [fx.floor(1, (0, 0, 0), 2.0), fx.cuboid(2, (-0.5, 0.0, -0.5), (0.5, 1.0, 0.5))]
    inp = dl.BakeInput(meshes, [fx.point_light(1, (1.0, 2.0, 0.0), 4.0), fx.point_light(2, (-1.0, 0.5, 1.0), 2.0)])
    baked = baker(inp, dl.BakeOptions(pixel_density=10.0))
    L = oracle.lib()
    for mesh, source in zip(baked.meshes, meshes):
        assert mesh.resolution == L.oracle_lightmap_size(mesh_area(source), 10.0, 2048)
        words = mesh.triangles
        assert mesh.triangle_count() == source.triangle_count()
        next_data = None
        for t in range(source.triangle_count()):
            v = TriangleView.load(words, t, baked.settings["bounce"])
            uv = np.ascontiguousarray(source.uv1[source.indices[3 * t: 3 * t + 3]].reshape(-1), np.float32)
            rect = np.zeros(12, np.uint32)
            L.oracle_rects(oracle.ptr(uv), mesh.resolution, oracle.ptr(rect))
            w, h = int(rect[2] - rect[0] + 1), int(rect[3] - rect[1] + 1)
            assert v.bounds == ((int(rect[0]) - 2) & 0xFFFFFFFF, (int(rect[1]) - 2) & 0xFFFFFFFF, w + 4)
            for k in range(v.light_count):
                e = v.light(k)
                assert e.light_index < len(baked.lights) and e.bounce_offset == 0
                if k > 0:
                    assert v.light(k - 1).light_index < e.light_index
                # payloads follow each other without gaps, in triangle and light order
                assert next_data is None or e.shadow_offset == next_data
                next_data = e.shadow_offset + ((w + 4) * (h + 4) + 31) // 32
        assert (len(words) if next_data is None else next_data) == len(words)
    for t in (6, 7):  # the box's bottom face faces away from both lights
        assert view(baked, 2, t).light_count == 0


# ---- tests/area_light_bake.rs (the bake itself, without the ECS app) ---------------------------

LAMP = (0.3, 3.0, 0.2)
AREA_BOX = ((-0.5, 0.5, -0.5), (0.5, 1.5, 0.5))


def area_floor():
    """A 6 m plane with UV1 u along +X and v along +Z, split along u + v = 1; triangle 0 is the
    half where u + v > 1."""
    uv = np.float32([(0, 0), (1, 0), (1, 1), (0, 1)])
    pos = np.float32([((u - 0.5) * 6.0, 0.0, (v - 0.5) * 6.0) for u, v in uv])
    return dl.BakeMesh(id=1, positions=pos, indices=np.uint32([1, 3, 2, 0, 3, 1]), uv1=uv,
                       normals=np.tile(Y, (4, 1)))


def area_bake(baker, light, preview):
    o = fx.options(pixel_density=8.0)
    if preview:  # BakePreset::Preview's options (src/bake/systems.rs:140-156)
        o.skip_bounce, o.area_light_samples, o.area_light_min_samples = True, 32, 0
        o.sun_map_resolution, o.sky_samples = 512, 16
    inp = dl.BakeInput([area_floor(), fx.cuboid(2, *AREA_BOX)], [light])
    return baker(inp, o)


def floor_shadows(baked):
    bits = baked.lights[0].shadow_bits_per_texel
    size = mesh_of(baked, 1).resolution
    values = np.zeros((size, size), np.float32)
    views = [view(baked, 1, 0), view(baked, 1, 1)]
    for y in range(size):
        for x in range(size):
            v = views[0 if x + y + 1 > size else 1]
            values[y, x] = next((s for s in (v.shadow_value(e, x, y, bits) for e in v.entries()) if s is not None), 0.0)
    return size, values


def brute_force_panel(world, half):
    """The share of a downward panel's light reaching `world`, over a 48x48 grid of panel
    points weighted by both cosines over distance squared."""
    steps = 48
    g = (np.arange(steps, dtype=np.float64) + 0.5) / steps * 2.0 - 1.0
    px, pz = np.meshgrid(LAMP[0] + g * half, LAMP[2] + g * half)
    d = np.stack([px - world[0], np.full_like(px, LAMP[1] - world[1]), pz - world[2]], -1)
    length2 = (d * d).sum(-1)
    weight = (d[..., 1] ** 2 / length2) / length2
    lo, hi = np.float64(AREA_BOX[0]), np.float64(AREA_BOX[1])
    inv = 1.0 / np.where(np.abs(d) < 1e-9, 1e-30, d)
    a, b = (lo - world) * inv, (hi - world) * inv
    near = np.maximum(np.minimum(a, b).max(-1), 0.0)
    far = np.minimum(np.maximum(a, b).min(-1), 1.0)
    blocked = near <= far
    return float(weight[~blocked].sum() / weight.sum())


def test_panels_bake_their_shape_with_soft_shadows(baker):
    down = scenes.rotation_x(-math.pi / 2)
    panel = fx.area_light(7, LAMP, 6.0, down, (1.5, 1.5))
    baked = area_bake(baker, panel, preview=False)
    assert len(baked.lights) == 1
    light = baked.lights[0]
    assert np.array_equal(np.float32(light.origin), np.float32(LAMP)) and light.radius == 6.0
    assert light.shadow_bits_per_texel == 4 and light.shape == dl.RECTANGLE
    assert np.allclose(light.rotation, down, atol=1e-6) and tuple(light.size[:2]) == (1.5, 1.5)
    size, values = floor_shadows(baked)
    errors = []
    for y in range(size):
        for x in range(size):
            u, v = (x + 0.5) / size, (y + 0.5) / size
            world = np.float64([(u - 0.5) * 6.0, 0.0, (v - 0.5) * 6.0])
            errors.append(abs(float(values[y, x]) - brute_force_panel(world, 0.75)))
    assert np.mean(errors) < 0.02 and max(errors) < 0.2, (np.mean(errors), max(errors))
    levels = set(np.rint(values * 15.0).astype(int).ravel().tolist())
    assert 0 in levels and 15 in levels and len(levels) >= 12, levels


def penumbra_across(values):
    """Texels strictly between shadow and light along the darkest row and column."""
    row = values[int(np.argmin(values.sum(axis=1)))]
    column = values[:, int(np.argmin(values.sum(axis=0)))]
    soft = lambda line: int(np.sum((line > 0.05) & (line < 0.95)))  # noqa: E731
    return soft(row), soft(column)


def test_tubes_soften_shadows_only_along_their_length(baker):
    along_x = area_bake(baker, fx.area_light(7, LAMP, 6.0, (0.0, 0.0, 0.0, 1.0), (1.0, 0.0)), preview=True)
    along_z = area_bake(baker, fx.area_light(7, LAMP, 6.0, scenes.rotation_y(math.pi / 2), (1.0, 0.0)), preview=True)
    assert along_x.lights[0].shape == dl.TUBE
    row, column = penumbra_across(floor_shadows(along_x)[1])
    assert row >= 6 and column <= 1, (row, column)
    row, column = penumbra_across(floor_shadows(along_z)[1])
    assert column >= 6 and row <= 1, (row, column)


def test_point_lights_keep_one_shadow_bit(baker):
    baked = area_bake(baker, fx.point_light(7, LAMP, 6.0), preview=True)
    assert baked.lights[0].shadow_bits_per_texel == 1 and baked.lights[0].shape == dl.POINT
    assert baked.stats["rays"] > 0 and baked.stats["texels"] > 0
    values = floor_shadows(baked)[1]
    assert np.all((values == 0.0) | (values == 1.0)) and np.any(values == 0.0), "the box casts a shadow"


# ---- tests/bake_api.rs: bake, write and read the file, read the result like the runtime -------

def api_input():
    floor = dl.BakeMesh(id=7, positions=np.float32([[-2, 0, -2], [2, 0, -2], [2, 0, 2], [-2, 0, 2]]),
                        indices=np.uint32([0, 2, 1, 0, 3, 2]), uv1=np.float32([[0, 0], [1, 0], [1, 1], [0, 1]]),
                        normals=np.tile(Y, (4, 1)))
    return dl.BakeInput([floor], [fx.point_light(2, (1.0, 1.0, 0.0), 3.0), fx.point_light(1, (-1.0, 1.0, 0.0), 3.0)])


def test_bake_encode_decode_round_trip(baker):
    from dynlight_gb300 import dynlight_file as f
    progress = dl.BakeProgress()
    scene = baker(api_input(), dl.BakeOptions(pixel_density=4.0, dynamic_geometry=dl.ANGULAR), progress)
    assert progress.stage == 4 and progress.fraction() == 1.0  # BakeStage::Done
    data = f.encode(scene)
    assert data[:8] == b"DYNLIGHT" and data[8:12] == (6).to_bytes(4, "little")
    back = f.decode(data)
    assert digest(back) == digest(scene)
    assert f.encode(back) == data, "encoding is canonical"
    future = bytearray(data)
    future[8:12] = (7).to_bytes(4, "little")
    with pytest.raises(f.FormatError) as e:
        f.decode(bytes(future))
    assert e.value == f.FormatError("UnsupportedVersion", found=7) and "re-bake" in str(e.value)


def cube_index(direction, res=64):
    """texel_index(direction_to_texel(d)) (src/shared/cube.rs:94-96) through the oracle."""
    out = np.zeros(3, np.uint32)
    oracle.lib().oracle_cube_texel(oracle.ptr(np.float32(direction)), res, oracle.ptr(out))
    face, x, y = (int(v) for v in out)
    return face * res * res + y * res + x


def test_baked_scene_reads_like_the_shader(baker):
    from dynlight_gb300.mirror import DISTANCE_CUBE_WORDS, distance_cube_value
    scene = baker(api_input(), dl.BakeOptions(pixel_density=4.0, dynamic_geometry=dl.ANGULAR))
    assert scene.light_bvh.shape == (1, 8) and scene.light_bvh[0][7] == 2, "two lights fit one leaf"
    mesh = scene.meshes[0]
    assert mesh.resolution == 16 and mesh.triangle_count() == 2
    for t in range(2):  # both lights reach both triangles, entries in BVH slot order
        v = TriangleView.load(mesh.triangles, t, False)
        assert v.light_count == 2
        for k in range(2):
            assert v.light(k).light_index == k
            assert v.shadow_bit(v.light(k), 8, 8) is True, "nothing blocks the floor"
    # angular distance cubes: exact distances, the floor 1 m below each light; misses store the radius
    assert scene.distance_cubes.size == 2 * DISTANCE_CUBE_WORDS
    for slot in range(2):
        assert abs(distance_cube_value(scene.distance_cubes, slot, cube_index((0, -1, 0))) - 1.0) < 0.01
        assert distance_cube_value(scene.distance_cubes, slot, cube_index((0, 1, 0))) == 3.0
