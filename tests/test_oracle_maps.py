"""The oracle's maps for moving meshes (distance cubes, sun maps, sky probes), pinned to the
reference's own unit tests of src/bake/distance_cubes.rs, src/bake/sun_map.rs and
src/bake/sky_probes.rs. CPU only."""
import ctypes as C
import math

import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import scenes
from oracle import oracle as orc
from oracle.oracle import f32, ptr

from . import fixtures as fx

L = orc.lib()
RES = 64
WORDS = RES * RES * 3  # per light: 6 faces x 64^2 f16 (mirror.rs:123)


def f16_value(cubes, slot, index):
    # distance_cube_value (mirror.rs:127-130)
    packed = int(cubes[slot * WORDS + (index >> 1)])
    return float(np.array([(packed >> ((index & 1) * 16)) & 0xFFFF], np.uint16).view(np.float16)[0])


def test_f16_packing_rounds_to_nearest_even():
    rng = np.random.default_rng(3)
    values = np.concatenate([rng.uniform(0, 70000, 20000), rng.uniform(0, 1e-4, 5000),
                             [0.0, 65504.0, 65519.9, 65520.0, 1e9, 2.0 ** -24, 2.0 ** -25, 3 * 2.0 ** -26,
                              5.960464477539063e-08, 1.0009765625, 1.00048828125, 1.000732421875]]).astype(np.float32)
    with np.errstate(over="ignore"):
        want = values.astype(np.float16).view(np.uint16)
    got = np.array([L.oracle_f16_bits(float(v)) for v in values], np.uint16)
    assert np.array_equal(got, want)


def bake(meshes, lights, **opts):
    o = fx.options(dynamic_geometry=dl.ANGULAR, **opts)
    scene, _, _ = orc.bake(dl.BakeInput(meshes, lights), o)
    return scene


def test_distance_cubes_store_hit_distances_in_texel_order():
    # distance_cubes.rs:119-144: a floor 1 m under two lights of radius 4
    floor = fx.floor(1, (0.0, -1.0, 0.0), 6.0)  # wider than the lights' 4 m reach
    lights = [fx.point_light(7, (0.0, 0.0, 0.0), 4.0), fx.point_light(8, (0.0, 0.0, 0.0), 4.0)]
    scene = bake([floor], lights)
    cubes = scene.distance_cubes
    assert cubes.size == 2 * WORDS
    center = RES // 2
    for face, expected in ((3, 1.0), (2, 4.0), (0, 4.0)):  # -Y, +Y, +X face centres
        index = face * RES * RES + center * RES + center
        for slot in range(2):
            assert abs(f16_value(cubes, slot, index) - expected) < 0.01, (face, slot)
    # a slanted texel of the -Y face: 1 / cos(angle) to the floor
    x, y = 10, 20
    u, v = (x + 0.5) / RES * 2 - 1, (y + 0.5) / RES * 2 - 1
    d = np.array([u, -1.0, v])  # any texel of face 3 points down with |y| = 1 before normalising
    expected = float(np.linalg.norm(d))
    assert abs(f16_value(cubes, 1, 3 * RES * RES + y * RES + x) - expected) < expected * 1e-3


def test_lighting_only_bakes_no_maps():
    floor = fx.floor(1, (0.0, -1.0, 0.0), 5.0)
    o = fx.options()
    scene, _, _ = orc.bake(dl.BakeInput([floor], [fx.point_light(7, (0, 0, 0), 4.0),
                                                  fx.sun_light(9, (0.2, 1.0, 0.1), 0.53),
                                                  fx.sky_light(10)]), o)
    assert scene.distance_cubes.size == 0 and scene.sun_maps == [] and scene.sky_probes is None


def sun_depths(m, world):
    # sun_map.rs:174-182: the stored depth and the depth of `world` itself, in map space
    rows = m.rows.astype(np.float64)
    p = rows[:, :3] @ np.asarray(world, np.float64) + rows[:, 3]
    size = m.resolution
    tx, ty = math.floor(p[0] * size), math.floor(p[1] * size)
    index = ty * size + tx
    word = int(m.texels[index // 2]) >> (16 * (index % 2))
    return (word & 0xFFFF) / 65535.0, p[2]


def overhead_sun(light_id=9):
    rot = scenes.rotation_x(-math.pi / 2)
    return dl.BakeLight(id=light_id, position=(0.0, 0.0, 0.0), radius=1.0, shape=dl.LightShape.sun(rot, 0.53))


def test_sun_maps_store_the_first_surface_along_the_rays():
    # sun_map.rs:199-233
    scene = bake([fx.floor(1, (0, 0, 0), 5.0), fx.cuboid(2, (-1.0, 0.0, -1.0), (1.0, 2.0, 1.0))],
                 [overhead_sun()], sun_map_resolution=64)
    (m,) = scene.sun_maps
    assert (m.resolution, m.texels.size) == (64, 64 * 64 // 2)
    for receiver, shaded in (((0.2, 1.0, -0.3), True), ((0.2, 2.5, -0.3), False), ((3.0, 0.5, 3.0), False),
                             ((3.0, -0.5, 3.0), True)):
        stored, depth = sun_depths(m, receiver)
        assert (depth > stored) == shaded, receiver
    top, _ = sun_depths(m, (0.0, 0.0, 0.0))
    ground, _ = sun_depths(m, (4.0, 0.0, -4.0))
    per_meter = float(np.linalg.norm(m.rows[2, :3]))
    assert abs((ground - top) / per_meter - 2.0) < 0.01


def test_sun_maps_cover_the_scene_across_slanted_rays():
    # sun_map.rs:235-254
    rot = scenes.rotation_arc((0, 0, 1), np.array([1.0, 1.0, 0.5]) / np.linalg.norm([1.0, 1.0, 0.5]))
    low = dl.BakeLight(id=9, position=(0.0, 0.0, 0.0), radius=1.0, shape=dl.LightShape.sun(rot, 0.0))
    scene = bake([fx.floor(1, (10.0, 0.0, 0.0), 2.0)], [low], sun_map_resolution=32)
    (m,) = scene.sun_maps
    for cx, cz in ((8.0, -2.0), (12.0, 2.0), (8.0, 2.0), (12.0, -2.0)):
        world = np.array([cx, 0.0, cz])
        p = m.rows[:, :3].astype(np.float64) @ world + m.rows[:, 3]
        assert np.all((p >= 0.0) & (p <= 1.0)), world
        stored, depth = sun_depths(m, world + np.array([0.0, 0.5, 0.0]))
        assert depth < stored
    stored, depth = sun_depths(m, (10.0, -0.5, 0.0))
    assert depth > stored


def test_empty_scenes_give_a_sun_map_nothing_is_behind():
    # sun_map.rs:244-254
    sun = dl.BakeLight(id=9, position=(0.0, 0.0, 0.0), radius=1.0,
                       shape=dl.LightShape.sun(scenes.rotation_x(-1.0), 0.53))
    scene = bake([], [sun], sun_map_resolution=256)
    (m,) = scene.sun_maps
    assert m.resolution == 1 and m.texels.tolist() == [0xFFFFFFFF]


def probe_grid(mn, mx, spacing):
    origin = np.zeros(3, np.float32)
    out_spacing = C.c_float()
    counts = np.zeros(3, np.uint32)
    L.oracle_probe_grid(ptr(f32(*mn)), ptr(f32(*mx)), spacing, ptr(origin), C.byref(out_spacing), ptr(counts))
    return origin, out_spacing.value, tuple(int(c) for c in counts)


def test_probe_grids_cover_the_bounds_and_stay_within_the_cap():
    # sky_probes.rs:196-214
    origin, spacing, counts = probe_grid((0, 0, 0), (4, 2, 0), 1.0)
    assert counts == (6, 4, 2)
    assert origin.tolist() == [-0.5, -0.5, -0.5]
    last = origin + (np.array(counts, np.float32) - 1) * np.float32(spacing)
    assert last.tolist() == [4.5, 2.5, 0.5]
    origin, spacing, counts = probe_grid((0, 0, 0), (500, 20, 300), 1.0)
    assert counts[0] * counts[1] * counts[2] <= 65536 and spacing > 1.0
    reach = (np.array(counts, np.float32) - 1) * np.float32(spacing)
    assert np.all(reach >= np.array([500, 20, 300], np.float32))


def test_inside_probes_take_their_neighbours_values():
    # sky_probes.rs:215-229
    counts = np.array([4, 1, 1], np.uint32)
    values = np.array([[0.5] * 6, [0] * 6, [0] * 6, [1.0] * 6], np.float32)
    valid = np.array([1, 0, 0, 1], np.uint8)
    L.oracle_fill_inside(ptr(counts), ptr(values), ptr(valid))
    assert valid.tolist() == [1, 1, 1, 1]
    assert values[1].tolist() == [0.5] * 6 and values[2].tolist() == [1.0] * 6
    lost = np.zeros((4, 6), np.float32)
    lost_valid = np.zeros(4, np.uint8)
    L.oracle_fill_inside(ptr(counts), ptr(lost), ptr(lost_valid))
    assert lost_valid.tolist() == [0, 0, 0, 0]


def test_sky_probes_see_open_sky_above_and_none_below_a_floor():
    # a floor under an open sky: probes above it see +Y open and -Y blocked; probes inside a
    # closed box are filled from their neighbours; without any static geometry there are none
    floor = fx.floor(1, (0.0, 0.0, 0.0), 4.0)
    scene = bake([floor], [fx.sky_light(10)], sky_probe_spacing=2.0, sky_samples=32)
    p = scene.sky_probes
    assert p is not None and p.words.size == 2 * p.counts[0] * p.counts[1] * p.counts[2]
    cx, cy, cz = p.counts
    words = p.words.reshape(cz, cy, cx, 2)
    top = words[cz // 2, cy - 1, cx // 2]
    openness = [((int(top[a // 4]) >> (8 * (a % 4))) & 0xFF) for a in range(6)]
    assert openness[2] == 255 and openness[3] < 255
    assert bake([], [fx.sky_light(10)]).sky_probes is None
