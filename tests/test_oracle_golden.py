"""Pins the oracle (the C++ restatement of the reference baker) to the reference's own
known-answer vectors, one test per reference unit test family. Each cites the reference test it
ports. CPU only."""
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


def test_lightmap_size_table():
    # src/bake/geometry.rs:147-157
    cases = [((1.0, 128.0, 2048), 128), ((4.0, 128.0, 2048), 256), ((2.0, 10.0, 2048), 15),
             ((1e6, 128.0, 2048), 2048), ((0.0, 128.0, 2048), 2), ((1e-9, 128.0, 2048), 2),
             ((float("nan"), 128.0, 2048), 2), ((float("inf"), 128.0, 64), 64),
             ((1.0, 128.0, 1), 2)]
    for args, want in cases:
        assert L.oracle_lightmap_size(*args) == want, args


def rects(uv, size):
    out = (C.c_uint32 * 12)()
    L.oracle_rects(ptr(f32(*uv)), size, out)
    return list(out)


def test_rects_follow_the_reference_bounds():
    # src/bake/mesh_builder.rs:171-193
    r = rects([0.25, 0.25, 0.5, 0.25, 0.25, 0.5], 16)
    assert r[0:4] == [2, 2, 10, 10]
    assert (r[4], r[6]) == (3, 8)
    assert (r[8], r[10]) == (2, 9)
    r = rects([0, 0, 0.05, 0, 0, 0.05], 16)
    assert (r[0], r[1]) == (0, 0)
    r = rects([3, 3, 4, 4, 3, 4], 16)
    assert (r[0], r[2]) == (15, 15)


def texels(mode, v, n, uv, face, size, owned=None, cap=4096):
    xy = np.zeros(cap * 2, np.uint32)
    pos = np.zeros(cap * 3, np.float32)
    nrm = np.zeros(cap * 3, np.float32)
    own = None if owned is None else np.ascontiguousarray(owned, np.uint8)
    count = L.oracle_texels(mode, ptr(f32(*v)), ptr(f32(*n)), ptr(f32(*uv)), ptr(f32(*face)),
                            size, None if own is None else ptr(own), cap, ptr(xy), ptr(pos),
                            ptr(nrm))
    return xy[:2 * count].reshape(-1, 2), pos[:3 * count].reshape(-1, 3), nrm[:3 * count].reshape(-1, 3)


def test_texels_interpolate_position_and_normal():
    # src/bake/texels.rs:147-167
    xy, pos, nrm = texels(0, [0, 0, 0, 4, 0, 0, 0, 0, 4], [0, 1, 0, 0, 2, 0, 0, 1, 1],
                          [0, 0, 1, 0, 0, 1], [0, 1, 0], 4)
    assert len(xy) == 10
    assert tuple(xy[0]) == (0, 0)
    assert np.allclose(pos[0], [0.5, 0.0, 0.5], atol=1e-5)
    assert np.all(np.abs(np.linalg.norm(nrm, axis=1) - 1) < 1e-5)
    assert np.all(xy.sum(axis=1) <= 3)


def test_thin_triangles_touch_texels_whose_centers_they_miss():
    # src/bake/texels.rs:169-196
    uv = [0.30, 0.05, 0.375, 0.05, 0.30, 0.95]
    v = [0.30, 0, 0.05, 0.375, 0, 0.05, 0.30, 0, 0.95]
    n = [0, 1, 0] * 3
    xy, _, _ = texels(0, v, n, uv, [0, 1, 0], 4)
    assert len(xy) == 0
    xy, pos, _ = texels(1, v, n, uv, [0, 1, 0], 4)
    assert [tuple(p) for p in xy] == [(1, 0), (1, 1), (1, 2), (1, 3)]
    for (x, y), p in zip(xy, pos):
        assert 0.30 - 1e-6 <= p[0] <= 0.375 + 1e-6
        assert abs(p[2] - (y + 0.5) / 4.0) < 0.13
    owned = np.zeros((4, 4), np.uint8)
    owned[2, :] = 1
    xy, _, _ = texels(1, v, n, uv, [0, 1, 0], 4, owned=owned)
    assert len(xy) == 3


def test_the_world_origin_is_a_valid_texel_and_opposing_normals_fall_back():
    # src/bake/texels.rs:198-219 (through triangle_texels of a 2-texel map)
    xy, pos, nrm = texels(0, [-1, 0, -1, 1, 0, -1, 0, 0, 0], [0, 1, 0] * 3, [0, 0, 1, 0, 0.5, 1],
                          [0, 1, 0], 2)
    assert len(xy) >= 1
    xy, pos, nrm = texels(0, [0, 0, 0, 1, 0, 0, 0, 0, 1], [0, 1, 0, 0, -1, 0, 0, 0, 0],
                          [0, 0, 1, 0, 0, 1], [0, -1, 0], 64)
    # texels near the (1, 0) edge midpoint interpolate opposite normals towards zero; where the
    # sum is exactly zero the face normal is used
    assert np.all(np.abs(np.linalg.norm(nrm, axis=1) - 1) < 1e-5)


def test_burial_rays_cover_the_hemisphere():
    # src/bake/mesh_texels.rs:169-200
    seen = []

    @orc.DIR_FN
    def always(d, _):
        seen.append((d[0], d[1], d[2]))
        return 1

    rays = C.c_uint32()
    assert L.oracle_is_buried(ptr(f32(0, 1, 0)), C.c_float(0.3), always, C.byref(rays)) == 1
    assert rays.value == 5
    opened = []

    @orc.DIR_FN
    def never(d, _):
        opened.append((d[0], d[1], d[2]))
        return 0

    assert L.oracle_is_buried(ptr(f32(0, 1, 0)), C.c_float(0.3), never, C.byref(rays)) == 0
    assert rays.value == 8 - 5 + 1
    for d in seen + opened:
        assert abs(math.sqrt(sum(x * x for x in d)) - 1) < 1e-5 and d[1] > 0
    count = [0]

    @orc.DIR_FN
    def all_but_second(d, _):
        count[0] += 1
        return int(count[0] != 2)

    assert L.oracle_is_buried(ptr(f32(0, 0, 1)), C.c_float(0.0), all_but_second, C.byref(rays)) == 1
    count[0] = 0

    @orc.DIR_FN
    def every_other(d, _):
        count[0] += 1
        return int(count[0] % 2 == 0)

    assert L.oracle_is_buried(ptr(f32(0, 0, 1)), C.c_float(0.0), every_other, C.byref(rays)) == 0


def pack(levels, w, h, bits):
    lv = np.ascontiguousarray(np.asarray(levels, np.uint8).reshape(-1))
    out = np.zeros(w * h + 1, np.uint32)
    n = L.oracle_pack_levels(ptr(lv), w, h, bits, ptr(out))
    return list(out[:n])


def test_bit_grids_are_lsb_first_row_major():
    # src/bake/bits.rs:140-152
    g = np.zeros((7, 5), np.uint8)
    g[0, 0] = g[0, 1] = g[6, 2] = 1
    assert pack(g, 5, 7, 1) == [0b11, 1]


def test_levels_pack_eight_per_word_and_round():
    # src/bake/shadow_grid.rs:184-193, 221-229
    g = np.zeros((3, 3), np.uint8)
    g[0, 0], g[0, 1], g[2, 2] = 15, 1, 7
    assert pack(g, 3, 3, 4) == [0x1F, 7]
    assert [L.oracle_level(f, b) for f, b in [(0.0, 4), (0.5, 4), (1.2, 4), (0.49, 1), (0.51, 1)]] == \
        [0, 8, 15, 0, 1]


def pad(levels, rect, bits, visited):
    lv = np.ascontiguousarray(np.asarray(levels, np.uint8))
    vis = np.ascontiguousarray(np.asarray(visited, np.uint8))
    L.oracle_pad_seams(ptr(lv), (C.c_uint32 * 4)(*rect), bits, ptr(vis), vis.shape[1], vis.shape[0])
    return lv


def test_seam_padding():
    # src/bake/seams.rs:134-189
    vis = np.zeros((1, 6), np.uint8)
    vis[0, 2] = 1
    out = pad(vis.copy(), (0, 0, 5, 0), 1, vis)
    assert list(out[0] != 0) == [True, True, True, True, True, False]
    vis = np.zeros((4, 4), np.uint8)
    vis[0, 3] = 1
    out = pad(vis.copy(), (0, 0, 3, 3), 1, vis)
    assert not out[1, 0] and out[0, 2] and out[1, 3]
    vis = np.zeros((4, 4), np.uint8)
    vis[1, 0] = 1
    out = pad(vis.copy(), (0, 0, 3, 3), 1, vis)
    assert not out[0, 3]
    vis = np.zeros((3, 3), np.uint8)
    vis[1, 1] = vis[0, 0] = 1
    lv = np.zeros((3, 3), np.uint8)
    lv[1, 1] = 1
    out = pad(lv, (0, 0, 2, 2), 1, vis)
    assert not out[0, 0] and out[0, 1] and out[1, 0]
    vis = np.zeros((1, 3), np.uint8)
    vis[0, 0] = vis[0, 2] = 1
    lv = np.array([[4, 0, 11]], np.uint8)
    assert list(pad(lv, (0, 0, 2, 0), 4, vis)[0]) == [4, 11, 11]


def dilate(levels, bits):
    lv = np.ascontiguousarray(np.asarray(levels, np.uint8))
    L.oracle_dilate(ptr(lv), lv.shape[1], lv.shape[0], bits)
    return lv


def test_dilation():
    # src/bake/seams.rs:190-231
    g = np.zeros((7, 7), np.uint8)
    g[2, 2] = 1
    g = dilate(g, 1)
    for x, y in [(1, 1), (2, 1), (3, 1), (1, 2), (1, 3)]:
        assert g[y, x], (x, y)
    assert not g[1, 4]
    for x, y in [(0, 0), (1, 0), (4, 0), (0, 4)]:
        assert g[y, x], (x, y)
    assert not g[0, 5] and not g[6, 6] and not g[3, 3]
    g = np.zeros((5, 5), np.uint8)
    g[2, 2], g[1, 2] = 6, 3
    g = dilate(g, 4)
    assert g[1, 1] == 6 and g[0, 0] == 6 and g[2, 2] == 6
    for w, h in [(1, 1), (1, 5), (5, 1), (2, 2), (3, 3)]:
        g = np.zeros((h, w), np.uint8)
        g[0, 0] = 1
        assert dilate(g, 1)[0, 0]


def serialize(crops, counts, entries, payload, bounce):
    cap = 256
    out = np.zeros(cap, np.uint32)
    cr = np.ascontiguousarray(np.asarray(crops, np.uint32).reshape(-1))
    cn = np.ascontiguousarray(np.asarray(counts, np.uint32))
    en = np.ascontiguousarray(np.asarray(entries, np.uint32).reshape(-1)) if entries else np.zeros(3, np.uint32)
    pl = np.ascontiguousarray(np.asarray(payload, np.uint32)) if payload else np.zeros(1, np.uint32)
    n = L.oracle_serialize(len(counts), ptr(cr), ptr(cn), ptr(en), ptr(pl), bounce, cap, ptr(out))
    return list(out[:n])


NONE = 0xFFFFFFFF


def test_triangle_words_layout():
    # src/bake/triangle_words.rs:104-162
    words = serialize([[4, 6, 8, 9], [0, 1, 2, 2]], [2, 0], [[3, 2, NONE], [7, 1, NONE]],
                      [0xAAAA, 0x1, 0xFF], 0)
    M = 0xFFFFFFFF
    assert words == [8, 2, 4, 9, 13, M - 1, M, 7, 2, 3, 14, 7, 16, 0, 0xAAAA, 0x1, 0xFF]
    words = serialize([[2, 2, 3, 3]], [2], [[0, 1, 2], [1, NONE, NONE]], [5, 9, 10], 1)
    assert words == [4, 0, 0, 6, 2, 0, 11, 12, 1, 0, 0, 5, 9, 10]
    words = serialize([[2, 2, 3, 3]], [2], [[0, 1, 2], [1, NONE, NONE]], [5, 9, 10], 0)
    assert words == [4, 0, 0, 6, 2, 0, 9, 1, 0, 5]


def spread(i, o, rect):
    out = (C.c_float * 2)()
    L.oracle_spread(i, o[0], o[1], rect, out)
    return out[0], out[1]


def test_spread_strips_and_cells():
    # src/bake/spread.rs:73-108
    for count in [1, 2, 4, 16, 64]:
        for axis, rect in [(0, 1), (1, 1), (0, 0)]:
            strips = sorted(int(spread(i, (0, 0), rect)[axis] * count) for i in range(count))
            assert strips == list(range(count))
    cells = sorted((int(spread(i, (0, 0), 1)[0] * 4), int(spread(i, (0, 0), 1)[1] * 4)) for i in range(16))
    assert cells == [(x, y) for x in range(4) for y in range(4)]
    off = (0.371, 0.913)
    for axis in range(2):
        v = sorted(spread(i, off, 1)[axis] for i in range(16))
        widest = max([v[0] + 1 - v[15]] + [b - a for a, b in zip(v, v[1:])])
        assert widest <= 2 / 16 + 1e-6
    assert spread(5, off, 0)[1] == np.float32(off[1])


def disk(sx, sy):
    out = (C.c_float * 2)()
    L.oracle_concentric_disk(sx, sy, out)
    return np.array([out[0], out[1]])


def test_concentric_disk():
    # src/bake/spread.rs:110-127
    assert np.array_equal(disk(0.5, 0.5), [0, 0])
    for c in [(0, 0), (1, 0), (0, 1), (1, 1)]:
        assert abs(np.linalg.norm(disk(*c)) - 1) < 1e-6
    assert np.allclose(disk(1.0, 0.5), [1, 0], atol=1e-6)
    assert abs(np.linalg.norm(disk(0.75, 0.6)) - 0.5) < 1e-6
    inside = sum(np.linalg.norm(disk(*spread(i, (0, 0), 1))) < 0.5 for i in range(256))
    assert 60 <= inside <= 68


def cosdir(n, s):
    out = (C.c_float * 3)()
    L.oracle_cosine_direction(ptr(f32(*n)), s[0], s[1], out)
    return np.array(list(out))


def test_cosine_directions_follow_the_cosine():
    # src/bake/sky.rs:55-70
    n = np.float32([0.3, 0.8, -0.5])
    n = n / np.linalg.norm(n)
    total = 0.0
    for i in range(1024):
        d = cosdir(n, spread(i, (0.3, 0.3), 1))
        assert abs(np.linalg.norm(d) - 1) < 1e-5 and np.dot(d, n) >= 0
        total += np.dot(d, n)
    assert abs(total / 1024 - 2 / 3) < 3e-3


def area_vis(rect, rotation, size, texel, samples=32, minimum=0, blocks=lambda p: False, reach=10.0,
             parts=(1, 2, 3)):
    pos, nrm = texel

    @orc.DIR_FN
    def blocked(d, dist):
        p = np.array(pos, np.float64) + np.array([d[0], d[1], d[2]]) * dist
        return int(bool(blocks(p)))

    frac, rays = C.c_float(), C.c_uint32()
    pp = np.ascontiguousarray(np.asarray(parts, np.uint64))
    some = L.oracle_area_visibility(rect, ptr(f32(*rotation)), ptr(f32(*size)), ptr(f32(0, 0, 0)),
                                    C.c_float(reach), ptr(f32(*pos)), ptr(f32(*nrm)), samples, minimum,
                                    ptr(pp), len(parts), blocked, C.byref(frac), C.byref(rays))
    return (frac.value, rays.value) if some else None


PANEL = (dl.scenes.rotation_x(-math.pi / 2), (2.0, 1.0))


def test_area_lights_adaptive_ray_counts():
    # src/bake/area.rs:225-241
    below = ((0.3, -2.0, 0.1), (0, 1, 0))
    tube = ((0, 0, 0, 1), (2.0, 0.0))
    assert area_vis(1, *PANEL, below) == (1.0, 5)
    assert area_vis(1, *PANEL, below, blocks=lambda p: True) == (0.0, 5)
    assert area_vis(0, *tube, below) == (1.0, 3)
    assert area_vis(1, *PANEL, below, minimum=16) == (1.0, 21)
    assert area_vis(0, *tube, below, minimum=16, blocks=lambda p: True) == (0.0, 19)
    assert area_vis(1, *PANEL, below, minimum=100) == (1.0, 37)


def test_area_lights_penumbrae():
    # src/bake/area.rs:243-271
    below = ((0.0, -2.0, 0.0), (0, 1, 0))
    bar = lambda p: -0.7 <= p[0] < -0.4
    assert area_vis(1, *PANEL, below, blocks=bar) == (1.0, 5)
    f, rays = area_vis(1, *PANEL, below, minimum=16, blocks=bar)
    assert rays == 37 and 0.7 < f < 0.95
    f, rays = area_vis(1, *PANEL, below, blocks=lambda p: p[0] < 0)
    assert rays == 37 and abs(f - 0.5) < 0.08
    f, _ = area_vis(1, *PANEL, ((1.5, -1.0, 0.0), (0, 1, 0)), blocks=lambda p: p[0] < 0)
    assert f > 0.6


def test_area_lights_out_of_reach():
    # src/bake/area.rs:273-298
    assert area_vis(1, *PANEL, ((0, 1, 0), (0, -1, 0))) is None
    assert area_vis(1, *PANEL, ((0, -2, 0), (0, -1, 0))) is None
    tube4 = ((0, 0, 0, 1), (4.0, 0.0))
    assert area_vis(0, *tube4, ((1.9, 1.0, 0.0), (0, -1, 0))) is not None
    beyond = ((3.5, 0.0, 0.0), (-1, 0, 0))
    assert area_vis(0, *tube4, beyond, samples=8, reach=1.6, parts=(0,)) is not None
    assert area_vis(0, *tube4, beyond, samples=8, reach=1.4, parts=(0,)) is None
    assert area_vis(0, *tube4, beyond, samples=8, reach=-2.0, parts=(0,)) is None


def sun_vis(degrees, normal, minimum, blocked, samples=64):
    rot = dl.scenes.rotation_x(-math.pi / 2)

    @orc.DIR_FN
    def cb(d, _):
        return int(bool(blocked(np.array([d[0], d[1], d[2]]))))

    frac, rays = C.c_float(), C.c_uint32()
    pp = np.ascontiguousarray(np.asarray([4, 5, 6], np.uint64))
    some = L.oracle_sun_visibility(ptr(f32(*rot)), C.c_float(degrees), ptr(f32(*normal)), samples, minimum,
                                   ptr(pp), 3, cb, C.byref(frac), C.byref(rays))
    return (frac.value, rays.value) if some else None


def test_sun_ray_counts_and_penumbra():
    # src/bake/sun.rs:88-143
    up = (0, 1, 0)
    assert sun_vis(0.0, up, 16, lambda d: False) == (1.0, 1)
    assert sun_vis(0.0, up, 16, lambda d: True) == (0.0, 1)
    assert sun_vis(0.0, (0, -1, 0), 16, lambda d: False) is None
    g = np.float32([1.0, -0.05, 0.0])
    assert sun_vis(0.0, g / np.linalg.norm(g), 0, lambda d: False) is not None
    assert sun_vis(0.53, up, 0, lambda d: False) == (1.0, 5)
    assert sun_vis(0.53, up, 16, lambda d: False) == (1.0, 21)
    f, rays = sun_vis(4.0, up, 16, lambda d: d[0] < 0)
    assert rays == 69 and abs(f - 0.5) < 0.06
    edge = math.tan(-0.5 * math.radians(2.0))
    f, _ = sun_vis(4.0, up, 16, lambda d: d[0] / d[1] < edge)
    assert 0.75 < f < 0.95
    widest = [1.0]

    def track(d):
        widest[0] = min(widest[0], d[1])
        return False

    sun_vis(4.0, up, 64, track)
    limit = math.cos(math.radians(2.0))
    assert limit - 1e-6 <= widest[0] < limit + 1e-4


def sky_vis(normal, samples, blocked):
    @orc.DIR_FN
    def cb(d, _):
        return int(bool(blocked(np.array([d[0], d[1], d[2]]))))

    pp = np.ascontiguousarray(np.asarray([1, 2, 3], np.uint64))
    return L.oracle_sky_visibility(ptr(f32(*normal)), samples, ptr(pp), 3, cb)


def test_sky_fractions():
    # src/bake/sky.rs:71-85
    assert sky_vis((0, 1, 0), 64, lambda d: False) == 1.0
    assert sky_vis((0, 1, 0), 64, lambda d: True) == 0.0
    assert abs(sky_vis((0, 1, 0), 64, lambda d: d[0] < 0) - 0.5) < 0.04
    low = math.sin(math.radians(30))
    assert abs(sky_vis((0, 1, 0), 256, lambda d: d[1] < low) - 0.75) < 0.02


def intersect(v, o, d, mx):
    t = C.c_float()
    w = (C.c_float * 3)()
    hit = L.oracle_intersect(ptr(f32(*v)), ptr(f32(*o)), ptr(f32(*d)), C.c_float(mx), C.byref(t), w)
    return (t.value, list(w)) if hit else None


def test_intersection_edge_cases():
    # src/bake/tests/occluder.rs:14-38
    quad = [0, 0, 0, 1, 0, 0, 0, 0, 1]
    t, w = intersect(quad, (0.25, 1, 0.25), (0, -1, 0), 10.0)
    assert t == 1.0 and abs(sum(w) - 1) < 1e-6
    assert intersect(quad, (0.25, -1, 0.25), (0, 1, 0), 10.0) is not None
    assert intersect(quad, (0.25, 1, 0.25), (0, -1, 0), 1.0) is not None
    assert intersect(quad, (0.25, 1, 0.25), (0, -1, 0), 0.999) is None
    assert intersect(quad, (0.25, 1, 0.25), (0, 1, 0), 10.0) is None
    assert intersect(quad, (0.25, 1, 0.25), (1, 0, 0), 10.0) is None


def pack_bounce(values, bits, rgb=False):
    v = np.ascontiguousarray(np.asarray(values, np.float32).reshape(-1))
    out = np.zeros(len(v) + 4, np.uint32)
    n = L.oracle_pack_bounce(ptr(v), len(values), int(rgb), bits, None, 0, ptr(out))
    return [int(x) for x in out[:n]]


def test_bounce_packing_words():
    # src/bake/bounce_pack.rs:129-212
    assert [len(pack_bounce([1.0] * 9, b)) for b in (8, 6, 5, 4)] == [3, 2, 2, 2]
    assert pack_bounce([1.0, 0.0, 1.0], 8) == [0x00FF00FF]
    assert pack_bounce([1.0] * 5, 6) == [(1 << 30) - 1]
    assert pack_bounce([[1.0, 0.0, 0.25], [1, 1, 1]], 8, rgb=True) == [0xFF7F00FF, 0xFFFF]
    assert len(pack_bounce([[1.0, 0.0, 0.25], [1, 1, 1]], 5, rgb=True)) == 1
    assert len(pack_bounce([[1, 1, 1]] * 16, 6, rgb=True)) == 9
    for b in (8, 6, 5, 4):
        words = pack_bounce([0.0, float("nan"), -1.0], b)
        mask = (1 << b) - 1
        per = 32 // b
        for i in range(3):
            assert (words[i // per] >> ((i % per) * b)) & mask == 0


def test_windowed_bounce_filters_match_a_full_map():
    # src/bake/bounce_map.rs:224-253
    size = 24
    tex = [(1, 1, 0.5), (2, 1, 0.25), (12, 13, 1.0), (13, 13, 0.75), (0, 3, 0.1)]
    arr = np.array([[x, y, v, v * 0.5, v * 0.25] for x, y, v in tex], np.float32)
    out = np.zeros(size * size * 3, np.float32)
    win = (C.c_uint32 * 4)()
    L.oracle_bounce_map(size, (C.c_uint32 * 4)(0, 0, 14, 14), ptr(arr), len(tex), ptr(out), win)
    w = win[2] - win[0] + 1
    got = out[:w * (win[3] - win[1] + 1) * 3].reshape(-1, w, 3)
    # full map, filters out of place (bounce_map.rs:167-222), in float32
    full = np.zeros((size, size), np.float32)
    for x, y, v in tex:
        full[y, x] = v
    order = [(0, 0), (-1, -1), (0, -1), (1, -1), (-1, 0), (1, 0), (-1, 1), (0, 1), (1, 1)]

    def at(m, x, y):
        return m[y, x] if 0 <= x < size and 0 <= y < size else np.float32(0)

    dil = np.zeros_like(full)
    for y in range(size):
        for x in range(size):
            for dx, dy in order:
                v = at(full, x + dx, y + dy)
                if v > 0:
                    dil[y, x] = v
                    break
    wts = (C.c_float * 7)()
    L.oracle_gaussian_weights(wts)
    wts = np.array(list(wts), np.float32)
    cur = dil
    for vertical in (False, True):
        nxt = np.zeros_like(cur)
        for y in range(size):
            for x in range(size):
                s = np.float32(0)
                for k in range(-3, 4):
                    sx, sy = (x, min(max(y + k, 0), size - 1)) if vertical else (min(max(x + k, 0), size - 1), y)
                    s = np.float32(s + at(cur, sx, sy) * wts[k + 3])
                nxt[y, x] = s / np.float32(wts.sum(dtype=np.float32))
        cur = nxt
    for y in range(15):
        for x in range(15):
            g = got[y - win[1], x - win[0]]
            e = cur[y, x]
            assert np.allclose(g, [e, e * 0.5, e * 0.25], atol=1e-6), (x, y)
    assert abs(float(wts.sum()) - 1) < 1e-6 and wts[0] == wts[6] and wts[3] > wts[2] > wts[1]


def cube_texel(d, res):
    out = (C.c_uint32 * 3)()
    L.oracle_cube_texel(ptr(f32(*d)), res, out)
    return tuple(out)


def test_cube_face_table_and_round_trips():
    # src/shared/cube.rs:117-201
    axes = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    for face, a in enumerate(axes):
        assert cube_texel(a, 2) [0] == face
    assert cube_texel((1, -0.5, -0.5), 4) == (0, 3, 3)
    assert cube_texel((0.5, 1.0, 0.5), 4) == (2, 3, 3)
    assert cube_texel((0.5, -1.0, -0.5), 4) == (3, 3, 3)
    assert cube_texel((-0.5, -0.5, -1.0), 4) == (5, 3, 3)
    res = 16
    out = (C.c_float * 3)()
    for face in range(6):
        for y in range(res):
            for x in range(res):
                L.oracle_cube_direction(face, x, y, res, out)
                d = list(out)
                assert abs(math.sqrt(sum(c * c for c in d)) - 1) < 1e-5
                assert cube_texel(d, res) == (face, x, y)
                assert cube_texel([c * 7.5 for c in d], res) == (face, x, y)
    f, x, y = cube_texel((0, 0, 0), 64)
    assert x < 64 and y < 64


def test_light_bvh_partitions_lights_and_matches_brute_force():
    # src/bake/light_bvh.rs:250-316
    state = [0x12345678]

    def nxt():
        state[0] = dl.scenes.splitmix64(state[0])
        return (state[0] >> 40) / float(1 << 24)

    def lights(n):
        pos, rad = [], []
        for _ in range(n):
            p = np.float32([nxt(), nxt(), nxt()]) * np.float32(40.0) - np.float32(20.0)
            pos.append(p)
            rad.append(np.float32(0.5 + nxt() * 4.0))
        return np.array(pos, np.float32), np.array(rad, np.float32)

    pos, rad = lights(57)
    nodes = (dl._abi.DlLightBvhNode * 200)()
    order = np.zeros(57, np.uint32)
    n = L.oracle_light_bvh(ptr(pos), ptr(rad), 57, nodes, ptr(order))
    assert sorted(order) == list(range(57)) and n < 2 * 57
    covered = [0] * 57
    for i in range(n):
        nd = nodes[i]
        if nd.count:
            assert nd.count <= 2
            for s in range(nd.left_first, nd.left_first + nd.count):
                covered[s] += 1
                p, r = pos[order[s]], rad[order[s]]
                assert all(nd.aabb_min[k] <= p[k] - r for k in range(3))
                assert all(nd.aabb_max[k] >= p[k] + r for k in range(3))
    assert covered == [1] * 57
    one = L.oracle_light_bvh(ptr(np.float32([1, 1, 1])), ptr(np.float32([2])), 1, nodes, ptr(order))
    assert one == 1 and nodes[0].count == 1 and list(nodes[0].aabb_min) == [-1, -1, -1]
    same = L.oracle_light_bvh(ptr(np.zeros(15, np.float32)), ptr(np.ones(5, np.float32)), 5, nodes, ptr(order))
    assert same == 1 and nodes[0].count == 5


def test_rng_streams():
    # src/bake/random.rs:33-51
    def seed(*parts):
        p = np.ascontiguousarray(np.asarray(parts, np.uint64))
        return L.oracle_seed(ptr(p), len(parts))

    assert seed(1, 2, 3) == seed(1, 2, 3)
    assert seed(1, 2, 3) != seed(1, 2, 4) and seed(1, 2, 3) != seed(3, 2, 1) and seed(0) != seed(0, 0)
    # The fold: splitmix64(acc ^ splitmix64(part)) from 0x0b4c_e5ee_d000_0000.
    sm = dl.scenes.splitmix64
    acc = 0x0B4CE5EED0000000
    for part in (7, 11):
        acc = sm(acc ^ sm(part))
    assert seed(7, 11) == acc


def test_transcendentals_are_correctly_rounded():
    # The oracle's policy: binary64 evaluation, one rounding (see oracle_math.hpp).
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.uniform(-8, 8, 4000), [0.0, 1e-8, math.pi / 4, 3.0]]).astype(np.float32)
    out = (C.c_float * 2)()
    bad = 0
    for x in xs:
        L.oracle_sincos(C.c_float(x), out)
        bad += out[0] != np.float32(math.sin(float(x))) or out[1] != np.float32(math.cos(float(x)))
    assert bad == 0


def acos_approx_f32(v):
    """glam's acos_approx restated in numpy binary32 (every operation rounds once): Abramowitz &
    Stegun 4.4.46, sqrt(1 - |x|) * p(|x|) by Horner's rule, pi minus it below zero."""
    f = np.float32
    v = np.asarray(v, np.float32)
    x = np.abs(v)
    omx = np.maximum(f(1) - x, f(0))
    r = np.full_like(x, f(-0.0012624911))
    for c in (0.0066700901, -0.0170881256, 0.0308918810, -0.0501743046, 0.0889789874, -0.2145988016,
              1.5707963050):
        r = (r * x).astype(np.float32) + f(c)
    r = r * np.sqrt(omx)
    return np.where(v >= 0, r, f(math.pi) - r).astype(np.float32)


def test_acos_approx_is_glams_polynomial():
    """The slerp angle of gather_triangle (src/bake/bounce.rs:270): glam's acos_approx, bit for
    bit, within its published accuracy of the true arccosine, exact at 1 and -1."""
    rng = np.random.default_rng(11)
    xs = np.concatenate([rng.uniform(-1, 1, 20000), np.linspace(-1, 1, 2001), [0.0, -0.0, 1.0, -1.0],
                         1 - rng.uniform(0, 1e-3, 2000), -1 + rng.uniform(0, 1e-3, 2000)]).astype(np.float32)
    want = acos_approx_f32(xs)
    got = np.array([L.oracle_acos_approx(C.c_float(x)) for x in xs], np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.abs(got.astype(np.float64) - np.arccos(xs.astype(np.float64))).max() < 1e-6
    assert L.oracle_acos_approx(C.c_float(1.0)) == 0.0
    assert L.oracle_acos_approx(C.c_float(-1.0)) == np.float32(math.pi)
    assert L.oracle_acos_approx(C.c_float(0.0)) == np.float32(1.5707963050)  # not pi/2 rounded


def test_slerp_is_unit_and_spans_the_arc():
    out = (C.c_float * 3)()
    a, b = f32(1, 0, 0), f32(0, 1, 0)
    L.oracle_slerp(ptr(a), ptr(b), C.c_float(0.5), out)
    assert np.allclose(list(out), [math.sqrt(0.5), math.sqrt(0.5), 0], atol=1e-6)
    L.oracle_slerp(ptr(a), ptr(b), C.c_float(0.0), out)
    assert np.allclose(list(out), [1, 0, 0], atol=1e-6)
    # lengths interpolate linearly: |slerp(a, 3b, 0.5)| = 2
    L.oracle_slerp(ptr(a), ptr(f32(0, 3, 0)), C.c_float(0.5), out)
    assert abs(np.linalg.norm(list(out)) - 2) < 1e-5
    # nearly equal vectors take the lerp; nearly opposite ones turn about an orthogonal axis
    L.oracle_slerp(ptr(a), ptr(f32(1, 1e-5, 0)), C.c_float(0.5), out)
    assert np.allclose(list(out), [1, 0.5e-5, 0], atol=1e-7)
    for s in (0.25, 0.5, 0.75):
        L.oracle_slerp(ptr(a), ptr(f32(-1, 0, 0)), C.c_float(s), out)
        v = np.array(list(out))
        assert abs(np.linalg.norm(v) - 1) < 1e-6 and abs(math.acos(max(-1.0, min(1.0, v[0]))) - math.pi * s) < 1e-5
    # the sine-weighted branch for a generic pair equals the closed form within f32 rounding
    rng = np.random.default_rng(3)
    for _ in range(200):
        p, q = rng.normal(size=3), rng.normal(size=3)
        p, q = p / np.linalg.norm(p), q / np.linalg.norm(q)
        s = float(rng.uniform(0.1, 1.0))
        L.oracle_slerp(ptr(f32(*p)), ptr(f32(*q)), C.c_float(s), out)
        th = math.acos(float(np.clip(np.dot(p, q), -1, 1)))
        want = (math.sin((1 - s) * th) * p + math.sin(s * th) * q) / math.sin(th)
        assert np.allclose(list(out), want, atol=2e-5)


def test_orthonormal_pair_and_rotation():
    out = (C.c_float * 6)()
    for n in [(0, 1, 0), (0, 0, -1), (0.6, 0.0, 0.8), (0.0, -0.6, 0.8)]:
        L.oracle_any_orthonormal_pair(ptr(f32(*n)), out)
        a, b, nn = np.array(out[:3]), np.array(out[3:]), np.array(n, np.float32)
        for v in (a, b):
            assert abs(np.linalg.norm(v) - 1) < 1e-6 and abs(np.dot(v, nn)) < 1e-6
        assert abs(np.dot(a, b)) < 1e-6
    r = (C.c_float * 3)()
    L.oracle_quat_rotate(ptr(f32(*dl.scenes.rotation_x(-math.pi / 2))), ptr(f32(0, 0, 1)), r)
    assert np.allclose(list(r), [0, 1, 0], atol=1e-6)  # a sun turned down is above (src/light/shape.rs:153-161)


def v3(*x):
    return ptr(f32(*x))


def test_closest_point_covers_every_region():
    # src/bake/geometry.rs:159-189: the seven Voronoi regions of a right triangle in z = 0
    tri = f32(0, 0, 0, 1, 0, 0, 0, 1, 0)
    cases = [((0.25, 0.25, 1.0), (0.25, 0.25, 0.0)), ((-1.0, -1.0, 0.0), (0, 0, 0)), ((2.0, -0.5, 0.0), (1, 0, 0)),
             ((-0.5, 2.0, 0.0), (0, 1, 0)), ((0.5, -1.0, 0.0), (0.5, 0.0, 0.0)), ((-1.0, 0.5, 0.0), (0.0, 0.5, 0.0)),
             ((1.0, 1.0, 0.0), (0.5, 0.5, 0.0))]
    out = np.zeros(3, np.float32)
    for p, want in cases:
        L.oracle_closest_point(v3(*p), ptr(tri), ptr(out))
        assert np.all(np.abs(out - np.float32(want)) <= 1e-6), (p, out)
    L.oracle_sphere_triangle.argtypes = [C.c_void_p, C.c_float, C.c_void_p]
    assert L.oracle_sphere_triangle(v3(0.2, 0.2, 0.5), 0.5, ptr(tri)) == 1
    assert L.oracle_sphere_triangle(v3(0.2, 0.2, 0.6), 0.5, ptr(tri)) == 0


def test_barycentrics_detect_outside_points_and_both_windings():
    # src/bake/geometry.rs:191-201
    w = np.zeros(3, np.float32)
    assert L.oracle_uv_barycentrics(ptr(f32(0, 0, 1, 0, 0, 1)), ptr(f32(0.25, 0.25)), ptr(w)) == 1
    assert np.all(np.abs(w - np.float32([0.5, 0.25, 0.25])) <= 1e-6)
    assert L.oracle_uv_barycentrics(ptr(f32(0, 0, 1, 0, 0, 1)), ptr(f32(0.75, 0.75)), ptr(w)) == 0
    assert L.oracle_uv_barycentrics(ptr(f32(0, 0, 0, 1, 1, 0)), ptr(f32(0.25, 0.25)), ptr(w)) == 1
    assert np.all(np.abs(w - np.float32([0.5, 0.25, 0.25])) <= 1e-6), "the flipped winding"
    assert L.oracle_uv_barycentrics(ptr(f32(0, 0, 1, 0, 2, 0)), ptr(f32(1, 0)), ptr(w)) == 0, "degenerate"


def test_boxes_and_areas():
    # src/bake/geometry.rs:203-215
    L.oracle_box_sphere_overlap.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float]
    L.oracle_box_half_area_x2.restype = C.c_float
    L.oracle_triangle_area.restype = C.c_float
    L.oracle_approx_eq.argtypes = [C.c_void_p, C.c_void_p, C.c_float]
    assert L.oracle_box_sphere_overlap(v3(0, 0, 0), v3(1, 1, 1), v3(2, 2, 2), 1.0) == 1, "touching boxes overlap"
    assert L.oracle_box_sphere_overlap(v3(0, 0, 0), v3(1, 1, 1), v3(2, 2, 2), 0.9) == 0
    assert L.oracle_box_half_area_x2(v3(0, 0, 0), v3(1, 1, 1), 0) == 6.0
    assert L.oracle_box_half_area_x2(v3(0, 0, 0), v3(0, 0, 0), 1) == 0.0, "the empty box"
    assert L.oracle_triangle_area(ptr(f32(0, 0, 0, 2, 0, 0, 0, 2, 0))) == 2.0
    assert L.oracle_approx_eq(v3(0, 1, 0), v3(0, 1.000001, 0), 1e-5) == 1
    assert L.oracle_approx_eq(v3(0, 1, 0), v3(0, -1, 0), 1e-5) == 0


class OneLight:
    """A BakeLight marshalled as a dl_light for the oracle's light helpers."""

    def __init__(self, light):
        self.m = dl.Marshalled(dl.BakeInput([], [light]))
        self.p = self.m.input.lights
        L.oracle_light_reach.restype = C.c_float

    def reach(self):
        return L.oracle_light_reach(self.p)

    def bits(self):
        return L.oracle_light_shadow_bits(self.p)

    def may_face(self, tri, normal):
        return L.oracle_light_may_face(self.p, ptr(f32(*np.ravel(tri))), v3(*normal)) == 1


def test_area_lights_reach_and_face_with_their_shape():
    # src/bake/light_shape.rs:77-113
    point = OneLight(fx.point_light(1, (0, 2, 0), 3.0))
    assert (point.reach(), point.bits()) == (3.0, 1)
    tube = OneLight(fx.area_light(1, (0, 2, 0), 5.0, (0.0, 0.0, 0.0, 1.0), (4.0, 0.0)))
    assert (tube.reach(), tube.bits()) == (3.0, 4)
    wall = np.float32([[1.5, 0, 0], [1.5, 1, 0], [1.5, 0, 1]])
    assert tube.may_face(wall, (1, 0, 0)), "a wall at x = 1.5 facing +X sees the tube's far end"
    assert not tube.may_face(wall + np.float32([1, 0, 0]), (1, 0, 0))
    panel = OneLight(fx.area_light(1, (0, 2, 0), 5.0, scenes.rotation_x(-math.pi / 2), (1.0, 1.0)))
    floor = np.float32([[0, 0, 0], [0, 0, 1], [1, 0, 0]])
    assert not panel.may_face(floor + np.float32([0, 3, 0]), (0, 1, 0)), "above a downward panel: its dark side"
    assert panel.may_face(floor, (0, 1, 0))


def test_suns_face_by_direction_and_soften_with_their_disk():
    # src/bake/light_shape.rs:114-128
    floor = np.float32([[0, 0, 0], [0, 0, 1], [1, 0, 0]])
    low = OneLight(fx.sun_light(1, (1.0, 0.02, 0.0), 0.0))
    assert low.bits() == 1, "no disk, hard shadows"
    assert low.may_face(floor, (0, 1, 0))
    assert low.may_face(floor, (0, -1, 0)), "within Henry's tolerance"
    assert not low.may_face(floor, (-1, 0, 0))
    below = np.float32([1.0, -0.11, 0.0])
    below = below / np.float32(np.linalg.norm(below))
    assert not OneLight(fx.sun_light(2, below, 0.0)).may_face(floor, (0, 1, 0))
    wide = OneLight(fx.sun_light(2, below, 10.0))
    assert wide.may_face(floor, (0, 1, 0)), "the top of a wide disk still reaches the floor"
    assert wide.bits() == 4


def test_crops_offset_by_two_and_dilate():
    # src/bake/shadows.rs:174-191
    for bits in (1, 4):
        levels = np.zeros((10, 10), np.uint8)
        levels[5, 4] = 1
        out = np.zeros(7 * 6, np.uint8)
        L.oracle_crop_shadows(ptr(levels), 10, 10, bits, ptr(np.uint32([0, 0, 9, 9])), ptr(np.uint32([4, 5, 6, 6])),
                              ptr(out))
        g = out.reshape(6, 7)
        assert g[2, 2] == 1, "texel (4, 5) lands at (2, 2)"
        assert (g[0, 0], g[1, 1]) == (1, 1), "dilated"
        assert g[3, 3] == 0, "interior texels are not dilated"


def test_any_light_only_looks_inside_both_rects():
    # src/bake/shadows.rs:193-205
    levels = np.zeros((4, 4), np.uint8)
    levels[3, 3] = 2
    region = ptr(np.uint32([10, 10, 13, 13]))
    hits = [L.oracle_any_light(ptr(levels), 4, 4, 4, region, ptr(np.uint32(q)))
            for q in ([12, 12, 20, 20], [0, 0, 12, 12], [0, 0, 5, 5])]
    assert hits == [1, 0, 0]


def rng_u32(seed, stream_id, count):
    out = np.zeros(count, np.uint32)
    L.oracle_rng_u32.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_void_p]
    L.oracle_rng_u32(seed, stream_id, count, ptr(out))
    return out


def for_light(seed, key, count):
    """EffectRng::for_light(seed, key) (src/effects/rng.rs:33-35): `count` u32 values."""
    sm = dl.scenes.splitmix64
    return rng_u32(sm(seed ^ sm(key)), key, count)


def test_pcg_streams_repeat_per_seed_and_differ_between_lights():
    # src/effects/rng.rs:96-107
    a, b, c = for_light(7, 1, 16), for_light(7, 1, 16), for_light(7, 2, 16)
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_pcg_floats_are_uniform_in_the_unit_interval():
    # src/effects/rng.rs:108-122: next_f32 = (u32 >> 8) * 2^-24
    values = (for_light(1, 99, 100_000) >> 8).astype(np.float32) * np.float32(1.0 / 16777216.0)
    assert values.min() >= 0.0 and values.max() < 1.0
    shares = np.bincount((values * np.float32(10.0)).astype(int), minlength=10) / values.size
    assert np.all(np.abs(shares - 0.1) < 0.01), shares


def test_splitmix_spreads_neighbouring_inputs():
    # src/effects/rng.rs:156-160
    sm = dl.scenes.splitmix64
    assert 16 <= bin(sm(1) ^ sm(2)).count("1") <= 48


def test_sphere_points_are_unit_and_centered():
    # src/bake/random.rs:41-51: 20 000 points of the keyed stream [7]
    out = np.zeros(3 * 20_000, np.float32)
    L.oracle_sphere_points(ptr(np.uint64([7])), 1, 20_000, ptr(out))
    p = out.reshape(-1, 3).astype(np.float64)
    assert np.all(np.abs(np.linalg.norm(p, axis=1) - 1.0) < 1e-4)
    assert np.linalg.norm(p.mean(axis=0)) < 0.02
