"""GPU parity of the maps for moving meshes (distance cubes, sun maps, sky probes) against the
oracle, bit for bit, in both geometry modes that bake them, in every form; and the .dynlight
payload of a scene with maps (src/bake/format/mod.rs:170-213, maps.rs:16-38)."""
import struct

import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import scenes
from oracle import oracle

from . import fixtures as fx
from .test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def assert_maps(got, want):
    assert got.maps_equal(want)
    assert got.distance_cubes.size == 6 * 64 * 64 // 2 * sum(
        1 for l in want.lights if l.shape not in (dl.SUN, dl.SKY))


def mixed_room(geometry):
    inp, opts = fx.determinism_room()
    opts.dynamic_geometry = geometry
    opts.sun_map_resolution = 96
    opts.sky_probe_spacing = 0.7
    opts.sky_samples = 32
    return inp, opts


@pytest.mark.parametrize("form", ["batched", "plain"])
@pytest.mark.parametrize("geometry", [dl.DISTANCE_CUBES, dl.ANGULAR])
def test_maps_of_every_light_kind_match_the_oracle(form, geometry):
    inp, opts = mixed_room(geometry)
    want, _, _ = oracle.bake(inp, opts)
    assert want.sun_maps and want.sky_probes is not None and want.distance_cubes.size
    got = dl.bake(inp, opts, form=form)
    assert_same(got, want)
    assert_maps(got, want)


def test_outdoor_maps_with_alpha_and_the_refined_form():
    inp, opts = scenes.outdoor(grid=65, chunks=2, boxes=30, point_lights=4, sky_samples=16, bounce_samples=8)
    opts.dynamic_geometry = dl.ANGULAR
    opts.sun_map_resolution = 257  # odd: the last word's upper half is the filler 1
    opts.sky_probe_spacing = 3.0
    for light in inp.lights[:2]:
        light.transparency = dl.TRANSPARENCY_ENABLED
    want, _, _ = oracle.bake(inp, opts)
    got = dl.bake(inp, opts)
    assert_same(got, want)
    assert_maps(got, want)
    refined_want = oracle.bake_ex(inp, opts, mode=oracle.REFINED, eps=dl.DEFAULT_REFINE_EPSILON)["scene"]
    refined = dl.bake(inp, opts, form="refined")
    assert_same(refined, refined_want)
    assert refined.maps_equal(refined_want)


def test_maps_of_an_empty_scene():
    # no static geometry: cubes store the radius, the sun map is one open texel, no probes
    opts = fx.options(dynamic_geometry=dl.ANGULAR)
    inp = dl.BakeInput([], [fx.point_light(7, (0, 1, 0), 3.0), fx.sun_light(9, (0.3, 1.0, 0.2), 0.53),
                            fx.sky_light(10)])
    want, _, _ = oracle.bake(inp, opts)
    got = dl.bake(inp, opts)
    assert got.maps_equal(want)
    assert got.sky_probes is None and got.sun_maps[0].resolution == 1
    radius = np.float16(3.0).view(np.uint16)
    assert np.all(got.distance_cubes == (int(radius) << 16 | int(radius)))


# ---- the payload ------------------------------------------------------------------------------

class Reader:
    """parse_payload (src/bake/format/mod.rs:218-299) over the uncompressed bytes."""

    def __init__(self, data):
        self.d, self.i = data, 0

    def take(self, fmt):
        v = struct.unpack_from("<" + fmt, self.d, self.i)
        self.i += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def words(self):
        n = self.take("Q")
        w = np.frombuffer(self.d, np.uint32, n, self.i).copy()
        self.i += 4 * n
        return w


def decode_payload(data):
    r = Reader(data)
    flags, geometry, density, max_size, cube_res = r.take("IIfII")
    lights = []
    for _ in range(r.take("Q")):
        lid = r.take("Q")
        origin = r.take("fff")
        radius, bounce_bits, shape = r.take("fII")
        rotation, size, bits = r.take("ffff"), r.take("ff"), r.take("I")
        lights.append((lid, shape, bits))
    bvh = r.words()
    meshes = []
    for _ in range(r.take("Q")):
        mid, chash, res, occludes = r.take("QQII")
        meshes.append((mid, res, r.words()))
    cubes = r.words()
    sun_maps = []
    for _ in range(r.take("Q")):
        res = r.take("I")
        rows = np.array(r.take("f" * 12), np.float32)
        sun_maps.append((res, rows, r.words()))
    probes = None
    if r.take("I"):
        origin, spacing, counts = r.take("fff"), r.take("f"), r.take("III")
        probes = (origin, spacing, counts, r.words())
    stats = r.take("IQQQQQQ")
    assert r.i == len(data), "trailing payload"
    return dict(flags=flags, geometry=geometry, lights=lights, bvh=bvh, meshes=meshes, cubes=cubes,
                sun_maps=sun_maps, probes=probes, stats=stats)


def test_payload_with_maps_round_trips_and_matches_the_oracle():
    import ctypes as C
    inp, opts = mixed_room(dl.ANGULAR)
    lib = dl.load_library()
    m = dl.Marshalled(inp)
    copts = dl.marshal_options(opts)
    cfg = dl.make_config("batched")
    out = C.POINTER(dl._abi.DlBakedScene)()
    assert lib.dl_bake_ex(C.byref(m.input), C.byref(copts), C.byref(cfg), None, C.byref(out), None) == 0
    try:
        payload, crc = dl.encode_payload(out.contents)
        scene = dl.scene_from_c(out.contents)
    finally:
        lib.dl_baked_scene_free(out)
    import zlib
    assert zlib.crc32(payload) == crc
    p = decode_payload(payload)
    assert p["geometry"] == dl.ANGULAR
    assert [mm[0] for mm in p["meshes"]] == [mm.id for mm in scene.meshes]
    assert all(np.array_equal(a[2], b.triangles) for a, b in zip(p["meshes"], scene.meshes))
    assert np.array_equal(p["cubes"], scene.distance_cubes)
    assert len(p["sun_maps"]) == len(scene.sun_maps)
    for (res, rows, texels), sm in zip(p["sun_maps"], scene.sun_maps):
        assert res == sm.resolution and np.array_equal(rows, sm.rows.reshape(-1))
        assert np.array_equal(texels, sm.texels)
    assert p["probes"][2] == scene.sky_probes.counts and np.array_equal(p["probes"][3], scene.sky_probes.words)
    # the oracle's scene through the same writer gives the same bytes
    lb = oracle.lib()
    oout = C.POINTER(dl._abi.DlBakedScene)()
    status = lb.oracle_bake(C.byref(m.input), C.byref(copts), None, 0, 0, C.byref(oout), None, None)
    assert status == 0
    try:
        want, want_crc = dl.encode_payload(oout.contents)
    finally:
        lb.oracle_free(oout)
    assert payload == want and crc == want_crc


def test_payload_encoded_on_the_device_equals_the_host_encoding():
    import zlib
    # a scene whose payload spans several 64 KiB chunks, with maps, and an empty one
    for inp, opts in (mixed_room(dl.ANGULAR),
                      scenes.outdoor(grid=65, chunks=2, boxes=20, point_lights=3, sky_samples=16, bounce_samples=8),
                      (dl.BakeInput([], [fx.point_light(7, (0, 1, 0), 3.0)]), fx.options())):
        s = dl.Session(inp, opts)
        try:
            s.run()
            payload, crc = s.encode_payload()
            import ctypes as C
            out = C.POINTER(dl._abi.DlBakedScene)()
            assert s.lib.dl_session_result(s.handle, C.byref(out)) == 0
            try:
                want, want_crc = dl.encode_payload(out.contents)
            finally:
                s.lib.dl_baked_scene_free(out)
        finally:
            s.close()
        assert payload == want
        assert crc == want_crc == zlib.crc32(want)
