"""The `.dynlight` file (`dynlight_file.py`) against the reference's format tests
(src/bake/format/tests.rs:31-359): round trips of a scene with every light kind and both maps,
light order and map count rules, sky probe rules, version and corruption errors, invalid payload
values, and streamed reads that agree with whole-buffer reads, errors included. Plus: the Python
payload writer gives the same bytes as the library's C++ writer on an oracle bake (CPU), and the
device-encoded payload of a session decodes to the bake (GPU)."""
import ctypes as C
import io
import math
import os
import struct
import zlib

import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import dynlight_file as f
from dynlight_gb300.dynlight_file import FormatError
from oracle import oracle

from . import fixtures as fx


def rot_x(angle):
    return tuple(float(v) for v in np.float32([math.sin(angle / 2), 0.0, 0.0, math.cos(angle / 2)]))


def sky(light_id):
    return dl.BakedLight(light_id, (0.0, 0.0, 0.0), 10.0, dl.SKY, (0.0, 0.0, 0.0, 1.0), (0.0, 0.0), 0, 8)


def sun(light_id):
    return dl.BakedLight(light_id, (0.0, 0.0, 0.0), 10.0, dl.SUN, rot_x(-1.0), (float(np.float32(0.53)), 0.0), 0, 4)


def sample():
    """tests.rs:31-122: three local lights (a panel with 5-bit bounce, a point, a tube), a sun
    and a sky; a BVH node; two meshes; distance cube words; one 3x3 sun map; 2x1x3 sky probes."""
    lights = [dl.BakedLight(42, (1.0, -2.5, 3.25), 6.0, dl.RECTANGLE, rot_x(-0.5),
                            (float(np.float32(1.6)), float(np.float32(0.4))), 5, 4),
              dl.BakedLight(7, (0.0, 0.0, 0.0), 0.5, dl.POINT, (0.0, 0.0, 0.0, 1.0), (0.0, 0.0), 0, 1),
              dl.BakedLight(9, (0.0, 1.0, 0.0), 3.0, dl.TUBE, (0.0, 0.0, 0.0, 1.0), (2.0, 0.0), 0, 2),
              sun(3), sky(11)]
    node = np.concatenate([np.float32([-1, -2, -3]).view(np.uint32), [0],
                           np.float32([4, 5, 6]).view(np.uint32), [2]]).astype(np.uint32).reshape(1, 8)
    meshes = [dl.BakedMesh(1, 0xABCD, 128, np.uint32([4, 0, 0, 5, 0]), True),
              dl.BakedMesh(2, 3, 2, np.zeros(0, np.uint32), False)]
    sun_map = dl.SunMap(np.float32([[1, 0, 0, 0], [0, 0.5, 0, 0.25], [-0.125] * 4]), 3,
                        np.uint32([0xFFFF0000, 1, 2, 3, 0x8000]))
    probes = dl.SkyProbes((-0.5, 0.25, 2.0), 1.5, (2, 1, 3), np.uint32([0x01010101 * i for i in range(12)]))
    settings = dict(bounce=True, colored_bounce=True, dynamic_geometry=dl.DISTANCE_CUBES, pixel_density=64.0,
                    max_lightmap_size=1024, distance_cube_resolution=64)
    stats = dict(meshes=2, triangles=1, texels=10, rays=20, lights_removed=1, bounce_rays=0, triangle_words=5)
    return dl.BakedScene(settings, lights, node, meshes, np.uint32([0x3C003C00, 7]), stats, [sun_map], probes)


def empty():
    settings = dict(bounce=False, colored_bounce=False, dynamic_geometry=dl.LIGHTING_ONLY, pixel_density=0.0,
                    max_lightmap_size=0, distance_cube_resolution=0)
    stats = dict(meshes=0, triangles=0, texels=0, rays=0, lights_removed=0, bounce_rays=0, triangle_words=0)
    return dl.BakedScene(settings, [], np.zeros((0, 8), np.uint32), [], np.zeros(0, np.uint32), stats, [], None)


def same(a, b):
    """Scenes equal field by field, floats by their binary32 bits."""
    bits = lambda v: np.float32(v).view(np.uint32).tolist()  # noqa: E731
    assert {k: (bits(v) if isinstance(v, float) else v) for k, v in a.settings.items()} == \
           {k: (bits(v) if isinstance(v, float) else v) for k, v in b.settings.items()}
    assert [(l.id, bits(l.origin), bits(l.radius), l.shape, bits(l.rotation), bits(list(l.size[:2])), l.bounce_bits,
             l.shadow_bits_per_texel) for l in a.lights] == \
           [(l.id, bits(l.origin), bits(l.radius), l.shape, bits(l.rotation), bits(list(l.size[:2])), l.bounce_bits,
             l.shadow_bits_per_texel) for l in b.lights]
    assert np.array_equal(np.asarray(a.light_bvh, np.uint32).reshape(-1), np.asarray(b.light_bvh, np.uint32).reshape(-1))
    assert [(m.id, m.content_hash, m.resolution, m.occludes, m.triangles.tolist()) for m in a.meshes] == \
           [(m.id, m.content_hash, m.resolution, m.occludes, m.triangles.tolist()) for m in b.meshes]
    assert a.stats == b.stats and a.maps_equal(b)
    return True


def test_scenes_round_trip():
    scene = sample()
    data = f.encode(scene)
    assert data[:8] == b"DYNLIGHT" and struct.unpack("<I", data[8:12])[0] == 6
    assert data[24:34] == b"\x1f\x8b\x08\x00\x00\x00\x00\x00\x00\xff", "gzip with mtime 0 and OS 255"
    assert same(f.decode(data), scene)
    assert f.encode(scene) == data, "encoding is deterministic"
    assert same(f.decode(f.encode(empty())), empty())
    kinds = [l.shape for l in scene.lights]
    assert (sum(k not in (dl.SUN, dl.SKY) for k in kinds), sum(k in (dl.SUN, dl.SKY) for k in kinds),
            sum(k == dl.SUN for k in kinds)) == (3, 2, 1)


def invalid(scene):
    with pytest.raises(FormatError) as e:
        f.decode_payload(f.write_payload(scene))
    return e.value


def test_suns_come_last_with_one_sun_map_each_or_none():
    s = sample()
    s.lights.insert(0, sun(4))
    assert invalid(s) == FormatError("Invalid", "light order")
    s = sample()
    s.lights.append(sun(5))
    assert invalid(s) == FormatError("Invalid", "light order")
    s = sample()
    s.lights.insert(4, sun(5))
    assert invalid(s) == FormatError("Invalid", "sun map count")
    s.sun_maps = []
    f.decode_payload(f.write_payload(s))  # no maps at all is fine
    s = sample()
    s.sun_maps[0].texels = s.sun_maps[0].texels[:-1]
    assert invalid(s) == FormatError("Invalid", "sun map")


def test_sky_probes_need_a_sky_and_whole_probes():
    s = sample()
    s.lights.pop()
    assert invalid(s) == FormatError("Invalid", "sky probes")
    s.sky_probes = None
    f.decode_payload(f.write_payload(s))
    for change in ("short", "empty", "huge"):
        s = sample()
        p = s.sky_probes
        if change == "short":
            p.words = p.words[:-1]
        elif change == "empty":
            p.counts = (2, 0, 3)
        else:
            p.counts = (1 << 16,) * 3
        assert invalid(s) == FormatError("Invalid", "sky probes"), change


def test_unknown_versions_are_rejected_clearly():
    data = bytearray(f.encode(sample()))
    for version in (7, 1, 4, 5):
        data[8:12] = struct.pack("<I", version)
        with pytest.raises(FormatError) as e:
            f.decode(bytes(data))
        assert e.value == FormatError("UnsupportedVersion", found=version)
        assert e.value.supported == 6 and "re-bake" in str(e.value)


def broken_files():
    data = f.encode(sample())
    wrong_checksum, wrong_length, flipped, old = (bytearray(data) for _ in range(4))
    wrong_checksum[20] ^= 1
    wrong_length[12] ^= 1
    flipped[len(flipped) - 12] ^= 0x55
    old[8:12] = struct.pack("<I", 5)
    return data, [bytes(wrong_checksum), bytes(wrong_length), bytes(flipped), bytes(old), data[:10], data[:-3],
                  b"PNG\0\0\0\0\0garbage-garbage-garbage"]


def test_corruption_is_detected():
    data, broken = broken_files()
    for bad, kind in [(b"PNG\0\0\0\0\0garbage-garbage-garbage", "NotDynlight"), (data[:10], "Truncated"),
                      (broken[0], "ChecksumMismatch")]:
        with pytest.raises(FormatError) as e:
            f.decode(bad)
        assert e.value.kind == kind
    for bad in (data[:-3], broken[1], broken[2]):
        with pytest.raises(FormatError):
            f.decode(bad)


def test_invalid_payload_values_are_rejected():
    s = sample()
    s.settings["max_lightmap_size"] = 1
    payload = bytearray(f.write_payload(s))
    payload[4] = 9
    with pytest.raises(FormatError) as e:
        f.decode_payload(bytes(payload))
    assert e.value == FormatError("Invalid", "dynamic geometry mode")
    shape = 20 + 8 + 28  # settings, the light count, then id, origin, radius and bounce bits
    payload = bytearray(f.write_payload(sample()))
    payload[shape] = 7
    with pytest.raises(FormatError) as e:
        f.decode_payload(bytes(payload))
    assert e.value == FormatError("Invalid", "light shape")
    for bits in (0, 3, 16):
        payload = bytearray(f.write_payload(sample()))
        payload[shape + 28] = bits
        with pytest.raises(FormatError) as e:
            f.decode_payload(bytes(payload))
        assert e.value == FormatError("Invalid", "shadow bits per texel")
    with pytest.raises(FormatError) as e:
        f.decode_payload(f.write_payload(sample()) + b"\0")
    assert e.value == FormatError("Invalid", "trailing payload")


class Dribble(io.RawIOBase):
    """At most 7 bytes per read, like a slow disk or network (tests.rs:297-308)."""

    def __init__(self, data):
        self.data = data

    def read(self, n=-1):
        k = min(7, len(self.data)) if n < 0 else min(n, 7, len(self.data))
        out, self.data = self.data[:k], self.data[k:]
        return out


def test_streamed_and_whole_buffer_reads_agree():
    big = sample()
    big.meshes = [dl.BakedMesh(i + 1, i, 8, (np.arange(10_000 + i, dtype=np.uint64) * 2_654_435_761 % (1 << 32))
                               .astype(np.uint32), i % 2 == 0) for i in range(5)]
    for scene in (sample(), empty(), big):
        data = f.encode(scene)
        whole = f.decode(data)
        assert same(whole, scene)
        assert same(f.decode_stream(io.BytesIO(data)), whole)
        assert same(f.decode_stream(Dribble(data)), whole)


def test_streamed_reads_report_the_same_errors():
    _, broken = broken_files()
    for bad in broken:
        with pytest.raises(FormatError) as whole:
            f.decode(bad)
        with pytest.raises(FormatError) as streamed:
            f.decode_stream(io.BytesIO(bad))
        assert streamed.value == whole.value, (whole.value.kind, streamed.value.kind)


def test_payload_writer_matches_the_library_writer():
    # the same bytes as dl_encode_payload (C++) for an oracle bake with every light kind and maps
    if not os.path.exists(dl.LIBRARY_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    inp, opts = fx.determinism_room()
    opts.dynamic_geometry, opts.sun_map_resolution, opts.sky_probe_spacing = dl.ANGULAR, 64, 0.75
    m, copts = dl.Marshalled(inp), dl.marshal_options(opts)
    out = C.POINTER(dl._abi.DlBakedScene)()
    lb = oracle.lib()
    assert lb.oracle_bake(C.byref(m.input), C.byref(copts), None, 0, 0, C.byref(out), None, None) == 0
    try:
        want, crc = dl.encode_payload(out.contents)
        scene = dl.scene_from_c(out.contents)
    finally:
        lb.oracle_free(out)
    assert scene.sun_maps and scene.sky_probes is not None and scene.distance_cubes.size
    assert f.write_payload(scene) == want and zlib.crc32(want) == crc
    assert same(f.decode(f.container(want, crc)), scene)


@pytest.mark.gpu
def test_device_payload_decodes_to_the_bake():
    inp, opts = fx.determinism_room()
    opts.dynamic_geometry, opts.sun_map_resolution, opts.sky_probe_spacing = dl.ANGULAR, 64, 0.75
    s = dl.Session(inp, opts)
    try:
        s.run()
        payload, crc = s.encode_payload()
        baked = s.result()
    finally:
        s.close()
    decoded = f.decode_stream(io.BytesIO(f.container(payload, crc)))
    assert same(decoded, baked)
    assert f.write_payload(baked) == payload
