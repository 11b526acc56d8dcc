"""The bake at the full sizes of the benchmark configurations: the outdoor scene against the
oracle word for word, and properties that do not depend on size — the batched and plain forms
agree word for word (two different schedules of the same per-texel work), launch shapes and
sample orders change no byte, a session repeats identically, the occluder BVH built on the
device and on the host gives the same bytes, and the payload encoded next to the resident words
equals the host encoding with zlib's CRC-32."""
import zlib

import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import scenes

from .test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def outdoor():
    return scenes.outdoor()  # C4: 546k triangles, sun + sky + 32 points, colored sun bounce


def test_outdoor_matches_the_oracle_at_full_size(outdoor):
    # the oracle on every host core (about 90 s on 16 cores): every word and statistic
    import os
    from oracle import oracle
    inp, opts = outdoor
    got = dl.bake(inp, opts)
    want, _, _ = oracle.bake(inp, opts, threads=os.cpu_count() or 1)
    assert_same(got, want)


def test_outdoor_forms_and_launch_shapes_agree(outdoor):
    inp, opts = outdoor
    batched = dl.bake(inp, opts)
    assert sum(len(m.triangles) for m in batched.meshes) > 100_000_000
    assert_same(dl.bake(inp, opts, form="plain"), batched)
    # one lane per texel and the widest groups; no autotuning
    assert_same(dl.bake(inp, opts, sample_lanes=1, chunk_texels=64), batched)
    assert_same(dl.bake(inp, opts, sample_lanes=16), batched)
    assert_same(dl.bake(inp, opts, no_autotune=1), batched)


def test_outdoor_session_repeats_and_device_payload(outdoor):
    import ctypes as C
    inp, opts = outdoor
    s = dl.Session(inp, opts)
    try:
        s.run()
        first = s.result()
        s.run()
        assert_same(s.result(), first)
        payload, crc = s.encode_payload()
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


@pytest.mark.parametrize("name", ["room_grid", "soft_rooms"])
def test_room_configurations_forms_agree(name):
    inp, opts = getattr(scenes, name)()  # C2 (one bounce, 512^2 photon cubes) and C3 (soft lights)
    assert_same(dl.bake(inp, opts, form="plain"), dl.bake(inp, opts))


def test_precision_stress_bvh_builders_agree():
    # C5: 2.5 M triangles with decals 1e-4 m above the terrain and slivers up to 1e4:1
    inp, opts = scenes.precision_stress()
    device_tree = dl.Session(inp, opts)
    host_tree = dl.Session(inp, opts, host_bvh=1)
    try:
        nd, td, dd = device_tree.occluder_bvh()
        nh, th, dh = host_tree.occluder_bvh()
        assert dd == dh and (nd == nh).all() and (td.view("u4") == th.view("u4")).all()
        device_tree.run()
        host_tree.run()
        assert_same(device_tree.result(), host_tree.result())
    finally:
        device_tree.close()
        host_tree.close()
