"""GPU parity: the CUDA bake (both forms) against the oracle, word for word.

Every comparison is of the final per-mesh `dynamic_triangles` words (the per-pair shadow bit and
level layout, src/bake/triangle_words.rs:1-13) plus the bake statistics; integer outputs, so the
bar is bit-exact."""
import math

import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import scenes
from oracle import oracle

from . import fixtures as fx

pytestmark = pytest.mark.gpu


def first_difference(a, b):
    for ma, mb in zip(a.meshes, b.meshes):
        if ma.id != mb.id or ma.resolution != mb.resolution:
            return f"mesh {ma.id}/{mb.id}: resolution {ma.resolution}/{mb.resolution}"
        if len(ma.triangles) != len(mb.triangles):
            return f"mesh {ma.id}: {len(ma.triangles)} vs {len(mb.triangles)} words"
        d = np.nonzero(ma.triangles != mb.triangles)[0]
        if len(d):
            return f"mesh {ma.id}: {len(d)} words differ, first at {d[0]}"
    return None


def assert_same(got, want):
    assert len(got.meshes) == len(want.meshes)
    assert got.words_equal(want), first_difference(got, want)
    assert got.stats == want.stats
    assert [l.id for l in got.lights] == [l.id for l in want.lights]
    assert np.array_equal(got.light_bvh, want.light_bvh)
    assert got.settings == want.settings


@pytest.mark.parametrize("form", ["batched", "plain"])
def test_small_room_matches_the_oracle(form):
    inp, opts = scenes.small_room()
    want, _, _ = oracle.bake(inp, opts)
    report = dl._abi.DlBakeReport()
    got = dl.bake(inp, opts, form=form, report=report)
    assert_same(got, want)
    assert report.kernel_launches > 0 and report.shadow_rays == want.stats["rays"]


@pytest.mark.parametrize("form", ["batched", "plain"])
def test_mixed_lights_match_the_oracle(form):
    # points, a panel, a tube, a soft and a hard sun, a sky (src/bake/tests/determinism.rs:11-44)
    inp, opts = fx.determinism_room()
    want, _, _ = oracle.bake(inp, opts)
    got = dl.bake(inp, opts, form=form)
    assert_same(got, want)
    bits = sorted({l.shadow_bits_per_texel for l in got.lights})
    assert bits == [1, 4, 8]


def test_soft_rooms_batched_and_plain_agree_with_the_oracle():
    inp, opts = scenes.soft_rooms(rooms=2, lights=24, boxes_per_room=6)
    want, _, _ = oracle.bake(inp, opts)
    batched = dl.bake(inp, opts, form="batched")
    plain = dl.bake(inp, opts, form="plain")
    assert_same(batched, want)
    assert_same(plain, want)


def test_outdoor_slice_with_sun_sky_and_colored_sun_bounce():
    inp, opts = scenes.outdoor(grid=65, chunks=2, boxes=40, point_lights=6, sky_samples=32,
                               bounce_samples=8)
    want, _, _ = oracle.bake(inp, opts)
    got = dl.bake(inp, opts)
    assert got.settings["bounce"] and got.settings["colored_bounce"]
    assert_same(got, want)


@pytest.mark.parametrize("compression", [8, 6, 4])
def test_local_light_bounce_matches_the_oracle(compression):
    # photon cubes, slerp gathers, last-triangle-wins maps, dilate/blur, dithered packing
    inp, opts = scenes.room_grid(rooms=2, lights=6, boxes_per_room=6, samples=16)
    opts.photon_cube_resolution = 64
    opts.bounce_compression = compression
    want, _, _ = oracle.bake(inp, opts)
    report = dl._abi.DlBakeReport()
    got = dl.bake(inp, opts, report=report)
    assert want.stats["bounce_rays"] > 0
    assert_same(got, want)
    assert report.photon_rays == 6 * 64 * 64 * 6


def test_colored_bounce_with_mixed_lights():
    inp, opts = fx.determinism_room()
    for l in inp.lights:
        if l.shape.kind != dl.SKY:
            l.illumination = dl.SINGLE_BOUNCE
            l.bounce = dl.BakeBounce(samples=12, intensity=1.5, compression=5 if l.id % 20 == 0 else None)
    opts.colored_bounce = True
    opts.photon_cube_resolution = 48
    want, _, _ = oracle.bake(inp, opts)
    for form in ("batched", "plain"):
        assert_same(dl.bake(inp, opts, form=form), want)


def test_alpha_tested_shadows():
    # a half-transparent plane (src/bake/tests/occluder.rs:85-98) over a floor
    plane = fx.floor(1, (0, 1.0, 0), 1.0)
    plane.uv0 = plane.uv1.copy()
    plane.alpha = dl.AlphaTexture(2, 1, np.array([255, 255, 255, 0, 255, 255, 255, 255], np.uint8))
    ground = fx.floor(2, (0, 0, 0), 2.0)
    lights = [fx.point_light(5, (0.1, 3.0, 0.2), 6.0, transparency=dl.TRANSPARENCY_ENABLED),
              fx.point_light(6, (0.3, 2.5, -0.2), 6.0)]
    inp = dl.BakeInput([plane, ground], lights)
    opts = fx.options(pixel_density=16.0)
    want, _, _ = oracle.bake(inp, opts)
    assert_same(dl.bake(inp, opts), want)


def test_thin_and_buried_geometry():
    # a pipe strip narrower than a texel and a box sunk into the floor
    # (src/bake/tests/coverage.rs:63-160 cover both cases)
    strip = dl.BakeMesh(id=3, positions=np.float32([[0, 0.5, 0], [2, 0.5, 0], [2, 0.5, 0.02], [0, 0.5, 0.02]]),
                        indices=np.uint32([0, 2, 1, 0, 3, 2]),
                        uv1=np.float32([[0.1, 0.1], [0.9, 0.1], [0.9, 0.103], [0.1, 0.103]]))
    sunk = fx.cuboid(4, (-1.0, -0.5, -1.0), (-0.2, 0.3, -0.2))
    ground = fx.floor(2, (0, 0, 0), 2.0)
    inp = dl.BakeInput([strip, sunk, ground], [fx.point_light(9, (0.5, 2.0, 0.5), 5.0)])
    opts = fx.options(pixel_density=24.0)
    want, burial, _ = oracle.bake(inp, opts)
    assert burial > 0
    assert_same(dl.bake(inp, opts), want)


def test_empty_and_lightless_scenes():
    empty, opts = dl.BakeInput(), fx.options(pixel_density=12.0)
    got = dl.bake(empty, opts)
    assert got.meshes == [] and got.lights == [] and len(got.light_bvh) == 0
    lone = dl.BakeInput([fx.floor(1, (0, 0, 0), 1.0)], [])
    got = dl.bake(lone, opts)
    want, _, _ = oracle.bake(lone, opts)
    assert_same(got, want)
    assert got.meshes[0].triangle_count() == 2


@pytest.mark.parametrize("form", ["batched", "plain"])
def test_two_triangle_scene_whose_bvh_root_is_a_leaf(form):
    # one mesh of two triangles (a floor and a wall leaning over it): the occluder BVH is a single
    # leaf beside an empty child; shadow, sky, soft sun and bounce rays all traverse it
    pos = np.array([(-2, 0, -2), (2, 0, -2), (0, 0, 2), (-1.5, 0.2, 0.5), (1.5, 0.2, 0.5), (0, 2.5, -0.5)],
                   np.float32)
    uv = np.array([(0, 0), (0.45, 0), (0.2, 0.9), (0.55, 0.1), (1, 0.1), (0.8, 0.9)], np.float32)
    mesh = dl.BakeMesh(id=1, positions=pos, indices=np.array([0, 2, 1, 3, 4, 5], np.uint32), uv1=uv)
    bounce = dl.BakeBounce(samples=32)
    lights = [fx.point_light(7, (0.3, 1.2, 1.5), 6.0), fx.sky_light(10),
              fx.sun_light(9, (0.2, 1.0, 0.6), 0.53, illumination=dl.SINGLE_BOUNCE, bounce=bounce)]
    inp, opts = dl.BakeInput([mesh], lights), fx.options(pixel_density=24.0, sky_samples=64, colored_bounce=True)
    want, _, _ = oracle.bake(inp, opts)
    got = dl.bake(inp, opts, form=form)
    assert_same(got, want)
    assert want.stats["rays"] > 0 and want.stats["bounce_rays"] > 0


def test_errors_mirror_the_reference():
    inp, opts = fx.determinism_room()
    inp.meshes[1].id = 5
    with pytest.raises(dl.BakeError) as e:
        dl.bake(inp, opts)
    assert e.value.kind == "DuplicateId"
    inp, opts = fx.determinism_room()
    inp.lights[0].radius = 0.0
    with pytest.raises(dl.BakeError) as e:
        dl.bake(inp, opts)
    assert e.value.kind == "InvalidLight"
    inp, opts = fx.determinism_room()
    inp.meshes[0].indices = np.append(inp.meshes[0].indices, np.uint32(99))
    with pytest.raises(dl.BakeError) as e:
        dl.bake(inp, opts)
    assert e.value.kind == "InvalidMesh"
    inp, opts = fx.determinism_room()
    opts.pixel_density = -1.0
    with pytest.raises(dl.BakeError) as e:
        dl.bake(inp, opts)
    assert e.value.kind == "InvalidOptions"


def test_cancelled_bakes_stop():
    inp, opts = fx.determinism_room()
    progress = dl.BakeProgress()
    progress.cancel()
    with pytest.raises(dl.BakeError) as e:
        dl.bake(inp, opts, progress=progress)
    assert e.value.kind == "Cancelled"


def test_sessions_repeat_identically():
    inp, opts = scenes.small_room()
    s = dl.Session(inp, opts)
    s.run()
    a = s.result()
    s.run()
    b = s.result()
    s.close()
    assert a.words_equal(b) and a.stats == b.stats


def test_bakes_after_releasing_the_cached_memory_repeat():
    # device memory that sessions free stays pooled for the next bake; dl_release_memory hands
    # it back, and the next bake allocates afresh
    inp, opts = fx.determinism_room()
    first = dl.bake(inp, opts)
    again = dl.bake(inp, opts)
    dl.load_library().dl_release_memory()
    fresh = dl.bake(inp, opts)
    assert_same(again, first)
    assert_same(fresh, first)


def test_tuning_does_not_change_the_bytes():
    # the GPU analogue of the reference's 1/4/7-thread determinism (determinism.rs:65-72)
    inp, opts = scenes.soft_rooms(rooms=2, lights=16, boxes_per_room=4)
    base = dl.bake(inp, opts)
    for tuning in [dict(chunk_texels=128), dict(blocks_per_sm=1), dict(chunk_texels=32, blocks_per_sm=2)]:
        other = dl.bake(inp, opts, **tuning)
        assert other.words_equal(base) and other.stats == base.stats, tuning


def test_register_budgets_do_not_change_the_bytes():
    # every register budget the tuners may pick (the same kernel compiled for 7 to 12 resident
    # blocks per SM, spilling more at the smaller budgets) writes the default budget's bytes,
    # sky, sun and both bounce kinds included
    rooms = scenes.room_grid(rooms=1, lights=4, boxes_per_room=3, samples=24)
    rooms[1].photon_cube_resolution = 48
    outdoor = scenes.outdoor(grid=33, chunks=2, boxes=12, point_lights=2, sky_samples=32, bounce_samples=64)
    for inp, opts in (rooms, outdoor):
        base = dl.bake(inp, opts)
        for m, gm in ((8, 8), (9, 9), (10, 10), (12, 6), (7, 10)):
            report = dl._abi.DlBakeReport()
            other = dl.bake(inp, opts, min_blocks=m, gather_min_blocks=gm, report=report)
            assert_same(other, base)  # the words carry the packed bounce maps
            assert report.tuned_min_blocks == m and report.tuned_gather_min_blocks == gm


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 32])
def test_sky_sample_lanes_do_not_change_the_bytes(lanes):
    # lanes sharing one sky texel's samples: an integer sum of open samples, so the same levels
    inp, opts = fx.determinism_room()
    want, _, _ = oracle.bake(inp, opts)
    for chunk in (32, 96):
        report = dl._abi.DlBakeReport()
        got = dl.bake(inp, opts, sample_lanes=lanes, chunk_texels=chunk, report=report)
        assert_same(got, want)
        assert report.tuned_sample_lanes == lanes and report.tuned_chunk_texels == chunk


@pytest.mark.parametrize("lanes", [1, 4, 16, 32])
def test_gather_sample_lanes_do_not_change_the_bytes(lanes):
    # lanes sharing one texel's bounce samples add them in sample order: the reference's sums;
    # sun bounces of 16 to 256 samples (a power of two) are traced in the coherent net order by
    # groups of 16 or 32 lanes and still summed in sample order
    inp, opts = scenes.room_grid(rooms=1, lights=4, boxes_per_room=3, samples=24)
    opts.photon_cube_resolution = 48
    sun_inp, sun_opts = scenes.outdoor(grid=33, chunks=2, boxes=12, point_lights=2, sky_samples=16,
                                       bounce_samples=24)
    cases = [(inp, opts), (sun_inp, sun_opts)]
    cases += [scenes.outdoor(grid=33, chunks=2, boxes=12, point_lights=2, sky_samples=16, bounce_samples=n)
              for n in (16, 64, 256)]
    for case, (i, o) in enumerate(cases):
        want, _, _ = oracle.bake(i, o)
        report = dl._abi.DlBakeReport()
        got = dl.bake(i, o, sample_lanes=lanes, report=report)
        assert_same(got, want)
        assert report.tuned_gather_lanes == lanes
    for i, o in (cases[1], cases[3]):
        refined_want = oracle.bake_ex(i, o, mode=oracle.REFINED, eps=dl.DEFAULT_REFINE_EPSILON)["scene"]
        assert_same(dl.bake(i, o, form="refined", sample_lanes=lanes), refined_want)


def test_autotuned_launch_shape_gives_the_default_bytes():
    # a scene with over a million queue items, so the first run times candidate shapes
    inp, opts = scenes.outdoor(grid=193, chunks=2, boxes=150, point_lights=6, sky_samples=64, bounce_samples=16)
    report = dl._abi.DlBakeReport()
    tuned = dl.bake(inp, opts, report=report)
    assert report.work_items >= (1 << 20)
    assert report.tune_trials > 1 and report.tuned_stack_depth >= 8
    again = dl._abi.DlBakeReport()
    assert dl.bake(inp, opts, report=again).words_equal(tuned)
    assert again.tune_trials == 0  # cached for this scene shape
    assert (again.tuned_chunk_texels, again.tuned_sample_lanes) == (report.tuned_chunk_texels,
                                                                     report.tuned_sample_lanes)
    default = dl.bake(inp, opts, no_autotune=1)
    assert default.words_equal(tuned) and default.stats == tuned.stats
    fixed = dl.bake(inp, opts, sample_lanes=8, chunk_texels=64)
    assert fixed.words_equal(tuned)
    with pytest.raises(dl.BakeError):
        dl.bake(inp, opts, sample_lanes=3)
