"""GPU precision forms: the refined form (binary64 re-tests of near-boundary ray/triangle tests,
Kahan sums) against the oracle's refined mode, word for word and bounce map for bounce map;
the bit-exact forms' bounce maps against the binary32 oracle; and the precision report (bit
flips and bounce error of each form against the FP64 oracle) on a slice of the precision-stress
scene."""
import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import compare, scenes
from oracle import oracle

from . import fixtures as fx
from .test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def _stress_slice():
    return scenes.precision_stress(grid=64, chunks=2, boxes=20, decals=2000, slivers=300, lights=24,
                                   sky_samples=32, bounce_samples=16)


@pytest.fixture(scope="module")
def stress():
    inp, opts = _stress_slice()
    bakes = {name: oracle.bake_ex(inp, opts, mode=mode, eps=dl.DEFAULT_REFINE_EPSILON, bounce_maps=True)
             for name, mode in (("f32", oracle.F32), ("refined", oracle.REFINED), ("f64", oracle.F64))}
    return inp, opts, bakes


def _gpu(inp, opts, form, **tuning):
    s = dl.Session(inp, opts, form=form, **tuning)
    try:
        s.run()
        scene = s.result()
        return scene, compare.session_maps(s, scene), s.report()
    finally:
        s.close()


def _maps_equal(got, want):
    assert set(got) == set(want)
    for key, (rect, v) in want.items():
        grect, gv = got[key]
        assert grect == rect, key
        assert np.array_equal(gv.view(np.uint32), v.view(np.uint32)), key


@pytest.mark.parametrize("form", ["batched", "plain"])
def test_bit_exact_forms_and_their_bounce_maps_match_the_binary32_oracle(stress, form):
    inp, opts, bakes = stress
    scene, maps, report = _gpu(inp, opts, form)
    assert_same(scene, bakes["f32"]["scene"])
    _maps_equal(maps, bakes["f32"]["maps"])
    assert report.retests == 0


def test_refined_form_matches_the_refined_oracle(stress):
    inp, opts, bakes = stress
    scene, maps, report = _gpu(inp, opts, "refined")
    assert_same(scene, bakes["refined"]["scene"])
    _maps_equal(maps, bakes["refined"]["maps"])
    assert report.retests > 0


def test_bounce_refined_form_matches_its_oracle_and_keeps_the_exact_masks(stress):
    """The bounce-refined form against the oracle's bounce-refined mode, word for word and bounce
    map for bounce map; its masks equal the batched form's bit for bit and its bounce is within
    1e-4 of the FP64 oracle, the two clauses of the target in one bake."""
    inp, opts, bakes = stress
    want = oracle.bake_ex(inp, opts, mode=oracle.REFINED_BOUNCE, eps=dl.DEFAULT_REFINE_EPSILON, bounce_maps=True)
    scene, maps, report = _gpu(inp, opts, "bounce_refined")
    assert_same(scene, want["scene"])
    _maps_equal(maps, want["maps"])
    assert report.retests > 0
    exact, _, _ = _gpu(inp, opts, "batched")
    flips = compare.bit_flips(scene, exact)
    assert all(v["flips"] == 0 for k, v in flips.items() if k != "bounce"), flips
    err = compare.bounce_error(maps, bakes["f64"]["maps"])
    assert err["maps"] > 0 and err["max"] <= 1e-4, err
    # every light kind, with a local and a sun bounce
    inp, opts = fx.determinism_room()
    for light, n in ((inp.lights[0], 16), (inp.lights[7], 32)):
        light.illumination = dl.SINGLE_BOUNCE
        light.bounce = dl.BakeBounce(samples=n)
    opts.photon_cube_resolution = 64
    want = oracle.bake_ex(inp, opts, mode=oracle.REFINED_BOUNCE, eps=dl.DEFAULT_REFINE_EPSILON)["scene"]
    got, _, _ = _gpu(inp, opts, "bounce_refined")
    assert_same(got, want)


@pytest.mark.parametrize("eps", [1e-7, 1e-6, 1e-5])
def test_refined_epsilon_sweep_matches_the_oracle(eps):
    inp, opts = scenes.precision_stress(grid=40, chunks=2, boxes=8, decals=600, slivers=120, lights=10,
                                        sky_samples=16, bounce_samples=8)
    want = oracle.bake_ex(inp, opts, mode=oracle.REFINED, eps=eps)["scene"]
    got, _, _ = _gpu(inp, opts, "refined", refine_epsilon=eps)
    assert_same(got, want)


def test_refined_form_on_mixed_lights_and_alpha():
    # every light kind (src/bake/tests/determinism.rs:11-44) and an alpha-tested occluder
    inp, opts = fx.determinism_room()
    want = oracle.bake_ex(inp, opts, mode=oracle.REFINED, eps=dl.DEFAULT_REFINE_EPSILON)["scene"]
    got, _, _ = _gpu(inp, opts, "refined")
    assert_same(got, want)
    plane = fx.floor(1, (0, 1.0, 0), 1.0)
    plane.uv0 = plane.uv1.copy()
    plane.alpha = dl.AlphaTexture(2, 1, np.array([255, 255, 255, 0, 255, 255, 255, 255], np.uint8))
    inp = dl.BakeInput([plane, fx.floor(2, (0, 0, 0), 2.0)],
                       [fx.point_light(5, (0.1, 3.0, 0.2), 6.0, transparency=dl.TRANSPARENCY_ENABLED)])
    opts = fx.options(pixel_density=16.0)
    want = oracle.bake_ex(inp, opts, mode=oracle.REFINED, eps=dl.DEFAULT_REFINE_EPSILON)["scene"]
    got, _, _ = _gpu(inp, opts, "refined")
    assert_same(got, want)


def test_precision_report_against_the_fp64_oracle(stress):
    inp, opts, bakes = stress
    plain, plain_maps, _ = _gpu(inp, opts, "batched")
    refined, refined_maps, _ = _gpu(inp, opts, "refined")
    f64, f64_maps = bakes["f64"]["scene"], bakes["f64"]["maps"]
    flips_plain = compare.bit_flips(plain, f64)
    flips_refined = compare.bit_flips(refined, f64)
    total = lambda f: sum(v["flips"] for v in f.values())
    assert total(flips_refined) <= total(flips_plain)
    err_refined = compare.bounce_error(refined_maps, f64_maps)
    assert err_refined["max"] <= 1e-4
    # the bit-exact form against the reference restatement: no flips at all
    assert total(compare.bit_flips(plain, bakes["f32"]["scene"])) == 0
