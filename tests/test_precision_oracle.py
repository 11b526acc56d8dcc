"""The oracle's precision modes (CPU): the reference's binary32, the refined form (binary64
re-tests of near-boundary ray/triangle tests, Kahan sums) and the FP64 oracle, plus the output
comparison that counts bit flips between bakes."""
import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import compare, scenes
from oracle import oracle


def _triangles(rng, n):
    """n well-shaped triangles (every altitude at least 0.2 of the longest edge)."""
    out = []
    while sum(len(t) for t in out) < n:
        v0 = rng.uniform(-5, 5, (n, 3))
        tri = np.stack([v0, v0 + rng.uniform(-3, 3, (n, 3)), v0 + rng.uniform(-3, 3, (n, 3))], 1)
        tri = tri.astype(np.float32).astype(np.float64)
        area2 = np.linalg.norm(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]), axis=1)
        longest = np.max([np.linalg.norm(tri[:, (k + 1) % 3] - tri[:, k], axis=1) for k in range(3)], axis=0)
        out.append(tri[area2 / longest >= 0.2 * longest])
    tri = np.concatenate(out)[:n]
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return tri, nrm


def _rays_at(rng, points, nrm):
    """Rays from 1..5 m away through `points`, at least 0.3 off the triangles' planes."""
    n = len(points)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    cos = np.einsum("ij,ij->i", d, nrm)
    d = d + nrm * (np.sign(cos) * 0.3)[:, None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    length = rng.uniform(1, 5, n)
    origin = points - d * length[:, None]
    return origin.astype(np.float32), d.astype(np.float32), (2 * length).astype(np.float32)


def test_rays_through_edges_take_the_binary64_verdict():
    rng = np.random.default_rng(5)
    n = 20000
    tri, nrm = _triangles(rng, n)
    s = rng.uniform(0.1, 0.9, n)[:, None]
    edge = rng.integers(0, 3, n)
    a = tri[np.arange(n), edge]
    b = tri[np.arange(n), (edge + 1) % 3]
    points = a + s * (b - a)  # on an edge, up to binary32 rounding
    o, d, mx = _rays_at(rng, points, nrm)
    h32, _, r32 = oracle.intersect_batch(oracle.F32, 1e-5, tri, o, d, mx)
    href, _, rref = oracle.intersect_batch(oracle.REFINED, 1e-5, tri, o, d, mx)
    h64, _, _ = oracle.intersect_batch(oracle.F64, 1e-5, tri, o, d, mx)
    assert r32 == 0 and rref == n  # every such ray lands in the margin
    assert np.array_equal(href, h64)
    assert np.count_nonzero(h32 != h64) > 0  # binary32 alone misjudges some edge rays


def test_rays_through_interiors_never_retest():
    rng = np.random.default_rng(6)
    n = 20000
    tri, nrm = _triangles(rng, n)
    w = rng.uniform(0.2, 0.6, (n, 2))
    points = tri[:, 0] + w[:, :1] * (tri[:, 1] - tri[:, 0]) + (w[:, 1:] * 0.5) * (tri[:, 2] - tri[:, 0])
    o, d, mx = _rays_at(rng, points, nrm)
    h32, t32, _ = oracle.intersect_batch(oracle.F32, 1e-5, tri, o, d, mx)
    href, tref, rref = oracle.intersect_batch(oracle.REFINED, 1e-5, tri, o, d, mx)
    h64, t64, _ = oracle.intersect_batch(oracle.F64, 1e-5, tri, o, d, mx)
    assert rref == 0
    assert h32.all() and np.array_equal(h32, href) and np.array_equal(href, h64)
    assert np.array_equal(t32, tref)  # outside the margins the refined hit is the binary32 hit
    assert np.allclose(t32, t64, rtol=1e-5)


def test_the_margin_grows_with_epsilon():
    rng = np.random.default_rng(7)
    n = 20000
    tri, nrm = _triangles(rng, n)
    w = rng.uniform(-0.01, 1.01, (n, 2))
    points = tri[:, 0] + w[:, :1] * (tri[:, 1] - tri[:, 0]) + w[:, 1:] * (tri[:, 2] - tri[:, 0])
    o, d, mx = _rays_at(rng, points, nrm)
    counts = [oracle.intersect_batch(oracle.REFINED, eps, tri, o, d, mx)[2]
              for eps in (1e-7, 1e-6, 1e-5, 1e-4)]
    assert counts == sorted(counts) and counts[-1] > counts[0]


def _stress():
    return scenes.precision_stress(grid=48, chunks=2, boxes=12, decals=1200, slivers=200, lights=12,
                                   sky_samples=16, bounce_samples=8)


@pytest.fixture(scope="module")
def stress_bakes():
    inp, opts = _stress()
    return inp, opts, {name: oracle.bake_ex(inp, opts, mode=mode, eps=1e-5, bounce_maps=True)
                       for name, mode in (("f32", oracle.F32), ("refined", oracle.REFINED),
                                          ("f64", oracle.F64), ("bounce", oracle.REFINED_BOUNCE))}


def _total(flips):
    return sum(v["flips"] for v in flips.values())


def test_binary32_mode_is_the_reference_oracle(stress_bakes):
    inp, opts, bakes = stress_bakes
    plain, _, _ = oracle.bake(inp, opts)
    assert plain.words_equal(bakes["f32"]["scene"])
    assert bakes["f32"]["retests"] == 0


def test_refined_mode_is_closer_to_fp64(stress_bakes):
    _, _, bakes = stress_bakes
    assert bakes["refined"]["retests"] > 0
    f32_flips = compare.bit_flips(bakes["f32"]["scene"], bakes["f64"]["scene"])
    ref_flips = compare.bit_flips(bakes["refined"]["scene"], bakes["f64"]["scene"])
    assert _total(ref_flips) <= _total(f32_flips)
    err = compare.bounce_error(bakes["refined"]["maps"], bakes["f64"]["maps"])
    assert err["maps"] > 0 and err["max"] <= 1e-4
    # every mode samples the same rays, so the statistics agree
    assert bakes["refined"]["scene"].stats == bakes["f32"]["scene"].stats == bakes["f64"]["scene"].stats


def test_bounce_refined_mode_keeps_the_binary32_masks(stress_bakes):
    """The bounce-refined form: its masks are the reference restatement's bit for bit (binary32
    visibility and burial), its bounce is the refined form's (refined photons and gathers, Kahan
    sums), so one bake meets both clauses: bit-identical masks and bounce near FP64."""
    _, _, bakes = stress_bakes
    hybrid, f32 = bakes["bounce"]["scene"], bakes["f32"]["scene"]
    flips = compare.bit_flips(hybrid, f32)
    assert {k: v["flips"] for k, v in flips.items() if k != "bounce"} == {k: 0 for k in flips if k != "bounce"}
    assert bakes["bounce"]["retests"] > 0
    err = compare.bounce_error(bakes["bounce"]["maps"], bakes["f64"]["maps"])
    assert err["maps"] > 0 and err["max"] <= 1e-4
    assert hybrid.stats == f32.stats


def test_bit_flips_count_planted_differences(stress_bakes):
    _, _, bakes = stress_bakes
    a = bakes["f32"]["scene"]
    assert _total(compare.bit_flips(a, a)) == 0
    # plant a mistake in a copy of the oracle's output: flip 3 bits of one shadow payload word
    b = dl.BakedScene(a.settings, a.lights, a.light_bvh,
                      [dl.BakedMesh(m.id, m.content_hash, m.resolution, m.triangles.copy(), m.occludes)
                       for m in a.meshes], a.distance_cubes, a.stats)
    ent = compare.entries(a)
    key = next(k for k, v in ent.items() if v[0] is not None and len(v[0]))
    mesh = next(m for m in b.meshes if m.id == key[0])
    words = mesh.triangles
    tri = key[1]
    off = int(words[4 * tri])
    stride = 3 if a.settings["bounce"] else 2
    for k in range(int(words[off])):
        e = off + 1 + k * stride
        if int(words[e]) == key[2]:
            words[int(words[e + 1])] ^= np.uint32(0b10110)
    flips = compare.bit_flips(b, a)
    cls = f"{a.lights[key[2]].shadow_bits_per_texel}-bit"
    assert flips[cls]["flips"] == 3 and flips[cls]["entries"] == 1
    assert _total(flips) == 3
