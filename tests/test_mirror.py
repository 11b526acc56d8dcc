"""The word reader (`mirror.py`) against words written by the oracle's serializer: the reference's
reader tests (src/bake/mirror.rs:132-199), every padded texel of hard and soft grids at map edges
in both entry layouts (src/bake/tests/layout.rs:25-83), colored bounce texels that straddle
words, the distance cube fetch and probe openness. CPU only."""
import numpy as np
import pytest

from dynlight_gb300 import scenes
from dynlight_gb300.mirror import (DISTANCE_CUBE_WORDS, MAX_TRIANGLE_LIGHTS, TriangleView,
                                   distance_cube_value, probe_openness)
from oracle import oracle

M = 0xFFFFFFFF
NONE = 0xFFFFFFFF


def serialize(records, bounce_layout):
    """records: [(crop (min_x, min_y, max_x, max_y), [(light, shadow words or None, bounce words
    or None)])] -> the mesh's words, from the oracle's serializer (triangle_words.rs)."""
    crops, counts, entries, payload = [], [], [], []
    for crop, lights in records:
        crops += list(crop)
        counts.append(len(lights))
        for light, shadow, bounce in lights:
            entries += [light, NONE if shadow is None else len(shadow), NONE if bounce is None else len(bounce)]
            payload += list(shadow or []) + list(bounce or [])
    arrays = [np.ascontiguousarray(np.asarray(a or [0], np.uint32)) for a in (crops, counts, entries, payload)]
    cap = 4 * len(records) + len(entries) + len(payload) + len(records) + 16
    out = np.zeros(cap, np.uint32)
    n = oracle.lib().oracle_serialize(len(records), *(oracle.ptr(a) for a in arrays), 1 if bounce_layout else 0,
                                      cap, oracle.ptr(out))
    assert n <= cap
    return out[:n]


def pack(levels, bits):
    """Row-major levels, `bits` each, LSB first, 32 // bits per word (bits.rs, shadow_grid.rs)."""
    per = 32 // bits
    words = [0] * -(-len(levels) // per)
    for i, level in enumerate(levels):
        words[i // per] |= int(level) << ((i % per) * bits)
    return words


def test_reads_back_what_the_builder_wrote():
    # mirror.rs:136-171: a padded 7x7 grid of crop (1, 0)-(3, 2) with lightmap texel (2, 1) lit
    grid = [0] * 49
    grid[3 * 7 + 3] = 1
    words = serialize([((1, 0, 3, 2), [(9, pack(grid, 1), [0x04030201, 0x08070605])])], True)
    v = TriangleView.load(words, 0, True)
    assert v.light_count == 1 and v.bounds == (M, M - 1, 7)
    e = v.light(0)
    assert e.light_index == 9
    assert v.shadow_bit(e, 2, 1) is True and v.shadow_bit(e, 1, 1) is False
    assert v.shadow_bit(e, M, M - 1) is False  # lightmap (-1, -2): local (0, 0) by wrapping
    assert v.bounce_texel(e, (5 + v.bounds[0]) & M, v.bounds[1], 8) == np.float32(6.0) / np.float32(255.0)


def test_soft_shadows_read_back_as_fractions():
    # mirror.rs:173-198: a padded 6x6 grid of 4-bit levels; lightmap (0, 0) is local (2, 2)
    grid = [0] * 36
    grid[2 * 6 + 2], grid[2 * 6 + 3] = 15, 5
    words = serialize([((0, 0, 1, 1), [(0, pack(grid, 4), None)])], False)
    v = TriangleView.load(words, 0, False)
    e = v.light(0)
    assert v.shadow_value(e, 0, 0, 4) == 1.0
    assert v.shadow_value(e, 1, 0, 4) == np.float32(5.0) / np.float32(15.0)
    assert v.shadow_value(e, 0, 1, 4) == 0.0


@pytest.mark.parametrize("bits", [1, 4, 8])
@pytest.mark.parametrize("bounce_layout", [False, True])
def test_every_padded_texel_reads_back(bits, bounce_layout):
    # layout.rs:25-83: triangles at the map's edges (x = 0, y = 0) and inside, pseudo-random levels
    crops = [(0, 0, 4, 2), (7, 3, 15, 20), (20, 0, 23, 23)]
    top = (1 << bits) - 1
    grids, records = [], []
    for i, (x0, y0, x1, y1) in enumerate(crops):
        w, h = x1 - x0 + 5, y1 - y0 + 5
        levels = [min(scenes.splitmix64(1000 * i + k) % (top + 2), top) for k in range(w * h)]
        grids.append((w, h, levels))
        records.append(((x0, y0, x1, y1), [(3 * i, pack(levels, bits), [7] if bounce_layout else None)]))
    words = serialize(records, bounce_layout)
    for t, ((x0, y0, _, _), (w, h, levels)) in enumerate(zip(crops, grids)):
        v = TriangleView.load(words, t, bounce_layout)
        e = v.light(0)
        assert e.light_index == 3 * t and (e.bounce_offset != 0) == bounce_layout
        for y in range(h):
            for x in range(w):
                got = v.shadow_value(e, (x0 + x - 2) & M, (y0 + y - 2) & M, bits)
                assert got == float(np.float32(levels[y * w + x]) / np.float32(top)), (t, x, y)


@pytest.mark.parametrize("bits", [4, 5, 6, 8])
def test_colored_bounce_texels_straddle_words(bits):
    # bounce_texel_rgb (mirror.rs:96-117): 3 * bits per pixel, packed back to back
    crop = (2, 3, 9, 7)
    w, h = crop[2] - crop[0] + 5, crop[3] - crop[1] + 5
    top = (1 << bits) - 1
    rgb = [[scenes.splitmix64(3 * k + c) % (top + 1) for c in range(3)] for k in range(w * h)]
    stream = 0
    for k, (r, g, b) in enumerate(rgb):
        stream |= (r | g << bits | b << (2 * bits)) << (3 * bits * k)
    nwords = -(-3 * bits * w * h // 32)
    bounce = [(stream >> (32 * i)) & M for i in range(nwords)]
    words = serialize([(crop, [(4, pack([1] * (w * h), 1), bounce)])], True)
    v = TriangleView.load(words, 0, True)
    e = v.light(0)
    for y in range(h):
        for x in range(w):
            got = v.bounce_texel_rgb(e, (crop[0] + x - 2) & M, (crop[1] + y - 2) & M, bits)
            want = tuple(float(np.float32(c) / np.float32(top)) for c in rgb[y * w + x])
            assert got == want, (x, y)


def test_light_counts_are_clamped_like_the_shader():
    words = serialize([((0, 0, 1, 1), [(1, pack([1] * 36, 1), None)])], False)
    words[words[0]] = 1000  # a corrupt light count
    assert TriangleView.load(words, 0, False).light_count == MAX_TRIANGLE_LIGHTS


def test_distance_cube_values_and_probe_openness():
    rng = np.random.default_rng(7)
    halves = rng.uniform(0.0, 60.0, 2 * 2 * DISTANCE_CUBE_WORDS).astype(np.float16)
    cubes = halves.view(np.uint32)  # two lights, little-endian f16 pairs
    for light, index in [(0, 0), (0, 1), (1, 12345), (1, 2 * DISTANCE_CUBE_WORDS - 1)]:
        assert distance_cube_value(cubes, light, index) == float(halves[light * 2 * DISTANCE_CUBE_WORDS + index])

    class Probes:
        counts = (3, 2, 4)
        words = None
    bytes_ = rng.integers(0, 256, (4, 2, 3, 8), dtype=np.uint32)
    bytes_[..., 6:] = 0
    Probes.words = (bytes_.reshape(-1, 2, 4) << (8 * np.arange(4, dtype=np.uint32))).sum(-1).astype(np.uint32).reshape(-1)
    for x, y, z in [(0, 0, 0), (2, 1, 3), (1, 0, 2)]:
        want = [float(np.float32(b) / np.float32(255.0)) for b in bytes_[z, y, x, :6]]
        assert probe_openness(Probes, x, y, z) == want
