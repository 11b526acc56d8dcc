"""The golden bake cases: small seeded scenes that cover every light kind, both bounce kinds, alpha
tests, burial, the maps for moving meshes and the refined form, and the digest of a bake that the
fixture file `bakes.json` stores for each.

A digest holds the baked settings (BakedSettings, src/bake/format/types.rs:139-153); per mesh
its id, lightmap resolution, word count and the SHA-256 of its `dynamic_triangles` words
(little-endian u32, the layout of src/bake/triangle_words.rs:1-13); the bake statistics; the
lights in slot order with their shadow and bounce bits and a SHA-256 over the binary32 bits of
their transforms; the SHA-256 of the light BVH words; and the SHA-256 of the distance cubes, sun
maps and sky probes (src/bake/format/types.rs:72-128). Integer outputs and float bit patterns
only, so an equal digest is a bit-exact bake.

`make_golden.py` writes the fixtures from the oracle; `tests/test_golden_bakes.py` checks the
oracle (CPU) and the CUDA forms (GPU) against them."""
import hashlib

import numpy as np

import dynlight_gb300 as dl
from dynlight_gb300 import scenes

from .. import fixtures as fx


def _sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<"), copy=False).tobytes())
    return h.hexdigest()


def _f32_bits(values):
    return np.asarray(values, np.float32).view(np.uint32)


def digest(scene):
    """The fixture record of a BakedScene (see the module docstring)."""
    meshes = [[m.id, m.resolution, int(len(m.triangles)), _sha(m.triangles.astype(np.uint32))]
              for m in scene.meshes]
    lights = [[l.id, l.shape, l.shadow_bits_per_texel, l.bounce_bits] for l in scene.lights]
    light_floats = [_f32_bits(list(l.origin) + [l.radius] + list(l.rotation) + list(l.size))
                    for l in scene.lights]
    maps = [scene.distance_cubes.astype(np.uint32)]
    for s in scene.sun_maps:
        maps += [np.uint32([s.resolution]), s.rows.astype(np.float32).view(np.uint32), s.texels.astype(np.uint32)]
    p = scene.sky_probes
    if p is not None:
        maps += [_f32_bits(list(p.origin) + [p.spacing]), np.uint32(p.counts), p.words.astype(np.uint32)]
    settings = {k: (f"f32:{int(_f32_bits(v)):08x}" if isinstance(v, float) else int(v))
                for k, v in sorted(scene.settings.items())}
    return {
        "settings": settings,
        "meshes": meshes,
        "stats": {k: int(v) for k, v in sorted(scene.stats.items())},
        "lights": lights,
        "light_floats_sha256": _sha(*light_floats) if light_floats else _sha(np.zeros(0, np.uint32)),
        "light_bvh_sha256": _sha(np.asarray(scene.light_bvh, np.uint32).reshape(-1)),
        "maps_sha256": _sha(*maps),
        "sun_maps": len(scene.sun_maps),
        "sky_probes": p is not None,
    }


# ---- the cases: name -> () -> (BakeInput, BakeOptions, form) ------------------------------------
# `form` is "exact" (the batched and plain forms and the binary32 oracle) or "refined" (the
# refined form and the oracle's refined mode at the default epsilon).

def _small_room():
    inp, opts = scenes.small_room()  # C1 shape: one room, 4 point lights
    return inp, opts, "exact"


def _mixed_lights():
    # points, a panel, a tube, a soft and a hard sun, a sky (src/bake/tests/determinism.rs:11-44)
    inp, opts = fx.determinism_room()
    return inp, opts, "exact"


def _soft_rooms():
    inp, opts = scenes.soft_rooms(rooms=2, lights=24, boxes_per_room=6)
    return inp, opts, "exact"


def _outdoor_slice():
    # sun + sky + points with the colored sun bounce on a terrain slice
    inp, opts = scenes.outdoor(grid=65, chunks=2, boxes=40, point_lights=6, sky_samples=32, bounce_samples=32)
    return inp, opts, "exact"


def _local_bounce():
    # photon cubes, slerp gathers, dithered packing at 6 bits
    inp, opts = scenes.room_grid(rooms=2, lights=6, boxes_per_room=6, samples=16)
    opts.photon_cube_resolution = 64
    opts.bounce_compression = 6
    return inp, opts, "exact"


def _colored_mixed_bounce():
    inp, opts = fx.determinism_room()
    for l in inp.lights:
        if l.shape.kind != dl.SKY:
            l.illumination = dl.SINGLE_BOUNCE
            l.bounce = dl.BakeBounce(samples=12, intensity=1.5, compression=5 if l.id % 20 == 0 else None)
    opts.colored_bounce = True
    opts.photon_cube_resolution = 48
    return inp, opts, "exact"


def _alpha_shadows():
    # a half-transparent plane (src/bake/tests/occluder.rs:85-98) over a floor
    plane = fx.floor(1, (0, 1.0, 0), 1.0)
    plane.uv0 = plane.uv1.copy()
    plane.alpha = dl.AlphaTexture(2, 1, np.array([255, 255, 255, 0, 255, 255, 255, 255], np.uint8))
    ground = fx.floor(2, (0, 0, 0), 2.0)
    lights = [fx.point_light(5, (0.1, 3.0, 0.2), 6.0, transparency=dl.TRANSPARENCY_ENABLED),
              fx.point_light(6, (0.3, 2.5, -0.2), 6.0)]
    return dl.BakeInput([plane, ground], lights), fx.options(pixel_density=16.0), "exact"


def _thin_and_buried():
    # a strip narrower than a texel and a box sunk into the floor (src/bake/tests/coverage.rs:63-160)
    strip = dl.BakeMesh(id=3, positions=np.float32([[0, 0.5, 0], [2, 0.5, 0], [2, 0.5, 0.02], [0, 0.5, 0.02]]),
                        indices=np.uint32([0, 2, 1, 0, 3, 2]),
                        uv1=np.float32([[0.1, 0.1], [0.9, 0.1], [0.9, 0.103], [0.1, 0.103]]))
    sunk = fx.cuboid(4, (-1.0, -0.5, -1.0), (-0.2, 0.3, -0.2))
    ground = fx.floor(2, (0, 0, 0), 2.0)
    inp = dl.BakeInput([strip, sunk, ground], [fx.point_light(9, (0.5, 2.0, 0.5), 5.0)])
    return inp, fx.options(pixel_density=24.0), "exact"


def _root_leaf():
    # two triangles: the occluder BVH is one leaf; shadow, sky, soft sun and bounce rays traverse it
    pos = np.array([(-2, 0, -2), (2, 0, -2), (0, 0, 2), (-1.5, 0.2, 0.5), (1.5, 0.2, 0.5), (0, 2.5, -0.5)],
                   np.float32)
    uv = np.array([(0, 0), (0.45, 0), (0.2, 0.9), (0.55, 0.1), (1, 0.1), (0.8, 0.9)], np.float32)
    mesh = dl.BakeMesh(id=1, positions=pos, indices=np.array([0, 2, 1, 3, 4, 5], np.uint32), uv1=uv)
    lights = [fx.point_light(7, (0.3, 1.2, 1.5), 6.0), fx.sky_light(10),
              fx.sun_light(9, (0.2, 1.0, 0.6), 0.53, illumination=dl.SINGLE_BOUNCE,
                           bounce=dl.BakeBounce(samples=32))]
    opts = fx.options(pixel_density=24.0, sky_samples=64, colored_bounce=True)
    return dl.BakeInput([mesh], lights), opts, "exact"


def _maps(geometry):
    def make():
        inp, opts = fx.determinism_room()
        opts.dynamic_geometry = geometry
        opts.sun_map_resolution = 96
        opts.sky_probe_spacing = 0.7
        opts.sky_samples = 32
        return inp, opts, "exact"
    return make


def _refined_outdoor_maps():
    # binary64 re-tests and Kahan sums, with angular maps, an odd sun map size and alpha lights
    inp, opts = scenes.outdoor(grid=65, chunks=2, boxes=30, point_lights=4, sky_samples=16, bounce_samples=8)
    opts.dynamic_geometry = dl.ANGULAR
    opts.sun_map_resolution = 257
    opts.sky_probe_spacing = 3.0
    for light in inp.lights[:2]:
        light.transparency = dl.TRANSPARENCY_ENABLED
    return inp, opts, "refined"


def _empty():
    return dl.BakeInput(), fx.options(pixel_density=12.0), "exact"


def _lightless():
    return dl.BakeInput([fx.floor(1, (0, 0, 0), 1.0)], []), fx.options(pixel_density=12.0), "exact"


CASES = {
    "small_room": _small_room,
    "mixed_lights": _mixed_lights,
    "soft_rooms": _soft_rooms,
    "outdoor_slice": _outdoor_slice,
    "local_bounce": _local_bounce,
    "colored_mixed_bounce": _colored_mixed_bounce,
    "alpha_shadows": _alpha_shadows,
    "thin_and_buried": _thin_and_buried,
    "root_leaf": _root_leaf,
    "maps_distance_cubes": _maps(dl.DISTANCE_CUBES),
    "maps_angular": _maps(dl.ANGULAR),
    "refined_outdoor_maps": _refined_outdoor_maps,
    "empty": _empty,
    "lightless": _lightless,
}


def oracle_bake(name, threads=0):
    """The oracle's bake of case `name` (the side of the fixtures that outputs are compared with)."""
    from oracle import oracle
    inp, opts, form = CASES[name]()
    if form == "refined":
        return oracle.bake_ex(inp, opts, mode=oracle.REFINED, eps=dl.DEFAULT_REFINE_EPSILON,
                              threads=threads)["scene"]
    return oracle.bake(inp, opts, threads=threads)[0]

