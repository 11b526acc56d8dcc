"""Input validation mirrors BakeError (src/bake/input.rs:198-373, src/bake/baker.rs:32-35,205-233).

The library validates options, ids, meshes and lights before its first CUDA call, so these run on
the CPU through the C ABI. Rules the C ABI cannot check (a dl_mesh has one vertex count for all of
its arrays, so per-vertex arrays of another length, and alpha data of the wrong size) are checked
by the Python mirror before marshalling, in the reference's order. The cases are host-side
injected faults: bad indices, non-finite positions, duplicate ids, malformed lights and options.
"""
import dataclasses
import os

import numpy as np
import pytest

import dynlight_gb300 as dl
from tests import fixtures as fx


@pytest.fixture(autouse=True)
def _library():
    if not os.path.exists(dl.LIBRARY_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")


def fails(inp, opts, kind, message, **kw):
    with pytest.raises(dl.BakeError) as e:
        dl.bake(inp, opts, **kw)
    assert e.value.kind == kind
    assert message in str(e.value), str(e.value)
    return str(e.value)


def room():
    return fx.determinism_room()


def test_duplicate_ids():
    inp, opts = room()
    inp.meshes[1].id = inp.meshes[0].id
    fails(inp, opts, "DuplicateId", "two meshes share BakeId")
    inp, opts = room()
    inp.lights[2].id = inp.lights[0].id
    fails(inp, opts, "DuplicateId", "two lights share BakeId")


@pytest.mark.parametrize("change, message", [
    (lambda m: setattr(m, "indices", np.append(m.indices, np.uint32(0))), "indices is not a multiple of 3"),
    (lambda m: setattr(m, "indices", np.concatenate([m.indices, np.uint32([0, 1, 999])])),
     "index 999 is out of range for"),
    (lambda m: m.positions.__setitem__((1, 2), np.nan), "non-finite vertex position"),
    (lambda m: m.positions.__setitem__((0, 0), np.inf), "non-finite vertex position"),
    (lambda m: setattr(m, "alpha", dl.AlphaTexture(2, 2, np.zeros(16, np.uint8))), "an alpha texture needs UV0"),
])
def test_mesh_rules_the_library_checks(change, message):
    inp, opts = room()
    inp.meshes[0].positions = np.array(inp.meshes[0].positions, np.float32)
    change(inp.meshes[0])
    text = fails(inp, opts, "InvalidMesh", message)
    assert f"mesh {inp.meshes[0].id:#018x}" in text


@pytest.mark.parametrize("change, message", [
    (lambda l: setattr(l, "radius", 0.0), "radius must be positive and finite"),
    (lambda l: setattr(l, "radius", float("inf")), "radius must be positive and finite"),
    (lambda l: setattr(l, "position", (0.0, float("nan"), 0.0)), "non-finite position"),
    (lambda l: setattr(l, "shape", dl.LightShape.rectangle((0, 0, 0, 2.0), 1.0, 1.0)),
     "area light rotation must be a unit quaternion"),
    (lambda l: setattr(l, "shape", dl.LightShape.tube((0, 0, 0, 1.0), -1.0)),
     "area light size must be finite and not negative"),
    (lambda l: setattr(l, "shape", dl.LightShape.sun((0, 0, 0, 1.0), 11.0)),
     "sun angular diameter must be 0 to 10 degrees"),
    (lambda l: setattr(l, "shape", dl.LightShape.sun((0, 0, 0.5, 0.5), 0.5)),
     "sun rotation must be a unit quaternion"),
])
def test_light_rules(change, message):
    inp, opts = room()
    change(inp.lights[1])
    fails(inp, opts, "InvalidLight", message)


OPTION_FAULTS = [("pixel_density", -1.0), ("pixel_density", float("nan")), ("max_lightmap_size", 1),
                 ("photon_cube_resolution", 0), ("area_light_samples", 0), ("sun_map_resolution", 0),
                 ("sun_map_resolution", 8193), ("sky_samples", 0), ("sky_probe_spacing", 0.0),
                 ("sky_probe_spacing", float("inf")), ("bounce_compression", 7),
                 # f32 values: a density that underflows to 0 or overflows to infinity as the f32
                 # BakeOptions holds (src/bake/input.rs:136-164), likewise the probe spacing
                 ("pixel_density", 1e-50), ("pixel_density", 1e50), ("sky_probe_spacing", 1e-60)]


@pytest.mark.parametrize("name, value", OPTION_FAULTS)
def test_option_rules_and_the_mirrors_copy_agree(name, value):
    inp, opts = room()
    opts = dataclasses.replace(opts, **{name: value})
    text = fails(inp, opts, "InvalidOptions", "invalid bake options: ")
    assert text == "InvalidOptions: " + dl._options_error(opts)


def test_f32_rounded_options_come_before_a_length_mismatch():
    """An f32-underflowing density and a per-vertex array of the wrong length: the mirror checks
    the options first (src/bake/baker.rs:32-35), as the f32 the library would receive, so it
    reports InvalidOptions as the reference does, not InvalidMesh."""
    inp, opts = room()
    inp.meshes[2].uv1 = inp.meshes[2].uv1[:-1]
    opts = dataclasses.replace(opts, pixel_density=1e-50)
    fails(inp, opts, "InvalidOptions", "pixel density must be positive")


def test_valid_options_pass_the_mirrors_copy():
    assert dl._options_error(room()[1]) is None
    assert dl._options_error(dl.BakeOptions()) is None


@pytest.mark.parametrize("change, message", [
    (lambda m: setattr(m, "uv1", m.uv1[:-1]), "UV1 coordinates for"),
    (lambda m: setattr(m, "normals", np.zeros((len(m.positions) + 2, 3), np.float32)), "normals for"),
    (lambda m: (setattr(m, "uv0", np.zeros((len(m.positions) - 1, 2), np.float32)),), "UV0 coordinates for"),
    (lambda m: (setattr(m, "uv0", np.zeros((len(m.positions), 2), np.float32)),
                setattr(m, "alpha", dl.AlphaTexture(2, 2, np.zeros(15, np.uint8)))),
     "alpha texture size doesn't match its data"),
])
def test_length_rules_stop_before_the_library(change, message):
    inp, opts = room()
    mesh = inp.meshes[2]
    change(mesh)
    v = len(mesh.positions)
    text = fails(inp, opts, "InvalidMesh", message)
    assert f"mesh {mesh.id:#018x}" in text
    if "coordinates" in message or "normals" in message:
        assert text.endswith(f"for {v} vertices")
    with pytest.raises(dl.BakeError):  # the session API checks the same
        dl.Session(inp, opts)


def test_errors_come_in_the_references_order():
    # a length fault in one mesh and an index fault in a mesh of lower id: the lower id reports
    inp, opts = room()
    by_id = sorted(inp.meshes, key=lambda m: m.id)
    low, high = by_id[0], by_id[-1]
    high.uv1 = high.uv1[:-1]
    low.indices = np.concatenate([low.indices, np.uint32([0, 1, 500])])
    text = fails(inp, opts, "InvalidMesh", "index 500 is out of range")
    assert f"mesh {low.id:#018x}" in text
    # within one mesh, an out-of-range index comes before a UV1 count (input.rs:245-256)
    inp, opts = room()
    m = inp.meshes[0]
    m.uv1 = m.uv1[:-1]
    m.indices = np.concatenate([m.indices, np.uint32([0, 1, 777])])
    fails(inp, opts, "InvalidMesh", "index 777 is out of range")
    # options come first, then duplicate ids
    inp, opts = room()
    inp.meshes[0].uv1 = inp.meshes[0].uv1[:-1]
    fails(inp, dataclasses.replace(opts, sky_samples=0), "InvalidOptions", "skies need at least one sample")
    inp.meshes[1].id = inp.meshes[3].id
    fails(inp, opts, "DuplicateId", "two meshes share BakeId")


def test_the_mirrors_messages_equal_the_librarys():
    # the same index fault reported by the mirror (with a length fault elsewhere) and by the library
    inp, opts = room()
    low = min(inp.meshes, key=lambda m: m.id)
    low.indices = np.concatenate([low.indices, np.uint32([0, 1, 321])])
    from_library = fails(inp, opts, "InvalidMesh", "index 321")
    high = max(inp.meshes, key=lambda m: m.id)
    high.uv1 = high.uv1[:-1]
    assert fails(inp, opts, "InvalidMesh", "index 321") == from_library


def test_invalid_tuning_is_an_argument_error():
    inp, opts = room()
    fails(inp, opts, "invalid argument", "sample_lanes", sample_lanes=3)
    fails(inp, opts, "invalid argument", "refine_epsilon", refine_epsilon=0.5)
    for m in (1, 6, 11, 13):
        fails(inp, opts, "invalid argument", "min_blocks", min_blocks=m)
    for m in (1, 7, 11, 12):
        fails(inp, opts, "invalid argument", "gather_min_blocks", gather_min_blocks=m)


@pytest.mark.parametrize("mesh_id", [0, 1, 0xFFFFFFFFFFFFFFFF])
def test_ids_print_as_the_library_prints_them(mesh_id):
    # a duplicate id reported by the library, then by the mirror (a length fault elsewhere)
    inp, opts = room()
    inp.meshes[0].id = inp.meshes[1].id = mesh_id
    from_library = fails(inp, opts, "DuplicateId", "two meshes share BakeId")
    inp.meshes[2].uv1 = inp.meshes[2].uv1[:-1]
    assert fails(inp, opts, "DuplicateId", "two meshes share BakeId") == from_library
    assert from_library.endswith(dl._hex_id(mesh_id))


def test_a_cancelled_bake_reports_cancelled_after_validation():
    # progress.check() follows validation in the reference (baker.rs:32-55): invalid input reports
    # its own error even when the bake was cancelled before it started; valid input is cancelled
    # before the library touches a device
    inp, opts = room()
    progress = dl.BakeProgress()
    progress.cancel()
    fails(inp, opts, "Cancelled", "the bake was cancelled", progress=progress)
    assert progress.stage == 0
    fails(inp, dataclasses.replace(opts, pixel_density=0.0), "InvalidOptions", "pixel density", progress=progress)
    inp.lights[0].id = inp.lights[1].id
    fails(inp, opts, "DuplicateId", "two lights share BakeId", progress=progress)
    inp, opts = room()
    inp.meshes[0].uv1 = inp.meshes[0].uv1[:-1]
    fails(inp, opts, "InvalidMesh", "UV1 coordinates", progress=progress)
