"""The occluder BVH built on the device (csrc/dl_bvh.cu) against the host builder
(csrc/dl_host.cpp), which apply the same rules: the two trees must agree node for node and
triangle for triangle, and bakes from either must give the oracle's bytes. Cases cover both of
the device builder's phases (nodes above 512 triangles, built a level at a time by many blocks,
and the subtrees a warp builds whole), leaves at the root, coincident centroids (split by index)
and scenes without occluders."""
import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import scenes
from oracle import oracle

from . import fixtures as fx
from .test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def _trees(inp, opts):
    out = []
    for host in (0, 1):
        s = dl.Session(inp, opts, host_bvh=host)
        try:
            out.append(s.occluder_bvh())
        finally:
            s.close()
    return out


def _assert_same_tree(inp, opts):
    (nd, td, dd), (nh, th, dh) = _trees(inp, opts)
    assert dd == dh
    assert nd.shape == nh.shape
    assert np.array_equal(nd, nh), f"first differing node {np.argwhere((nd != nh).any(axis=1))[:3].ravel()}"
    assert np.array_equal(td.view(np.uint32), th.view(np.uint32))
    return nd, dd


def _stack(n, spacing, mesh_id=1):
    """n copies of one small quad's two triangles spaced `spacing` apart along x (0: coincident)."""
    pos, idx, uv = [], [], []
    for k in range(n):
        x = np.float32(k * spacing)
        base = len(pos)
        pos += [(x, 0, 0), (x + 0.5, 0, 0), (x + 0.5, 0, 0.5), (x, 0, 0.5)]
        uv += [(0, 0), (1, 0), (1, 1), (0, 1)]
        idx += [base, base + 1, base + 2, base, base + 2, base + 3]
    return dl.BakeMesh(id=mesh_id, positions=np.array(pos, np.float32), indices=np.array(idx, np.uint32),
                       uv1=np.array(uv, np.float32))


CASES = {
    "outdoor": lambda: scenes.outdoor(grid=129, chunks=4, boxes=120, point_lights=3, sky_samples=16,
                                      bounce_samples=8),
    "precision_stress": lambda: scenes.precision_stress(grid=64, chunks=2, boxes=20, decals=2000, slivers=300,
                                                        lights=4, sky_samples=16, bounce_samples=8),
    "rooms": lambda: scenes.room_grid(rooms=2, lights=3, boxes_per_room=6, samples=8),
    "small_room": lambda: scenes.small_room(),
    "coincident": lambda: (dl.BakeInput([_stack(3000, 0.0), fx.floor(2, (0, -1, 0), 3.0)],
                                        [fx.point_light(7, (0, 2, 0), 6.0)]), fx.options()),
    "one_quad": lambda: (dl.BakeInput([fx.floor(1, (0, 0, 0), 1.0)], [fx.point_light(7, (0, 2, 0), 6.0)]),
                         fx.options()),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_device_tree_equals_host_tree(name):
    inp, opts = CASES[name]()
    nodes, depth = _assert_same_tree(inp, opts)
    assert len(nodes) >= 1 and depth >= 1


def test_unbalanced_and_mixed_trees_equal():
    # triangles at geometric spacing (lopsided SAH splits) beside coincident stacks
    pos, idx, uv = [], [], []
    for k in range(1500):
        x = np.float32(1.02 ** k)
        base = len(pos)
        pos += [(x, 0, 0), (x * 1.001, 0.1, 0), (x, 0, 0.1)]
        uv += [(0, 0), (1, 0), (0, 1)]
        idx += [base, base + 1, base + 2]
    lopsided = dl.BakeMesh(id=3, positions=np.array(pos, np.float32), indices=np.array(idx, np.uint32),
                           uv1=np.array(uv, np.float32))
    inp = dl.BakeInput([_stack(700, 0.0, 1), _stack(900, 0.25, 2), lopsided], [fx.point_light(7, (0, 2, 0), 6.0)])
    _assert_same_tree(inp, fx.options())


def test_scene_without_occluders():
    floor = fx.floor(1, (0, 0, 0), 2.0)
    floor.occludes = False
    inp = dl.BakeInput([floor], [fx.point_light(7, (0, 2, 0), 6.0)])
    for host in (0, 1):
        s = dl.Session(inp, fx.options(), host_bvh=host)
        try:
            nodes, tris, depth = s.occluder_bvh()
            assert len(tris) == 0 and depth == 0
            s.run()
        finally:
            s.close()


@pytest.mark.parametrize("host", [0, 1])
def test_bakes_from_either_tree_match_the_oracle(host):
    inp, opts = CASES["outdoor"]()
    want, _, _ = oracle.bake(inp, opts)
    assert_same(dl.bake(inp, opts, host_bvh=host), want)
