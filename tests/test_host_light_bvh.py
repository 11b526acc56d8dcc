"""The library's host light BVH (csrc/dl_host.cpp, through prepare_scene) against the oracle's
restatement of the reference's SAH build (src/bake/light_bvh.rs:59-189): on seeded light sets
with clusters, coincident lights and radii over four orders of magnitude, the nodes (as the
.dynlight file stores them) and the light slot order are identical. The slot order indexes the
runtime's light buffer, so any difference changes every baked word. CPU only."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle
from oracle.oracle import ptr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bvh_tool(tmp_path_factory):
    exe = tmp_path_factory.mktemp("native") / "light_bvh_check"
    csrc = os.path.join(ROOT, "dynamiclighting-bevy_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-x", "c++",
                    "-I", csrc, os.path.join(ROOT, "tests", "native", "light_bvh_check.cpp"),
                    os.path.join(csrc, "dl_host.cpp"), "-o", str(exe)], check=True)
    return exe


def light_set(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        pos = rng.uniform(-50, 50, (n, 3))
        rad = rng.uniform(1, 12, n)
    elif kind == "clusters":  # a few tight groups, like lamps along corridors
        centers = rng.uniform(-200, 200, (max(1, n // 16), 3))
        pos = centers[rng.integers(0, len(centers), n)] + rng.normal(0, 0.5, (n, 3))
        rad = rng.uniform(2, 6, n)
    elif kind == "coincident":  # many lights at a handful of exact positions
        pos = rng.uniform(-5, 5, (3, 3))[rng.integers(0, 3, n)]
        rad = rng.choice([1.0, 2.5, 4.0], n)
    else:  # radii from 0.01 m to 100 m
        pos = rng.uniform(-30, 30, (n, 3))
        rad = 10.0 ** rng.uniform(-2, 2, n)
    return np.float32(pos), np.float32(rad)


def library_bvh(bvh_tool, tmp_path, pos, rad):
    src, dst = tmp_path / "lights.bin", tmp_path / "bvh.bin"
    src.write_bytes(np.uint32([len(rad)]).tobytes() + np.concatenate([pos, rad[:, None]], 1).astype(np.float32).tobytes())
    subprocess.run([str(bvh_tool), str(src), str(dst)], check=True)
    data = np.frombuffer(dst.read_bytes(), np.uint32)
    count = int(data[0])
    return data[1:1 + 8 * count].reshape(count, 8), data[1 + 8 * count:]


def oracle_bvh(pos, rad):
    n = len(rad)
    nodes = np.zeros((max(2 * n, 1), 8), np.uint32)
    order = np.zeros(max(n, 1), np.uint32)
    count = oracle.lib().oracle_light_bvh(ptr(np.ascontiguousarray(pos.reshape(-1))), ptr(rad), n, ptr(nodes),
                                          ptr(order))
    return nodes[:count], order[:n]


@pytest.mark.parametrize("kind", ["uniform", "clusters", "coincident", "radii"])
@pytest.mark.parametrize("n", [1, 2, 7, 64, 513, 2000])
def test_host_light_bvh_equals_the_oracle(bvh_tool, tmp_path, kind, n):
    pos, rad = light_set(kind, n, seed=1000 * n + len(kind))
    nodes, order = library_bvh(bvh_tool, tmp_path, pos, rad)
    want_nodes, want_order = oracle_bvh(pos, rad)
    assert np.array_equal(order, want_order)
    assert nodes.shape == want_nodes.shape and np.array_equal(nodes, want_nodes)
