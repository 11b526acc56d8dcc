"""The library's occluder BVH builder (host C++, csrc/dl_host.cpp) on a seeded scene: every
occluder in exactly one leaf, every triangle inside its padded boxes, the reported depth. The
multithreaded top levels must give a valid tree for any thread count. CPU only."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bvh_build_covers_every_occluder(tmp_path):
    exe = tmp_path / "bvh_check"
    csrc = os.path.join(ROOT, "dynamiclighting-bevy_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-x", "c++",
                    "-I", csrc, os.path.join(ROOT, "tests", "native", "bvh_check.cpp"),
                    os.path.join(csrc, "dl_host.cpp"), "-o", str(exe)], check=True)
    for grid, extra in ((257, 20000), (5, 3), (2, 0)):
        out = subprocess.run([str(exe), str(grid), str(extra)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "failures 0" in out.stdout
