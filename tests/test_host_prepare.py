"""The host's scene preparation (csrc/dl_host.cpp prepare_scene) on a scene large enough for its
threaded passes: occluder list, lightmap sizes and triangle count equal a sequential
recomputation of the reference's rules (mesh_builder.rs:21-51, occluder.rs:80-97), and with
several invalid meshes the error names the first in id order. CPU only."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_threaded_preparation_equals_the_sequential_rules(tmp_path):
    exe = tmp_path / "prepare_check"
    csrc = os.path.join(ROOT, "dynamiclighting-bevy_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-x", "c++",
                    "-I", csrc, os.path.join(ROOT, "tests", "native", "prepare_check.cpp"),
                    os.path.join(csrc, "dl_host.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and "prepare failures 0" in out.stdout, out.stdout + out.stderr
