"""The library's binary32 double-float sin/cos paths must return exactly what the binary64 paths
(the oracle's) return; its rounding test sends the undecidable cases to binary64. Its acos_approx
(glam's, for the bounce slerp) must equal the oracle's restatement bit for bit. CPU only: the same
header compiles for host and device with identical IEEE operations."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_double_float_sincos_equals_the_binary64_path(tmp_path):
    exe = tmp_path / "sincos_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                    "-I", os.path.join(ROOT, "dynamiclighting-bevy_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "sincos_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "2000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    lines = [l.split() for l in out.stdout.splitlines() if "binary64_fallbacks" in l]
    assert len(lines) == 1, out.stdout  # sin/cos
    for fields in lines:
        assert int(fields[-3]) == 0, out.stdout  # mismatches
        assert int(fields[-1]) < 2000000 // 1000, out.stdout  # the binary64 path is rare


def test_acos_approx_equals_the_oracles(tmp_path):
    exe = tmp_path / "acos_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-ffp-contract=off", "-fno-fast-math",
                    "-I", os.path.join(ROOT, "dynamiclighting-bevy_gb300", "csrc"), "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "native", "acos_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and "mismatches 0" in out.stdout, out.stdout


def test_sky_sample_order_is_a_clustered_permutation(tmp_path):
    exe = tmp_path / "order_check"
    csrc = os.path.join(ROOT, "dynamiclighting-bevy_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-x", "c++",
                    "-I", csrc, os.path.join(ROOT, "tests", "native", "order_check.cpp"),
                    os.path.join(csrc, "dl_host.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and "failures 0" in out.stdout, out.stdout
