"""The library's binary32 double-float sin/cos path must return exactly what the binary64 path
(the oracle's) returns; its rounding test sends the undecidable cases to binary64. CPU only: the
same header compiles for host and device with identical IEEE operations."""
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
    fields = out.stdout.split()
    fallbacks = int(fields[-1])
    assert fallbacks < 2000000 // 1000, out.stdout  # the binary64 path is rare
