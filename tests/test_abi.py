"""The C ABI library loads and exports every symbol include/dynlight.h declares, and the ctypes
mirror's struct layouts match the header's (CPU only; no compute call)."""
import ctypes as C
import os
import re
import subprocess

import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dynlight.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dl_[a-z0-9_]+)\s*\(", text)) - {"dl_status"})


def test_header_declares_what_the_mirror_binds():
    assert declared_functions() == sorted(_abi.EXPORTS)


def test_library_exports_every_declared_symbol():
    if not os.path.exists(dl.LIBRARY_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    lib = C.CDLL(dl.LIBRARY_PATH)
    for name in declared_functions():
        assert hasattr(lib, name), name
    lib.dl_abi_version.restype = C.c_uint32
    assert lib.dl_abi_version() == 2
    lib.dl_status_string.restype = C.c_char_p
    assert lib.dl_status_string(1) == b"cancelled"


def test_struct_layouts_match_the_header(tmp_path):
    src = tmp_path / "sizes.c"
    names = list(_abi.STRUCTS)
    src.write_text('#include <stdio.h>\n#include "dynlight.h"\nint main(void){\n' + "".join(
        f'printf("{n} %zu\\n", sizeof({n}));\n' for n in names) + "return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    sizes = dict(line.split() for line in out.strip().splitlines())
    for n, cls in _abi.STRUCTS.items():
        assert int(sizes[n]) == C.sizeof(cls), n


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    monkeypatch.setattr(dl, "_LIB", None)
    with pytest.raises(RuntimeError, match="not built"):
        dl.load_library(str(tmp_path / "nope.so"))


def test_argument_errors_are_named_without_a_gpu():
    """Entry points reject null or out-of-range arguments before any CUDA call, with a status and
    a message in dl_last_error (the C ABI's form of the reference's BakeError text)."""
    if not os.path.exists(dl.LIBRARY_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    lib = C.CDLL(dl.LIBRARY_PATH)
    lib.dl_last_error.restype = C.c_char_p
    invalid_argument = 21
    null = C.c_void_p()
    n, crc = C.c_uint64(), C.c_uint32()
    assert lib.dl_encode_payload(null, C.byref(null), C.byref(n), C.byref(crc)) == invalid_argument
    assert lib.dl_last_error() == b"null argument"
    assert lib.dl_session_report(null, null) == invalid_argument
    assert lib.dl_last_error() == b"null argument"
    assert lib.dl_session_create(null, null, null, C.byref(null)) == invalid_argument
    assert lib.dl_last_error() == b"null argument"
    assert lib.dl_session_run(null, null) == invalid_argument
    assert lib.dl_last_error() == b"null session"
    # the non-allocating filter checks its window before it touches a device
    buf_a, buf_b = (C.c_float * 3)(), (C.c_float * 3)()
    args = (C.c_uint32(0), C.c_uint32(1), C.c_uint32(0), C.c_uint32(0), C.c_uint32(4), null)
    assert lib.dl_filter_bounce_window_noalloc(buf_a, buf_b, *args) == invalid_argument
    assert b"texels" in lib.dl_last_error()
    args = (C.c_uint32(1), C.c_uint32(1), C.c_uint32(4), C.c_uint32(0), C.c_uint32(4), null)
    assert lib.dl_filter_bounce_window_noalloc(buf_a, buf_b, *args) == invalid_argument
    assert lib.dl_last_error() == b"the window does not lie inside the map"
    assert lib.dl_filter_bounce_window_noalloc(buf_a, buf_a, *args) == invalid_argument
    assert b"distinct" in lib.dl_last_error()
    # the cache-bandwidth probe checks its level, size and passes before it touches a device
    gbs = C.c_double(-1.0)
    for level, size, passes in ((0, 1 << 26, 1), (3, 1 << 26, 1), (2, 1 << 10, 1), (2, 1 << 26, 0),
                                (1, (1 << 32) + 16, 1)):
        assert lib.dl_probe_read_bandwidth(0, level, C.c_uint64(size), passes, C.byref(gbs)) == invalid_argument
        assert b"dl_probe_read_bandwidth" in lib.dl_last_error()
    assert lib.dl_probe_read_bandwidth(0, 2, C.c_uint64(1 << 26), 1, null) == invalid_argument
