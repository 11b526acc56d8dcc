"""TEST INFRASTRUCTURE — ctypes binding of the parity oracle (oracle/_build/liboracle.so).

The oracle is a C++ restatement of the reference CPU baker. Only the tests, the smoke check
and the benchmark's CPU-baseline leg use it, always as the checker or the timed CPU baseline,
never as a path of the product.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build():
    """Compiles the oracle with its Makefile (g++, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        _lib.oracle_last_error.restype = C.c_char_p
        _lib.oracle_seed.restype = C.c_uint64
        _lib.oracle_lightmap_size.restype = C.c_uint32
        _lib.oracle_level.restype = C.c_uint8
        for name in ("oracle_acos", "oracle_tan"):
            getattr(_lib, name).restype = C.c_float
            getattr(_lib, name).argtypes = [C.c_float]
        _lib.oracle_sky_visibility.restype = C.c_float
        _lib.oracle_lightmap_size.argtypes = [C.c_float, C.c_float, C.c_uint32]
        _lib.oracle_level.argtypes = [C.c_float, C.c_uint32]
        _lib.oracle_sincos.argtypes = [C.c_float, C.c_void_p]
        _lib.oracle_spread.argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_uint32, C.c_void_p]
        _lib.oracle_concentric_disk.argtypes = [C.c_float, C.c_float, C.c_void_p]
        _lib.oracle_cosine_direction.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_void_p]
        _lib.oracle_is_buried.argtypes = [C.c_void_p, C.c_float, DIR_FN, C.c_void_p]
        _lib.oracle_intersect.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                          C.c_void_p, C.c_void_p]
        _lib.oracle_slerp.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
    return _lib


DIR_FN = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_float), C.c_float)


def f32(*x):
    return np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1))


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def bake(inp, options, threads=0, brute_force=False, progress=None):
    """Runs the oracle bake; returns (BakedScene, burial_rays, photon_rays) or raises BakeError."""
    import dynlight_gb300 as dl
    m = dl.Marshalled(inp)
    opts = dl.marshal_options(options)
    out = C.POINTER(dl._abi.DlBakedScene)()
    burial, photon = C.c_uint64(), C.c_uint64()
    lb = lib()
    status = lb.oracle_bake(C.byref(m.input), C.byref(opts),
                            C.byref(progress.raw) if progress else None, C.c_uint32(threads),
                            C.c_uint32(1 if brute_force else 0), C.byref(out), C.byref(burial),
                            C.byref(photon))
    if status != 0:
        raise dl.BakeError(status, (lb.oracle_last_error() or b"").decode())
    try:
        return dl.scene_from_c(out.contents), burial.value, photon.value
    finally:
        lb.oracle_free(out)
