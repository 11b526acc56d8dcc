"""TEST INFRASTRUCTURE — ctypes binding of the parity oracle (oracle/_build/liboracle.so).

The oracle is a C++ restatement of the reference CPU baker. Only the tests, the smoke check
and the benchmark's CPU-baseline leg use it: as what the library's outputs are compared with,
or as the timed CPU baseline, never as a path of the product.
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
        for name in ("oracle_acos_approx", "oracle_tan"):
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
        _lib.oracle_bake_ex.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                        C.c_uint32, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]
        _lib.oracle_intersect_batch.restype = C.c_uint64
        _lib.oracle_intersect_batch.argtypes = [C.c_uint32, C.c_float, C.c_uint32] + [C.c_void_p] * 6
        _lib.oracle_captured_map.restype = C.c_uint32
        _lib.oracle_captured_map.argtypes = [C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_uint32]
        _lib.oracle_captured_map_count.restype = C.c_uint32
        _lib.oracle_f16_bits.restype = C.c_uint16
        _lib.oracle_f16_bits.argtypes = [C.c_float]
        _lib.oracle_probe_grid.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p,
                                           C.c_void_p]
        _lib.oracle_fill_inside.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.oracle_capture_all_bounce.argtypes = [C.c_uint32]
    return _lib


# Precision modes of bake_ex: the reference's binary32, the GPU library's refined form, and the
# FP64 oracle (binary64 ray/triangle tests, sums and fractions over the same binary32 samples).
F32, REFINED, F64, REFINED_BOUNCE = 0, 1, 2, 3


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


def bake_ex(inp, options, mode=F32, eps=1.0e-4, threads=0, brute_force=False, bounce_maps=False):
    """Runs the oracle bake in precision `mode`. Returns a dict with the BakedScene ("scene"),
    "burial_rays", "photon_rays", "retests" and, with bounce_maps, every filtered bounce map as
    {(mesh id, slot): (window, float32 [h, w, 3])} under "maps"."""
    import dynlight_gb300 as dl
    m = dl.Marshalled(inp)
    opts = dl.marshal_options(options)
    out = C.POINTER(dl._abi.DlBakedScene)()
    burial, photon, retests = C.c_uint64(), C.c_uint64(), C.c_uint64()
    lb = lib()
    lb.oracle_capture_all_bounce(1 if bounce_maps else 0)
    status = lb.oracle_bake_ex(C.byref(m.input), C.byref(opts), None, threads, 1 if brute_force else 0,
                               mode, eps, C.byref(out), C.byref(burial), C.byref(photon),
                               C.byref(retests))
    maps = {}
    if bounce_maps:
        mid, slot = C.c_uint64(), C.c_uint32()
        rect = np.zeros(4, np.uint32)
        for i in range(lb.oracle_captured_map_count()):
            n = lb.oracle_captured_map(i, C.byref(mid), C.byref(slot), rect.ctypes.data, None, 0)
            rgb = np.zeros(n * 3, np.float32)
            lb.oracle_captured_map(i, C.byref(mid), C.byref(slot), rect.ctypes.data, rgb.ctypes.data, n)
            w, h = int(rect[2] - rect[0] + 1), int(rect[3] - rect[1] + 1)
            maps[(mid.value, slot.value)] = (tuple(int(x) for x in rect), rgb.reshape(h, w, 3))
        lb.oracle_capture_all_bounce(0)
    if status != 0:
        raise dl.BakeError(status, (lb.oracle_last_error() or b"").decode())
    try:
        scene = dl.scene_from_c(out.contents)
    finally:
        lb.oracle_free(out)
    return {"scene": scene, "burial_rays": burial.value, "photon_rays": photon.value,
            "retests": retests.value, "maps": maps}


def intersect_batch(mode, eps, tris, origins, dirs, max_t):
    """Ray/triangle tests in precision `mode`: (hit bool[n], t float32[n], retests)."""
    tris = f32(tris)
    n = tris.size // 9
    o, d, mx = f32(origins), f32(dirs), f32(max_t)
    hit = np.zeros(n, np.uint8)
    t = np.zeros(n, np.float32)
    r = lib().oracle_intersect_batch(mode, eps, n, ptr(tris), ptr(o), ptr(d), ptr(mx), ptr(hit), ptr(t))
    return hit.astype(bool), t, r
