"""dynlight GB300 baker: the host-side mirror of the reference's bake API.

`bake(input, options, progress)` mirrors `dynlight::bake::bake` (src/bake/baker.rs:27-31) and
returns a `BakedScene` with the same fields (src/bake/format/types.rs:13-37). The inputs mirror
`BakeInput`, `BakeMesh`, `BakeLight`, `BakeOptions` and `BakeProgress`
(src/bake/input.rs:17-164, src/bake/progress.rs:41-110); errors raise `BakeError` with the
reference's error kinds (src/bake/input.rs:198-209).

Every call goes through the CUDA library's C ABI (include/dynlight.h); there is no CPU path. When
the library is not built the call fails loudly with the build command to run.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _abi
from ._abi import (DlAlphaTexture, DlBakeConfig, DlBakedScene, DlBakeInput, DlBakeOptions,
                   DlBakeReport, DlLight, DlMesh, DlProgress)

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(PACKAGE_DIR, "_build", "libdynlight_gb300.so")

# Light shapes (src/bake/format/lights.rs:27-54 codes).
POINT, RECTANGLE, TUBE, SUN, SKY = 0, 1, 2, 3, 4
DIRECT, SINGLE_BOUNCE = 0, 1
TRANSPARENCY_DISABLED, TRANSPARENCY_ENABLED, TRANSPARENCY_ENABLED_MAX = 0, 1, 2
LIGHTING_ONLY, DISTANCE_CUBES, ANGULAR = 0, 1, 2
FORM_BATCHED, FORM_PLAIN, FORM_REFINED, FORM_BOUNCE_REFINED = 0, 1, 2, 3
DEFAULT_REFINE_EPSILON = 1e-4  # dl_bake_config.refine_epsilon when left 0
FORMS = {"batched": FORM_BATCHED, "plain": FORM_PLAIN, "refined": FORM_REFINED,
         "bounce_refined": FORM_BOUNCE_REFINED}

ERROR_KINDS = {1: "Cancelled", 2: "DuplicateId", 3: "InvalidMesh", 4: "InvalidLight",
               5: "InvalidOptions"}


class BakeError(Exception):
    """A failed bake: `kind` is the reference's BakeError variant or the library status."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.kind = ERROR_KINDS.get(status, _abi.STATUS.get(status, f"status {status}"))
        super().__init__(f"{self.kind}: {message}" if message else self.kind)


@dataclass
class AlphaTexture:
    """AlphaTexture (src/bake/input.rs:62-77): RGBA8 rows, texels with alpha < cutoff pass light."""
    width: int
    height: int
    rgba8: np.ndarray
    cutoff: float = 0.5


@dataclass
class LightShape:
    """LightShape (src/light/shape.rs:19-30): the kind plus rotation (x, y, z, w) and size."""
    kind: int = POINT
    rotation: Sequence[float] = (0.0, 0.0, 0.0, 1.0)
    size: Sequence[float] = (0.0, 0.0)

    @staticmethod
    def point():
        return LightShape(POINT)

    @staticmethod
    def rectangle(rotation, width, height):
        return LightShape(RECTANGLE, tuple(rotation), (width, height))

    @staticmethod
    def tube(rotation, length):
        return LightShape(TUBE, tuple(rotation), (length, 0.0))

    @staticmethod
    def sun(rotation, angular_diameter_degrees):
        return LightShape(SUN, tuple(rotation), (angular_diameter_degrees, 0.0))

    @staticmethod
    def sky():
        return LightShape(SKY)

    def is_distant(self):
        return self.kind in (SUN, SKY)


@dataclass
class BakeBounce:
    """BakeBounce (src/bake/input.rs:116-134)."""
    samples: int = 32
    intensity: float = 1.0
    compression: Optional[int] = None  # bits per pixel, None: the options'


@dataclass
class BakeMesh:
    """BakeMesh (src/bake/input.rs:24-45), world space."""
    id: int
    positions: np.ndarray          # (V, 3) float32
    indices: np.ndarray            # (3T,) uint32
    uv1: np.ndarray                # (V, 2) float32
    normals: Optional[np.ndarray] = None
    uv0: Optional[np.ndarray] = None
    alpha: Optional[AlphaTexture] = None
    occludes: bool = True
    albedo: Sequence[float] = (1.0, 1.0, 1.0)
    content_hash: int = 0

    def triangle_count(self):
        return len(self.indices) // 3


@dataclass
class BakeLight:
    """BakeLight (src/bake/input.rs:101-112)."""
    id: int
    position: Sequence[float]
    radius: float
    illumination: int = DIRECT
    transparency: int = TRANSPARENCY_DISABLED
    bounce: BakeBounce = field(default_factory=BakeBounce)
    shape: LightShape = field(default_factory=LightShape)


@dataclass
class BakeInput:
    meshes: List[BakeMesh] = field(default_factory=list)
    lights: List[BakeLight] = field(default_factory=list)

    def triangle_count(self):
        return sum(m.triangle_count() for m in self.meshes)


@dataclass
class BakeOptions:
    """BakeOptions (src/bake/input.rs:136-194) with BakeSettings' defaults (settings.rs:67-81)."""
    pixel_density: float = 128.0
    max_lightmap_size: int = 2048
    bounce_compression: int = 8
    dynamic_geometry: int = ANGULAR
    skip_bounce: bool = False
    photon_cube_resolution: int = 512
    area_light_samples: int = 64
    area_light_min_samples: int = 16
    sun_map_resolution: int = 2048
    sky_samples: int = 64
    sky_probe_spacing: float = 1.0
    colored_bounce: bool = False
    seed: int = 0


class BakeProgress:
    """BakeProgress (src/bake/progress.rs:41-110): stage, done/total and a cancel flag the
    library polls between stages and in its device work queue."""

    def __init__(self):
        self.raw = DlProgress()

    def cancel(self):
        self.raw.cancel = 1

    def is_cancelled(self):
        return bool(self.raw.cancel)

    @property
    def stage(self):
        return self.raw.stage

    def fraction(self):
        """Progress through the current stage, 0 to 1; 1 once the bake is done (progress.rs:71-81)."""
        if self.raw.stage >= 4:  # BakeStage::Done, or a stage past the known ones
            return 1.0
        return min(self.raw.done / self.raw.total, 1.0) if self.raw.total else 0.0


# ---- marshalling ----------------------------------------------------------------------------

def _f32(a, cols):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, cols))
    return a


def _hex_id(i):
    """A BakeId as the library's messages print it (C's %#018llx)."""
    return f"{i:#018x}" if i else "0" * 18


def _options_error(o: BakeOptions):
    """BakeOptions::validate (src/bake/input.rs:336-373) with the library's messages. The float
    options are checked as the f32 values the library receives (BakeOptions holds f32), so a
    density that underflows or overflows f32 fails here as it fails there."""
    bad = None
    with np.errstate(over="ignore", under="ignore"):
        density, spacing = (float(np.float32(v)) for v in (o.pixel_density, o.sky_probe_spacing))
    if not (math.isfinite(density) and density > 0.0):
        bad = "pixel density must be positive"
    elif o.max_lightmap_size < 2:
        bad = "the maximum shadow map size must be at least 2"
    elif o.photon_cube_resolution == 0:
        bad = "the photon cube resolution must be positive"
    elif o.area_light_samples == 0:
        bad = "area lights need at least one sample"
    elif not 1 <= o.sun_map_resolution <= 8192:
        bad = "the sun map resolution must be 1 to 8192"
    elif o.sky_samples == 0:
        bad = "skies need at least one sample"
    elif not (math.isfinite(spacing) and spacing > 0.0):
        bad = "the sky probe spacing must be positive"
    elif o.bounce_compression not in (8, 6, 5, 4):
        bad = "bounce compression must be 8, 6, 5 or 4 bits"
    elif o.dynamic_geometry > ANGULAR:
        bad = "unknown dynamic geometry mode"
    return None if bad is None else "invalid bake options: " + bad


def _mesh_error(m: BakeMesh):
    """BakeMesh::validate (src/bake/input.rs:233-284) in the reference's order. Returns
    (reason, length_rule): length_rule marks the rules the C ABI cannot check, because a dl_mesh
    carries one vertex count for all of its arrays."""
    idx = np.asarray(m.indices, dtype=np.uint32).reshape(-1)
    pos = np.asarray(m.positions, dtype=np.float32).reshape(-1, 3)
    v = pos.shape[0]
    if len(idx) % 3:
        return f"{len(idx)} indices is not a multiple of 3", False
    if len(idx) and int(idx.max()) >= v:
        return f"index {int(idx[np.argmax(idx >= v)])} is out of range for {v} vertices", False
    n_uv1 = np.asarray(m.uv1, dtype=np.float32).reshape(-1, 2).shape[0]
    if n_uv1 != v:
        return f"{n_uv1} UV1 coordinates for {v} vertices", True
    if m.normals is not None and len(m.normals):
        n_nrm = np.asarray(m.normals, dtype=np.float32).reshape(-1, 3).shape[0]
        if n_nrm != v:
            return f"{n_nrm} normals for {v} vertices", True
    if not np.isfinite(pos).all():
        return "non-finite vertex position", False
    if m.uv0 is not None:
        n_uv0 = np.asarray(m.uv0, dtype=np.float32).reshape(-1, 2).shape[0]
        if n_uv0 != v:
            return f"{n_uv0} UV0 coordinates for {v} vertices", True
    if m.alpha is not None:
        if m.uv0 is None:
            return "an alpha texture needs UV0", False
        if np.asarray(m.alpha.rgba8, dtype=np.uint8).size != m.alpha.width * m.alpha.height * 4:
            return "alpha texture size doesn't match its data", True
    return None, False


def _lengths_disagree(m: BakeMesh):
    """Whether a per-vertex array or the alpha texture's data disagrees with the mesh's sizes."""
    v = np.asarray(m.positions).size // 3
    rows = lambda a, k: np.asarray(a).size // k  # noqa: E731
    return (rows(m.uv1, 2) != v or (m.normals is not None and len(m.normals) and rows(m.normals, 3) != v)
            or (m.uv0 is not None and rows(m.uv0, 2) != v)
            or (m.alpha is not None and np.asarray(m.alpha.rgba8).size != m.alpha.width * m.alpha.height * 4))


def _check_array_lengths(inp: BakeInput, options: BakeOptions):
    """Raises the reference's error for an input whose arrays disagree in length with its
    positions. The C ABI reads every per-vertex array with the mesh's one vertex count, so such an
    input must not reach it. When no length rule fails, this does nothing and the library checks
    everything else. Otherwise the whole validation runs here in the reference's order (options,
    duplicate mesh ids, then each mesh in id order; src/bake/baker.rs:32-35,205-218), so the first
    error reported is the reference's."""
    if not any(_lengths_disagree(m) for m in inp.meshes):
        return
    err = _options_error(options)
    if err:
        raise BakeError(5, err)
    meshes = sorted(inp.meshes, key=lambda m: int(m.id))
    for a, b in zip(meshes, meshes[1:]):
        if int(a.id) == int(b.id):
            raise BakeError(2, "two meshes share BakeId " + _hex_id(int(b.id)))
    for m in meshes:
        reason, _ = _mesh_error(m)
        if reason:
            raise BakeError(3, f"mesh {_hex_id(int(m.id))}: {reason}")


class Marshalled:
    """The C structs of one BakeInput plus the arrays they point into (kept alive here)."""

    def __init__(self, inp: BakeInput):
        self.keep = []
        n = len(inp.meshes)
        self.meshes = (DlMesh * max(n, 1))()
        for i, m in enumerate(inp.meshes):
            pos = _f32(m.positions, 3)
            uv1 = _f32(m.uv1, 2)
            idx = np.ascontiguousarray(np.asarray(m.indices, dtype=np.uint32).reshape(-1))
            d = self.meshes[i]
            d.id = int(m.id) & 0xFFFFFFFFFFFFFFFF
            d.content_hash = int(m.content_hash) & 0xFFFFFFFFFFFFFFFF
            d.vertex_count = pos.shape[0]
            d.occludes = 1 if m.occludes else 0
            d.index_count = idx.shape[0]
            d.positions = pos.ctypes.data_as(_abi.f32p)
            d.indices = idx.ctypes.data_as(_abi.u32p)
            d.uv1 = uv1.ctypes.data_as(_abi.f32p)
            self.keep += [pos, uv1, idx]
            if m.normals is not None and len(m.normals):
                nrm = _f32(m.normals, 3)
                d.normals = nrm.ctypes.data_as(_abi.f32p)
                self.keep.append(nrm)
            if m.uv0 is not None:
                uv0 = _f32(m.uv0, 2)
                d.uv0 = uv0.ctypes.data_as(_abi.f32p)
                self.keep.append(uv0)
            if m.alpha is not None:
                rgba = np.ascontiguousarray(np.asarray(m.alpha.rgba8, dtype=np.uint8).reshape(-1))
                tex = DlAlphaTexture(m.alpha.width, m.alpha.height,
                                     rgba.ctypes.data_as(_abi.u8p), m.alpha.cutoff, 0)
                self.keep += [rgba, tex]
                d.alpha = C.pointer(tex)
            d.albedo[:] = [float(x) for x in m.albedo]
        k = len(inp.lights)
        self.lights = (DlLight * max(k, 1))()
        for i, l in enumerate(inp.lights):
            d = self.lights[i]
            d.id = int(l.id) & 0xFFFFFFFFFFFFFFFF
            d.position[:] = [float(x) for x in l.position]
            d.radius = float(l.radius)
            d.illumination = l.illumination
            d.transparency = l.transparency
            d.bounce_samples = l.bounce.samples
            d.bounce_intensity = l.bounce.intensity
            d.bounce_compression = -1 if l.bounce.compression is None else l.bounce.compression
            d.shape = l.shape.kind
            d.rotation[:] = [float(x) for x in l.shape.rotation]
            d.size[:] = [float(x) for x in l.shape.size]
        self.input = DlBakeInput(C.cast(self.meshes, C.POINTER(DlMesh)), n,
                                 C.cast(self.lights, C.POINTER(DlLight)), k)


def marshal_options(o: BakeOptions) -> DlBakeOptions:
    return DlBakeOptions(o.pixel_density, o.max_lightmap_size, o.bounce_compression,
                         o.dynamic_geometry, int(o.skip_bounce), o.photon_cube_resolution,
                         o.area_light_samples, o.area_light_min_samples, o.sun_map_resolution,
                         o.sky_samples, o.sky_probe_spacing, int(o.colored_bounce),
                         int(o.seed) & 0xFFFFFFFFFFFFFFFF)


# ---- results --------------------------------------------------------------------------------

@dataclass
class BakedMesh:
    id: int
    content_hash: int
    resolution: int
    triangles: np.ndarray  # uint32 dynamic_triangles words
    occludes: bool

    def triangle_count(self):
        return int(self.triangles[0]) // 4 if len(self.triangles) else 0


@dataclass
class BakedLight:
    id: int
    origin: tuple
    radius: float
    shape: int
    rotation: tuple
    size: tuple
    bounce_bits: int
    shadow_bits_per_texel: int


@dataclass
class SunMap:
    """SunMap (src/bake/format/types.rs:115-128)."""
    rows: np.ndarray       # (3, 4) float32: world to map space
    resolution: int
    texels: np.ndarray     # uint32, two unorm16 depths per word


@dataclass
class SkyProbes:
    """SkyProbes (src/bake/format/types.rs:72-113)."""
    origin: tuple
    spacing: float
    counts: tuple
    words: np.ndarray      # uint32, two per probe


@dataclass
class BakedScene:
    settings: dict
    lights: List[BakedLight]
    light_bvh: np.ndarray  # (n, 8) uint32 words per node, as the file stores them
    meshes: List[BakedMesh]
    distance_cubes: np.ndarray
    stats: dict
    sun_maps: List[SunMap] = field(default_factory=list)
    sky_probes: Optional[SkyProbes] = None

    def words_equal(self, other: "BakedScene") -> bool:
        return (len(self.meshes) == len(other.meshes)
                and all(a.id == b.id and a.resolution == b.resolution
                        and np.array_equal(a.triangles, b.triangles)
                        for a, b in zip(self.meshes, other.meshes)))

    def maps_equal(self, other: "BakedScene") -> bool:
        """Distance cubes, sun maps and sky probes equal bit for bit."""
        if not np.array_equal(self.distance_cubes, other.distance_cubes):
            return False
        if len(self.sun_maps) != len(other.sun_maps):
            return False
        for a, b in zip(self.sun_maps, other.sun_maps):
            if (a.resolution != b.resolution or not np.array_equal(a.rows.view(np.uint32), b.rows.view(np.uint32))
                    or not np.array_equal(a.texels, b.texels)):
                return False
        a, b = self.sky_probes, other.sky_probes
        if (a is None) != (b is None):
            return False
        if a is None:
            return True
        return (np.float32(a.spacing).view(np.uint32) == np.float32(b.spacing).view(np.uint32)
                and np.array_equal(np.float32(a.origin).view(np.uint32), np.float32(b.origin).view(np.uint32))
                and a.counts == b.counts and np.array_equal(a.words, b.words))


def scene_from_c(s: DlBakedScene) -> BakedScene:
    """Copies a dl_baked_scene into numpy-backed Python objects."""
    st = s.settings
    settings = dict(bounce=bool(st.bounce), colored_bounce=bool(st.colored_bounce),
                    dynamic_geometry=st.dynamic_geometry, pixel_density=st.pixel_density,
                    max_lightmap_size=st.max_lightmap_size,
                    distance_cube_resolution=st.distance_cube_resolution)
    lights = []
    for i in range(s.light_count):
        l = s.lights[i]
        lights.append(BakedLight(l.id, tuple(l.origin), l.radius, l.shape, tuple(l.rotation),
                                 tuple(l.size), l.bounce_bits, l.shadow_bits_per_texel))
    nb = s.light_bvh_count
    if nb:
        raw = C.cast(s.light_bvh, C.POINTER(C.c_uint32 * (8 * nb))).contents
        bvh = np.frombuffer(raw, dtype=np.uint32).reshape(nb, 8).copy()
    else:
        bvh = np.zeros((0, 8), np.uint32)
    meshes = []
    for i in range(s.mesh_count):
        m = s.meshes[i]
        n = m.word_count
        words = (np.ctypeslib.as_array(m.triangles, shape=(n,)).copy() if n
                 else np.zeros(0, np.uint32))
        meshes.append(BakedMesh(m.id, m.content_hash, m.resolution, words, bool(m.occludes)))
    nd = s.distance_cube_words
    cubes = (np.ctypeslib.as_array(s.distance_cubes, shape=(nd,)).copy() if nd
             else np.zeros(0, np.uint32))
    t = s.stats
    stats = dict(meshes=t.meshes, triangles=t.triangles, texels=t.texels, rays=t.rays,
                 lights_removed=t.lights_removed, bounce_rays=t.bounce_rays,
                 triangle_words=t.triangle_words)

    def words_of(ptr, n):
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy() if n else np.zeros(0, np.uint32)

    sun_maps = []
    for i in range(s.sun_map_count):
        m = s.sun_maps[i]
        sun_maps.append(SunMap(np.array(list(m.rows), np.float32).reshape(3, 4), m.resolution,
                               words_of(m.texels, m.word_count)))
    probes = None
    if s.sky_probes:
        p = s.sky_probes.contents
        probes = SkyProbes(tuple(p.origin), p.spacing, tuple(p.counts), words_of(p.words, p.word_count))
    return BakedScene(settings, lights, bvh, meshes, cubes, stats, sun_maps, probes)


# ---- the library ------------------------------------------------------------------------------

_LIB = None


def load_library(path: str = LIBRARY_PATH):
    """Loads the CUDA library. Raises when it is missing: there is no fallback."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(
            f"the dynlight CUDA library is not built ({path}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` from the repository root")
    lib = C.CDLL(path)
    P = C.POINTER
    lib.dl_abi_version.restype = C.c_uint32
    lib.dl_status_string.restype = C.c_char_p
    lib.dl_status_string.argtypes = [C.c_int]
    lib.dl_last_error.restype = C.c_char_p
    lib.dl_bake_ex.restype = C.c_int
    lib.dl_bake_ex.argtypes = [P(DlBakeInput), P(DlBakeOptions), P(DlBakeConfig), P(DlProgress),
                               P(P(DlBakedScene)), P(DlBakeReport)]
    lib.dl_bake.restype = C.c_int
    lib.dl_bake.argtypes = [P(DlBakeInput), P(DlBakeOptions), P(DlProgress), P(P(DlBakedScene))]
    lib.dl_baked_scene_free.argtypes = [P(DlBakedScene)]
    lib.dl_default_options.argtypes = [P(DlBakeOptions)]
    lib.dl_session_create.restype = C.c_int
    lib.dl_session_create.argtypes = [P(DlBakeInput), P(DlBakeOptions), P(DlBakeConfig),
                                      P(C.c_void_p)]
    lib.dl_session_run.restype = C.c_int
    lib.dl_session_run.argtypes = [C.c_void_p, P(DlProgress)]
    lib.dl_session_result.restype = C.c_int
    lib.dl_session_result.argtypes = [C.c_void_p, P(P(DlBakedScene))]
    lib.dl_session_report.restype = C.c_int
    lib.dl_session_report.argtypes = [C.c_void_p, P(DlBakeReport)]
    lib.dl_session_destroy.argtypes = [C.c_void_p]
    lib.dl_encode_payload.restype = C.c_int
    lib.dl_encode_payload.argtypes = [P(DlBakedScene), P(P(C.c_uint8)), P(C.c_uint64),
                                      P(C.c_uint32)]
    lib.dl_free.argtypes = [C.c_void_p]
    lib.dl_session_encode_payload.restype = C.c_int
    lib.dl_session_encode_payload.argtypes = [C.c_void_p, P(P(C.c_uint8)), P(C.c_uint64), P(C.c_uint32)]
    lib.dl_release_memory.restype = None
    lib.dl_release_memory.argtypes = []
    lib.dl_session_occluder_bvh.restype = C.c_int
    lib.dl_session_occluder_bvh.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                            P(C.c_uint32), P(C.c_uint32)]
    lib.dl_session_bounce_map.restype = C.c_int
    lib.dl_session_bounce_map.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p,
                                          C.c_uint32, P(C.c_uint32)]
    lib.dl_filter_bounce_window_noalloc.restype = C.c_int
    lib.dl_filter_bounce_window_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                                    C.c_uint32, C.c_uint32, C.c_void_p]
    lib.dl_probe_read_bandwidth.restype = C.c_int
    lib.dl_probe_read_bandwidth.argtypes = [C.c_int, C.c_uint32, C.c_uint64, C.c_uint32, P(C.c_double)]
    _LIB = lib
    return lib


def _raise(lib, status):
    raise BakeError(status, (lib.dl_last_error() or b"").decode())


def make_config(form="batched", **tuning) -> DlBakeConfig:
    cfg = DlBakeConfig()
    cfg.form = FORMS[form] if isinstance(form, str) else int(form)
    for k, v in tuning.items():
        if not hasattr(cfg, k):
            raise TypeError(f"unknown bake tuning {k!r}")
        setattr(cfg, k, float(v) if k == "refine_epsilon" else int(v))
    return cfg


def bake(inp: BakeInput, options: BakeOptions, progress: Optional[BakeProgress] = None,
         form="batched", report: Optional[DlBakeReport] = None, **tuning) -> BakedScene:
    """bake() (src/bake/baker.rs:27-31) on the GPU through dl_bake_ex."""
    lib = load_library()
    _check_array_lengths(inp, options)
    m = Marshalled(inp)
    opts = marshal_options(options)
    cfg = make_config(form, **tuning)
    out = C.POINTER(DlBakedScene)()
    status = lib.dl_bake_ex(C.byref(m.input), C.byref(opts), C.byref(cfg),
                            C.byref(progress.raw) if progress else None, C.byref(out),
                            C.byref(report) if report is not None else None)
    if status != 0:
        _raise(lib, status)
    try:
        return scene_from_c(out.contents)
    finally:
        lib.dl_baked_scene_free(out)


class Session:
    """A device-resident bake (dl_session_*): create uploads and builds the BVH once, run
    repeats every device stage, result downloads and serializes."""

    def __init__(self, inp: BakeInput, options: BakeOptions, form="batched", **tuning):
        self.lib = load_library()
        _check_array_lengths(inp, options)
        self._m = Marshalled(inp)
        self._opts = marshal_options(options)
        self._cfg = make_config(form, **tuning)
        self.handle = C.c_void_p()
        status = self.lib.dl_session_create(C.byref(self._m.input), C.byref(self._opts),
                                            C.byref(self._cfg), C.byref(self.handle))
        if status != 0:
            _raise(self.lib, status)

    def run(self, progress: Optional[BakeProgress] = None):
        status = self.lib.dl_session_run(self.handle, C.byref(progress.raw) if progress else None)
        if status != 0:
            _raise(self.lib, status)

    def result(self) -> BakedScene:
        out = C.POINTER(DlBakedScene)()
        status = self.lib.dl_session_result(self.handle, C.byref(out))
        if status != 0:
            _raise(self.lib, status)
        try:
            return scene_from_c(out.contents)
        finally:
            self.lib.dl_baked_scene_free(out)

    def report(self) -> DlBakeReport:
        r = DlBakeReport()
        self.lib.dl_session_report(self.handle, C.byref(r))
        return r

    def encode_payload(self) -> tuple:
        """The last run's .dynlight payload built on the device and its CRC-32
        (dl_session_encode_payload)."""
        data = C.POINTER(C.c_uint8)()
        length = C.c_uint64()
        crc = C.c_uint32()
        status = self.lib.dl_session_encode_payload(self.handle, C.byref(data), C.byref(length), C.byref(crc))
        if status != 0:
            _raise(self.lib, status)
        try:
            return bytes(np.ctypeslib.as_array(data, shape=(length.value,))), crc.value
        finally:
            self.lib.dl_free(data)

    def bounce_map(self, mesh_id: int, slot: int):
        """The last run's filtered bounce map of (mesh id, light slot) before quantization:
        (window (min_x, min_y, max_x, max_y), float32 array [h, w, 3]), or None without one."""
        rect = np.zeros(4, np.uint32)
        n = C.c_uint32()
        status = self.lib.dl_session_bounce_map(self.handle, mesh_id, slot, rect.ctypes.data, None, 0,
                                                C.byref(n))
        if status != 0:
            _raise(self.lib, status)
        if n.value == 0:
            return None
        rgb = np.zeros(n.value * 3, np.float32)
        status = self.lib.dl_session_bounce_map(self.handle, mesh_id, slot, rect.ctypes.data,
                                                rgb.ctypes.data, n.value, C.byref(n))
        if status != 0:
            _raise(self.lib, status)
        w, h = int(rect[2] - rect[0] + 1), int(rect[3] - rect[1] + 1)
        return tuple(int(x) for x in rect), rgb.reshape(h, w, 3)

    def occluder_bvh(self):
        """The session's occluder BVH as the traversal reads it: (nodes uint32 [n, 16] — child
        boxes as float bits, then the two child references as int32 bits and two zero words —,
        triangles float32 [occluders, 12] in leaf order, depth)."""
        n, depth = C.c_uint32(), C.c_uint32()
        status = self.lib.dl_session_occluder_bvh(self.handle, None, 0, None, 0, C.byref(n), C.byref(depth))
        if status != 0:
            _raise(self.lib, status)
        occluders = int(self.report().occluders)
        nodes = np.zeros((n.value, 16), np.uint32)
        tris = np.zeros((occluders, 12), np.float32)
        status = self.lib.dl_session_occluder_bvh(self.handle, nodes.ctypes.data, n.value, tris.ctypes.data,
                                                  occluders, C.byref(n), C.byref(depth))
        if status != 0:
            _raise(self.lib, status)
        return nodes, tris, depth.value

    def close(self):
        if self.handle:
            self.lib.dl_session_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def encode_payload(scene_c) -> tuple:
    """The uncompressed .dynlight payload and its CRC-32 (src/bake/format/mod.rs:170-213)."""
    lib = load_library()
    data = C.POINTER(C.c_uint8)()
    length = C.c_uint64()
    crc = C.c_uint32()
    status = lib.dl_encode_payload(scene_c, C.byref(data), C.byref(length), C.byref(crc))
    if status != 0:
        _raise(lib, status)
    try:
        return bytes(np.ctypeslib.as_array(data, shape=(length.value,))), crc.value
    finally:
        lib.dl_free(data)


# The .dynlight file and the shader-side word reader: host code over finished bakes.
from . import dynlight_file, mirror  # noqa: E402,F401
