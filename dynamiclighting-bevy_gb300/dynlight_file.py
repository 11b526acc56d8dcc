"""The `.dynlight` file around a bake (src/bake/format/mod.rs:1-304, codec.rs, lights.rs,
maps.rs): a 24-byte header — magic "DYNLIGHT", format version 6 (u32 LE), the uncompressed
payload length (u64 LE) and the payload's CRC-32 (u32 LE) — then a gzip stream of the payload.

`write_payload` gives the same payload bytes as the library's `dl_encode_payload` and the
device-side `Session.encode_payload`; `container` wraps a payload in the header and gzip (mtime 0,
OS byte 255, level 6, as the reference's flate2 writer sets them; the deflate bytes themselves
differ between deflate libraries, which loaders do not see). `decode` checks magic, version,
length and checksum, then parses the payload with the reference's validity rules and raises
`FormatError` with the reference's error kinds. Host code; no part of the bake."""
import struct
import zlib

import numpy as np

from . import BakedLight, BakedMesh, BakedScene, SkyProbes, SunMap

MAGIC = b"DYNLIGHT"
FORMAT_VERSION = 6
HEADER_BYTES = 24
MAX_SUN_MAP_RESOLUTION = 8192
MAX_SKY_PROBES = 65536
SUN_SHAPE, SKY_SHAPE = 3, 4
_LIGHT_BYTES, _SUN_MAP_BYTES, _MESH_BYTES = 60, 60, 32


class FormatError(Exception):
    """FormatError (format/mod.rs:50-78): kind is one of NotDynlight, UnsupportedVersion,
    Truncated, Decompress, ChecksumMismatch, Invalid; `what` names the invalid field, `found`
    and `supported` the versions."""

    def __init__(self, kind, what=None, found=None):
        self.kind, self.what, self.found, self.supported = kind, what, found, FORMAT_VERSION
        messages = {
            "NotDynlight": "not a .dynlight file (bad magic)",
            "UnsupportedVersion": f".dynlight format version {found} is not supported (this build reads "
                                  f"version {FORMAT_VERSION}); re-bake the scene",
            "Truncated": ".dynlight file is truncated or has corrupt lengths",
            "Decompress": f".dynlight payload doesn't decompress: {what}",
            "ChecksumMismatch": ".dynlight payload checksum mismatch",
            "Invalid": f".dynlight file has an invalid {what}",
        }
        super().__init__(messages[kind])

    def __eq__(self, other):
        return (isinstance(other, FormatError) and (self.kind, self.found) == (other.kind, other.found)
                and (self.kind == "Decompress" or self.what == other.what))

    def __hash__(self):
        return hash((self.kind, self.what, self.found))


# ---- writing ----------------------------------------------------------------------------------

def _words(a):
    a = np.ascontiguousarray(np.asarray(a, np.uint32).reshape(-1))
    return struct.pack("<Q", a.size) + a.astype("<u4", copy=False).tobytes()


def write_payload(scene):
    """The payload sections in order (format/mod.rs:170-213, lights.rs:27-52, maps.rs:16-38)."""
    s = scene.settings
    out = [struct.pack("<IIfII", int(bool(s["bounce"])) | int(bool(s["colored_bounce"])) << 1,
                       s["dynamic_geometry"], s["pixel_density"], s["max_lightmap_size"],
                       s["distance_cube_resolution"]),
           struct.pack("<Q", len(scene.lights))]
    for l in scene.lights:
        out.append(struct.pack("<Q4fII4f2fI", l.id, *l.origin, l.radius, l.bounce_bits, l.shape,
                               *l.rotation, *l.size[:2], l.shadow_bits_per_texel))
    out.append(_words(scene.light_bvh))
    out.append(struct.pack("<Q", len(scene.meshes)))
    for m in scene.meshes:
        out.append(struct.pack("<QQII", m.id, m.content_hash, m.resolution, int(bool(m.occludes))))
        out.append(_words(m.triangles))
    out.append(_words(scene.distance_cubes))
    out.append(struct.pack("<Q", len(scene.sun_maps)))
    for sm in scene.sun_maps:
        out.append(struct.pack("<I", sm.resolution) + np.asarray(sm.rows, "<f4").reshape(-1).tobytes())
        out.append(_words(sm.texels))
    p = scene.sky_probes
    out.append(struct.pack("<I", int(p is not None)))
    if p is not None:
        out.append(struct.pack("<4f3I", *p.origin, p.spacing, *p.counts))
        out.append(_words(p.words))
    st = scene.stats
    out.append(struct.pack("<I6Q", st["meshes"], st["triangles"], st["texels"], st["rays"],
                           st["lights_removed"], st["bounce_rays"], st["triangle_words"]))
    return b"".join(out)


def container(payload, crc=None):
    """The file bytes of `payload`: header, then a gzip stream (format/mod.rs:101-119)."""
    crc = zlib.crc32(payload) if crc is None else crc
    head = MAGIC + struct.pack("<IQI", FORMAT_VERSION, len(payload), crc)
    deflate = zlib.compressobj(6, zlib.DEFLATED, -15)
    body = deflate.compress(payload) + deflate.flush()
    gz = b"\x1f\x8b\x08\x00" + struct.pack("<I", 0) + b"\x00\xff"  # no flags, mtime 0, XFL 0, OS 255
    return head + gz + body + struct.pack("<II", zlib.crc32(payload), len(payload) & 0xFFFFFFFF)


def encode(scene):
    """encode (format/mod.rs:101-119): the whole file of a baked scene."""
    return container(write_payload(scene))


# ---- reading ----------------------------------------------------------------------------------

class _Bytes:
    """A payload held whole, read front to back."""

    def __init__(self, data):
        self.data, self.at = memoryview(data), 0

    def read(self, n):
        b = self.data[self.at:self.at + n]
        self.at += len(b)
        return b


class _UnexpectedEnd(Exception):
    """The gzip stream ended before its trailer."""


class _Inflating:
    """The payload inflated from a gzip file object as it is read, with its CRC-32 and length
    kept over the bytes handed out (stream.rs:12-26)."""

    def __init__(self, source):
        self.source, self.inflate, self.pending = source, zlib.decompressobj(16 + 15), b""
        self.crc = self.count = 0

    def read(self, n):
        parts, have = [], 0
        while have < n:
            if not self.pending:
                if self.inflate.eof:
                    break
                chunk = self.inflate.unconsumed_tail or self.source.read(1 << 16)
                if not chunk:
                    raise _UnexpectedEnd()
                try:
                    self.pending = self.inflate.decompress(chunk, max(n - have, 1 << 16))
                except zlib.error as e:
                    raise FormatError("Decompress", str(e)) from None
                continue
            part, self.pending = self.pending[:n - have], self.pending[n - have:]
            parts.append(part)
            have += len(part)
        out = b"".join(parts)
        self.crc, self.count = zlib.crc32(out, self.crc), self.count + len(out)
        return out


class _Reader:
    """Little-endian values off a payload of declared length, every length checked against
    what is left (codec.rs: a count whose items cannot fit is Truncated)."""

    def __init__(self, source, length):
        self.source, self.left = source, length

    def remaining(self):
        return self.left

    def take(self, n):
        if n > self.left:
            raise FormatError("Truncated")
        try:
            b = self.source.read(n)
        except _UnexpectedEnd:  # codec.rs maps an early end of the stream to Truncated
            raise FormatError("Truncated") from None
        if len(b) != n:
            raise FormatError("Truncated")
        self.left -= n
        return b

    def unpack(self, fmt):
        return struct.unpack(fmt, self.take(struct.calcsize(fmt)))

    def u32(self):
        return self.unpack("<I")[0]

    def count(self, item_bytes):
        n = self.unpack("<Q")[0]
        if n * max(item_bytes, 1) > self.left:
            raise FormatError("Truncated")
        return n

    def words(self):
        n = self.count(4)
        return np.frombuffer(self.take(4 * n), "<u4").astype(np.uint32)


def _finite(values):
    return bool(np.all(np.isfinite(np.float32(values))))


def _group(shape):
    return 2 if shape == SKY_SHAPE else 1 if shape == SUN_SHAPE else 0


def _lights(r):
    lights = []
    for _ in range(r.count(_LIGHT_BYTES)):
        lid, ox, oy, oz, radius, bounce, shape = r.unpack("<Q4fII")
        if bounce not in (0, 4, 5, 6, 8):
            raise FormatError("Invalid", "bounce compression")
        rotation, size = r.unpack("<4f"), r.unpack("<2f")
        if not (_finite(rotation) and _finite(size)) or shape > SKY_SHAPE:
            raise FormatError("Invalid", "light shape")
        if lights and _group(lights[-1].shape) > _group(shape):
            raise FormatError("Invalid", "light order")
        bits = r.u32()
        if bits not in (1, 2, 4, 8):
            raise FormatError("Invalid", "shadow bits per texel")
        lights.append(BakedLight(lid, (ox, oy, oz), radius, shape, rotation, size, bounce, bits))
    return lights


def _maps(r, suns, skies):
    """maps::decode (maps.rs:40-97): no sun maps or one per sun; sky probes only with a sky."""
    n = r.count(_SUN_MAP_BYTES)
    if n not in (0, suns):
        raise FormatError("Invalid", "sun map count")
    sun_maps = []
    for _ in range(n):
        resolution = r.u32()
        rows = np.float32(r.unpack("<12f")).reshape(3, 4)
        texels = r.words()
        if not (1 <= resolution <= MAX_SUN_MAP_RESOLUTION and _finite(rows)
                and texels.size == (resolution * resolution + 1) // 2):
            raise FormatError("Invalid", "sun map")
        sun_maps.append(SunMap(rows, resolution, texels))
    flag = r.u32()
    if flag == 0:
        return sun_maps, None
    if flag != 1 or skies == 0:
        raise FormatError("Invalid", "sky probes")
    origin, spacing, counts = r.unpack("<3f"), r.unpack("<f")[0], r.unpack("<3I")
    words = r.words()
    total = counts[0] * counts[1] * counts[2]
    if not (_finite(origin) and _finite(spacing) and spacing > 0.0 and min(counts) >= 1
            and total <= MAX_SKY_PROBES and words.size == 2 * total):
        raise FormatError("Invalid", "sky probes")
    return sun_maps, SkyProbes(origin, spacing, counts, words)


def decode_payload(payload):
    """decode_payload (format/mod.rs:215-219) of a payload held whole."""
    return _parse(_Reader(_Bytes(payload), len(payload)))


def _parse(r):
    """parse_payload (format/mod.rs:221-294): the sections in order, nothing read twice."""
    flags, geometry = r.unpack("<II")
    if flags > 3:
        raise FormatError("Invalid", "settings flag")
    if geometry > 2:
        raise FormatError("Invalid", "dynamic geometry mode")
    density, max_size, cube_res = r.unpack("<fII")
    settings = dict(bounce=bool(flags & 1), colored_bounce=bool(flags & 2), dynamic_geometry=geometry,
                    pixel_density=density, max_lightmap_size=max_size, distance_cube_resolution=cube_res)
    lights = _lights(r)
    bvh = r.words()
    if bvh.size % 8:
        raise FormatError("Invalid", "light BVH")
    meshes = []
    for _ in range(r.count(_MESH_BYTES)):
        mid, content_hash, resolution, occludes = r.unpack("<QQII")
        if occludes > 1:
            raise FormatError("Invalid", "mesh shadow flag")
        meshes.append(BakedMesh(mid, content_hash, resolution, r.words(), bool(occludes)))
    cubes = r.words()
    sun_maps, probes = _maps(r, sum(l.shape == SUN_SHAPE for l in lights), sum(l.shape == SKY_SHAPE for l in lights))
    m, *rest = r.unpack("<I6Q")
    stats = dict(zip(("meshes", "triangles", "texels", "rays", "lights_removed", "bounce_rays", "triangle_words"),
                     [m] + rest))
    if r.remaining():
        raise FormatError("Invalid", "trailing payload")
    return BakedScene(settings, lights, bvh.reshape(-1, 8), meshes, cubes, stats, sun_maps, probes)


def _header(head):
    """parse_header (format/mod.rs:126-148): (payload length, checksum)."""
    if len(head) < HEADER_BYTES or head[:8] != MAGIC:
        raise FormatError("NotDynlight" if len(head) >= 8 and head[:8] != MAGIC else "Truncated")
    version, length, checksum = struct.unpack("<IQI", head[8:HEADER_BYTES])
    if version != FORMAT_VERSION:
        raise FormatError("UnsupportedVersion", found=version)
    return length, checksum


def decode(data):
    """decode (format/mod.rs:150-168): header, gzip, length and CRC-32, then the payload."""
    data = bytes(data)
    length, checksum = _header(data[:HEADER_BYTES])
    inflate = zlib.decompressobj(16 + 15)
    try:
        payload = inflate.decompress(data[HEADER_BYTES:], min(length + 1, 1 << 62))
    except zlib.error as e:
        raise FormatError("Decompress", str(e)) from None
    if len(payload) > length:
        raise FormatError("Truncated")
    if not inflate.eof:
        raise FormatError("Decompress", "unexpected end of the gzip stream")
    if len(payload) != length:
        raise FormatError("Truncated")
    if zlib.crc32(payload) != checksum:
        raise FormatError("ChecksumMismatch")
    return decode_payload(payload)


def decode_stream(source):
    """decode_stream (stream.rs:28-71): parses a file object as it is read, holding neither the
    file nor the payload whole; the same result and errors as decode."""
    head = b""
    while len(head) < HEADER_BYTES:
        chunk = source.read(HEADER_BYTES - len(head))
        if not chunk:
            break
        head += chunk
    length, checksum = _header(head)
    inflating = _Inflating(source)
    try:
        scene, error = _parse(_Reader(inflating, length)), None
    except FormatError as e:
        if e.kind == "Decompress":
            raise
        scene, error = None, e
    try:
        if error is None:
            inflating.read(1)  # one byte past the declared length must not exist
        else:
            while inflating.read(1 << 16):
                pass
    except (FormatError, _UnexpectedEnd) as e:
        if error is None:
            raise FormatError("Decompress", str(e) or "unexpected end of the gzip stream") from None
    if inflating.count != length:
        raise FormatError("Truncated")
    if inflating.crc != checksum:
        raise FormatError("ChecksumMismatch")
    if error is not None:
        raise error
    return scene
