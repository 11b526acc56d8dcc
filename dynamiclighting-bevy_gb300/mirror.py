"""Reads baked words the way the runtime shader does: a triangle's header, its light entries,
and shadow and bounce texels at lightmap coordinates; the distance cube fetch; sky probe
openness. Host code over finished bakes (src/bake/mirror.rs:1-130, which mirrors the shader's
`DynamicTriangle` load / set-active-light / shadow and bounce reads; src/bake/format/types.rs:95-101
for the probes). It computes nothing of the bake itself.

Word layout (src/bake/triangle_words.rs:1-13): triangle t's header is the four words at 4t —
the offset of its light data, then the padded bounds `(min_x - 2, min_y - 2, width + 4)` with
unsigned wrap-around; at the light-data offset, the light count and then per light
`(light slot, shadow offset[, bounce offset])`, three words when the scene has bounce data.
Texel (x, y) of a triangle's grid is at `(y - min_y + 2) * W + (x - min_x + 2)` in unsigned
32-bit arithmetic, so coordinates left of or above the map wrap like the shader's."""
from dataclasses import dataclass

import numpy as np

MAX_TRIANGLE_LIGHTS = 256  # the shader clamps a corrupt light count to this
DISTANCE_CUBE_WORDS = 64 * 64 * 3  # per light: six 64x64 faces of f16, two per word
_U32 = 0xFFFFFFFF


@dataclass(frozen=True)
class LightEntry:
    light_index: int    # the light's slot in the baked light list
    shadow_offset: int  # word offset of its shadow grid, 0 when it has none
    bounce_offset: int  # word offset of its bounce grid, 0 when it has none


class TriangleView:
    """One triangle of a mesh's `dynamic_triangles` words."""

    def __init__(self, words, triangle_index, bounce_layout):
        self.words = np.asarray(words, np.uint32)
        header = self.words[4 * triangle_index: 4 * triangle_index + 4]
        self._data = int(header[0]) + 1
        self.bounds = (int(header[1]), int(header[2]), int(header[3]))
        self.light_count = min(int(self.words[int(header[0])]), MAX_TRIANGLE_LIGHTS)
        self._stride = 3 if bounce_layout else 2

    @classmethod
    def load(cls, words, triangle_index, bounce_layout):
        return cls(words, triangle_index, bounce_layout)

    def light(self, k):
        """The k-th light entry (k < light_count)."""
        at = self._data + k * self._stride
        bounce = int(self.words[at + 2]) if self._stride == 3 else 0
        return LightEntry(int(self.words[at]), int(self.words[at + 1]), bounce)

    def entries(self):
        return [self.light(k) for k in range(self.light_count)]

    def entry_for(self, light_index):
        """The entry of baked light slot `light_index`, or None when the triangle has none."""
        for e in self.entries():
            if e.light_index == light_index:
                return e
        return None

    def _grid_index(self, x, y):
        lx = (x - self.bounds[0]) & _U32
        ly = (y - self.bounds[1]) & _U32
        return (ly * self.bounds[2] + lx) & _U32

    def shadow_value(self, entry, x, y, bits):
        """The light reaching lightmap texel (x, y), 0 to 1, for a light stored with `bits` per
        texel (1, 4 or 8); None when the entry holds no shadow grid."""
        if entry.shadow_offset == 0:
            return None
        index = self._grid_index(x & _U32, y & _U32)
        per_word, top = 32 // bits, (1 << bits) - 1
        word = int(self.words[entry.shadow_offset + index // per_word])
        return float(np.float32((word >> ((index % per_word) * bits)) & top) / np.float32(top))

    def shadow_bit(self, entry, x, y):
        """Whether a one-bit (hard) shadow texel is lit; None without a shadow grid."""
        v = self.shadow_value(entry, x, y, 1)
        return None if v is None else v > 0.5

    def bounce_texel(self, entry, x, y, bits_per_pixel):
        """The stored (square-rooted) white bounce at (x, y), 0 to 1."""
        index = self._grid_index(x & _U32, y & _U32)
        per_word, top = 32 // bits_per_pixel, (1 << bits_per_pixel) - 1
        word = int(self.words[entry.bounce_offset + index // per_word])
        return float(np.float32((word >> ((index % per_word) * bits_per_pixel)) & top) / np.float32(top))

    def bounce_texel_rgb(self, entry, x, y, bits_per_pixel):
        """The stored (square-rooted) red, green and blue of a colored bounce texel: three
        `bits_per_pixel` channels packed back to back across word boundaries."""
        index = self._grid_index(x & _U32, y & _U32)
        pixel_bits, top = 3 * bits_per_pixel, (1 << bits_per_pixel) - 1
        offset, shift = divmod(index * pixel_bits, 32)
        at = entry.bounce_offset + offset
        value = int(self.words[at]) >> shift
        if shift + pixel_bits > 32:
            value |= (int(self.words[at + 1]) << (32 - shift)) & _U32
        return tuple(float(np.float32((value >> (c * bits_per_pixel)) & top) / np.float32(top))
                     for c in range(3))


def distance_cube_value(cubes, light, index):
    """The stored distance of cube texel `index` of the light in BVH slot `light` (f16 pairs)."""
    word = int(np.asarray(cubes, np.uint32)[light * DISTANCE_CUBE_WORDS + (index >> 1)])
    return float(np.uint16((word >> ((index & 1) * 16)) & 0xFFFF).view(np.float16))


def probe_openness(probes, x, y, z):
    """The six openness values (+X, -X, +Y, -Y, +Z, -Z; 0 to 1) of sky probe (x, y, z): probes
    x fastest, then y, then z, two words each, one unorm8 per axis."""
    cx, cy, _ = probes.counts
    index = (z * cy + y) * cx + x
    w = np.asarray(probes.words, np.uint32)[2 * index: 2 * index + 2]
    return [float(np.float32((int(w[a // 4]) >> (8 * (a % 4))) & 0xFF) / np.float32(255.0)) for a in range(6)]
