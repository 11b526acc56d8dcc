"""Output comparison for precision reports.

Two bakes of the same input are compared output by output: every (mesh, triangle, light) entry
of the dynamic-triangle words (src/bake/triangle_words.rs:47-89) is decoded, and the bits of its
shadow payload (one mask per light class: 1-bit hard, 4-bit soft, 8-bit sky levels,
src/bake/shadow_grid.rs:91-106) and of its bounce payload (src/bake/bounce_pack.rs:28-86) are
compared word by word. An entry present in one bake only (optimize dropped it in the other,
src/bake/shadows.rs:54-73) counts all its set bits as flips. Bounce irradiance is compared on
the filtered maps before quantization (src/bake/bounce_map.rs:67-137).
"""
from collections import defaultdict

import numpy as np


def _popcount(words: np.ndarray) -> int:
    if words.size == 0:
        return 0
    return int(np.unpackbits(np.ascontiguousarray(words, np.uint32).view(np.uint8)).sum())


def entries(scene):
    """{(mesh id, triangle, light slot): (shadow words or None, bounce words or None)}."""
    stride = 3 if scene.settings["bounce"] else 2
    out = {}
    for mesh in scene.meshes:
        w = np.asarray(mesh.triangles, np.uint32)
        if w.size == 0:
            continue
        tris = int(w[0]) // 4
        refs = []  # (triangle, slot, kind, payload offset)
        for t in range(tris):
            off = int(w[4 * t])
            for k in range(int(w[off])):
                e = off + 1 + k * stride
                slot = int(w[e])
                if w[e + 1]:
                    refs.append((t, slot, 0, int(w[e + 1])))
                if stride == 3 and w[e + 2]:
                    refs.append((t, slot, 1, int(w[e + 2])))
                out.setdefault((mesh.id, t, slot), [None, None])
        # payloads are appended in entry order, so each ends where the next begins
        starts = sorted(r[3] for r in refs) + [w.size]
        end_of = {s: e for s, e in zip(starts[:-1], starts[1:])}
        for t, slot, kind, start in refs:
            out[(mesh.id, t, slot)][kind] = w[start:end_of[start]]
    return {k: tuple(v) for k, v in out.items()}


def bit_flips(a, b):
    """Flipped bits of bake `a` against bake `b`, per output class: {"1-bit", "4-bit", "8-bit",
    "bounce"} -> {"flips": n, "bits": total payload bits of b, "entries": entries that differ}."""
    ea, eb = entries(a), entries(b)
    bits_of = {i: l.shadow_bits_per_texel for i, l in enumerate(b.lights)}
    res = defaultdict(lambda: {"flips": 0, "bits": 0, "entries": 0})
    for key in set(ea) | set(eb):
        slot = key[2]
        pa = ea.get(key, (None, None))
        pb = eb.get(key, (None, None))
        for kind, cls in ((0, f"{bits_of.get(slot, 1)}-bit"), (1, "bounce")):
            x, y = pa[kind], pb[kind]
            if x is None and y is None:
                continue
            if y is not None:
                res[cls]["bits"] += int(y.size) * 32
            if x is not None and y is not None and x.size == y.size:
                n = _popcount(x ^ y)
            else:
                n = (_popcount(x) if x is not None else 0) + (_popcount(y) if y is not None else 0)
            res[cls]["flips"] += n
            res[cls]["entries"] += int(n > 0)
    return dict(res)


def bounce_error(maps_a, maps_b, floor=1.0e-4):
    """Relative error of bounce maps `maps_a` against `maps_b` ({(mesh id, slot): (window,
    [h, w, 3])}): per texel |a - b| / max(|b|, floor * max|b| of its map). Returns
    {"max": worst, "mean": average over texels, "texels": texels compared, "maps": maps}."""
    worst, total, count = 0.0, 0.0, 0
    for key, (rect_b, vb) in maps_b.items():
        if key not in maps_a:
            continue
        rect_a, va = maps_a[key]
        if rect_a != rect_b or va.shape != vb.shape:
            raise ValueError(f"bounce map windows differ for {key}: {rect_a} vs {rect_b}")
        va64, vb64 = va.astype(np.float64), vb.astype(np.float64)
        scale = max(float(np.abs(vb64).max()), 0.0)
        if scale == 0.0:
            err = np.abs(va64 - vb64)
        else:
            err = np.abs(va64 - vb64) / np.maximum(np.abs(vb64), floor * scale)
        worst = max(worst, float(err.max()))
        total += float(err.sum())
        count += err.size
    return {"max": worst, "mean": total / count if count else 0.0, "texels": count,
            "maps": len(maps_b)}


def session_maps(session, scene):
    """Every filtered bounce map of a Session's last run, keyed like bounce_error's input."""
    maps = {}
    for mesh in scene.meshes:
        for slot in range(len(scene.lights)):
            m = session.bounce_map(mesh.id, slot)
            if m is not None:
                maps[(mesh.id, slot)] = m
    return maps
