"""Output comparison for precision reports.

Two bakes of the same input are compared output by output: every (mesh, triangle, light) entry
of the dynamic-triangle words (src/bake/triangle_words.rs:47-89) is decoded, and the bits of its
shadow payload (one mask per light class: 1-bit hard, 4-bit soft, 8-bit sky levels,
src/bake/shadow_grid.rs:91-106) and of its bounce payload (src/bake/bounce_pack.rs:28-86) are
compared word by word. An entry present in one bake only (optimize dropped it in the other,
src/bake/shadows.rs:54-73) counts all its set bits as flips. Bounce irradiance is compared on
the filtered maps before quantization (src/bake/bounce_map.rs:67-137).
"""
import numpy as np


_PC16 = np.array([bin(i).count("1") for i in range(1 << 16)], np.uint8)


def _popcounts(words: np.ndarray) -> np.ndarray:
    """Set bits of each uint32 word."""
    w = np.ascontiguousarray(words, np.uint32)
    return _PC16[w & 0xFFFF].astype(np.int64) + _PC16[w >> 16]


def _popcount(words: np.ndarray) -> int:
    return int(_popcounts(words).sum()) if words.size else 0


def _layout(words: np.ndarray, stride: int):
    """Entries of one mesh's words as arrays: triangle, light slot, shadow and bounce payload
    offsets (0 when absent), and the end of the light-data block."""
    w = np.asarray(words, np.uint32)
    tris = int(w[0]) // 4
    offs = w[0:4 * tris:4].astype(np.int64)
    cnt = w[offs].astype(np.int64)
    n = int(cnt.sum())
    tri = np.repeat(np.arange(tris), cnt)
    k = np.arange(n) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    e = np.repeat(offs, cnt) + 1 + k * stride
    slot = w[e].astype(np.int64)
    shadow = w[e + 1].astype(np.int64)
    bounce = w[e + 2].astype(np.int64) if stride == 3 else np.zeros(n, np.int64)
    header_end = int(offs[-1] + 1 + cnt[-1] * stride) if tris else 0
    return tri, slot, shadow, bounce, header_end


def entries(scene):
    """{(mesh id, triangle, light slot): (shadow words or None, bounce words or None)}."""
    stride = 3 if scene.settings["bounce"] else 2
    out = {}
    for mesh in scene.meshes:
        w = np.asarray(mesh.triangles, np.uint32)
        if w.size == 0:
            continue
        tri, slot, shadow, bounce, _ = _layout(w, stride)
        # payloads are appended in entry order, so each ends where the next begins
        starts = np.sort(np.concatenate([shadow[shadow > 0], bounce[bounce > 0]]))
        ends = dict(zip(starts.tolist(), np.append(starts[1:], w.size).tolist()))
        for t, sl, so, bo in zip(tri.tolist(), slot.tolist(), shadow.tolist(), bounce.tolist()):
            out[(mesh.id, t, sl)] = (w[so:ends[so]] if so else None, w[bo:ends[bo]] if bo else None)
    return out


def _classes(b):
    bits = [l.shadow_bits_per_texel for l in b.lights]
    return [f"{x}-bit" for x in sorted(set(bits))] + ["bounce"], bits


def bit_flips(a, b):
    """Flipped bits of bake `a` against bake `b`, per output class: {"1-bit", "4-bit", "8-bit",
    "bounce"} -> {"flips": n, "bits": total payload bits of b, "entries": entries that differ}.
    Meshes whose entry layout is the same in both are compared word for word with vector
    operations; the others entry by entry."""
    names, bits = _classes(b)
    index = {n: i for i, n in enumerate(names)}
    slot_class = np.array([index[f"{x}-bit"] for x in bits] + [0], np.int64)
    flips = np.zeros(len(names), np.int64)
    total = np.zeros(len(names), np.int64)
    differ = np.zeros(len(names), np.int64)
    stride = 3 if b.settings["bounce"] else 2
    slow = []
    for ma, mb in zip(a.meshes, b.meshes):
        wa, wb = np.asarray(ma.triangles, np.uint32), np.asarray(mb.triangles, np.uint32)
        if wb.size == 0 and wa.size == 0:
            continue
        if wa.size != wb.size or wb.size == 0:
            slow.append((ma, mb))
            continue
        tri, slot, shadow, bounce, header_end = _layout(wb, stride)
        if not np.array_equal(wa[:header_end], wb[:header_end]):
            slow.append((ma, mb))
            continue
        # label every payload word with its entry's class, then sum popcounts per class
        starts = np.concatenate([shadow[shadow > 0], bounce[bounce > 0]])
        cls = np.concatenate([slot_class[slot[shadow > 0]], np.full(int((bounce > 0).sum()), index["bounce"])])
        order = np.argsort(starts)
        starts, cls = starts[order], cls[order]
        if starts.size == 0:
            continue
        seg = np.searchsorted(starts, np.arange(starts[0], wb.size), side="right") - 1
        xor = _popcounts(wa[starts[0]:] ^ wb[starts[0]:])
        flips += np.bincount(cls[seg], weights=xor, minlength=len(names)).astype(np.int64)
        total += np.bincount(cls[seg], minlength=len(names)) * 32
        per_seg = np.bincount(seg, weights=xor, minlength=starts.size)
        differ += np.bincount(cls, weights=(per_seg > 0), minlength=len(names)).astype(np.int64)
    res = {n: {"flips": int(flips[i]), "bits": int(total[i]), "entries": int(differ[i])}
           for i, n in enumerate(names)}
    if slow:
        ea = entries(type(a)(a.settings, a.lights, a.light_bvh, [m for m, _ in slow], a.distance_cubes, a.stats))
        eb = entries(type(b)(b.settings, b.lights, b.light_bvh, [m for _, m in slow], b.distance_cubes, b.stats))
        for key in set(ea) | set(eb):
            pa = ea.get(key, (None, None))
            pb = eb.get(key, (None, None))
            for kind, cls_name in ((0, f"{bits[key[2]]}-bit"), (1, "bounce")):
                x, y = pa[kind], pb[kind]
                if x is None and y is None:
                    continue
                if y is not None:
                    res[cls_name]["bits"] += int(y.size) * 32
                if x is not None and y is not None and x.size == y.size:
                    n = _popcount(x ^ y)
                else:
                    n = (_popcount(x) if x is not None else 0) + (_popcount(y) if y is not None else 0)
                res[cls_name]["flips"] += n
                res[cls_name]["entries"] += int(n > 0)
    return {k: v for k, v in res.items() if v["bits"] or v["flips"]}


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
