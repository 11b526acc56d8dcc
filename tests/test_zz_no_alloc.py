"""The non-allocating bounce filter (dl_filter_bounce_window_noalloc) against the bake.

For callers that cannot allocate device memory, the library filters one bounce-map window in
their own buffers, with its intermediate in a fixed device array. This test feeds it the
pre-filter window of one (mesh, light) of a bake (captured from the oracle, whose gathers match
the GPU bake word for word), calls it twice in a row, and checks each output against the bounce
words the existing entry point, dl_bake, wrote for every triangle of that window: 8-bit white
bounce has no dither, so each stored byte is floor(sqrt(clamp(v)) * 255) of the filtered value.
"""
import ctypes as C

import numpy as np
import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import scenes
from oracle import oracle
from oracle.oracle import f32, ptr

pytestmark = pytest.mark.gpu


def bounce_scene():
    inp, opts = scenes.small_room()
    for l in inp.lights:
        l.illumination = dl.SINGLE_BOUNCE
        l.bounce = dl.BakeBounce(samples=16)
    opts.photon_cube_resolution = 64
    opts.bounce_compression = 8
    return inp, opts


def capture(inp, opts, mesh_id, slot):
    L = oracle.lib()
    L.oracle_capture_bounce(C.c_uint64(mesh_id), C.c_uint32(slot))
    oracle.bake(inp, opts)
    rect = (C.c_uint32 * 4)()
    size = C.c_uint32()
    cap = 1 << 20
    pre = np.zeros(cap * 3, np.float32)
    post = np.zeros(cap * 3, np.float32)
    n = L.oracle_captured_bounce(rect, C.byref(size), ptr(pre), ptr(post), cap)
    assert n > 0
    return list(rect), size.value, pre[:n * 3].copy(), post[:n * 3].copy()


def expected_bytes(filtered, rect, crop):
    """The padded crop grid's 8-bit bounce values (bounce_pack.rs:74-86 without dither)."""
    x0, y0, x1, _ = rect
    w = x1 - x0 + 1
    gw, gh = crop[2] - crop[0] + 5, crop[3] - crop[1] + 5
    out = []
    for gy in range(gh):
        for gx in range(gw):
            v = np.float32(0)
            if 2 <= gx < gw - 2 and 2 <= gy < gh - 2:
                x, y = crop[0] + gx - 2, crop[1] + gy - 2
                v = filtered[((y - y0) * w + (x - x0)) * 3]
            c = np.float32(min(max(v, np.float32(0)), np.float32(1)))
            out.append(int(np.float32(np.sqrt(c)) * np.float32(255)))
    return out


def stored_bytes(words, offset, count):
    return [(int(words[offset + i // 4]) >> (8 * (i % 4))) & 0xFF for i in range(count)]


def test_noalloc_filter_matches_the_bake_twice_in_a_row():
    torch = pytest.importorskip("torch")
    lib = dl.load_library()
    inp, opts = bounce_scene()
    baked = dl.bake(inp, opts)                       # the existing entry point
    room = baked.meshes[0]
    words = room.triangles
    # the light with the most bounce entries on the room's triangles
    counts = {}
    for t in range(inp.meshes[0].triangle_count()):
        ld = int(words[4 * t])
        for k in range(int(words[ld])):
            light, _, boff = (int(x) for x in words[ld + 1 + 3 * k: ld + 4 + 3 * k])
            counts[light] = counts.get(light, 0) + (boff != 0)
    slot = max(counts, key=counts.get)
    assert counts[slot] > 0
    rect, size, pre, post = capture(inp, opts, room.id, slot)
    w, h = rect[2] - rect[0] + 1, rect[3] - rect[1] + 1
    dev = torch.device("cuda:0")
    src = torch.from_numpy(pre).to(dev)
    stream = torch.cuda.current_stream(dev)
    mesh = inp.meshes[0]
    res = room.resolution
    checked = 0
    outputs = []
    for call in range(2):
        out = torch.full((w * h * 3,), float("nan"), dtype=torch.float32, device=dev)
        status = lib.dl_filter_bounce_window_noalloc(C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()), w, h,
                                                     rect[0], rect[1], size, C.c_void_p(stream.cuda_stream))
        assert status == 0, lib.dl_last_error()
        torch.cuda.synchronize()
        filtered = out.cpu().numpy()
        outputs.append(filtered)
        assert np.array_equal(filtered, post), "filter differs from the oracle's BounceMap"
        for t in range(mesh.triangle_count()):
            ld = int(words[4 * t])
            for k in range(int(words[ld])):
                light, _, boff = (int(x) for x in words[ld + 1 + 3 * k: ld + 4 + 3 * k])
                if light != slot or boff == 0:
                    continue
                uv = mesh.uv1[mesh.indices[3 * t: 3 * t + 3]].reshape(-1)
                rects = (C.c_uint32 * 12)()
                oracle.lib().oracle_rects(ptr(f32(*uv)), res, rects)
                crop = list(rects)[0:4]
                want = expected_bytes(filtered, rect, crop)
                assert stored_bytes(words, boff, len(want)) == want, (call, t)
                checked += 1
    assert checked > 0
    assert np.array_equal(outputs[0], outputs[1])


def test_noalloc_filter_rejects_windows_beyond_its_limit():
    lib = dl.load_library()
    side = 513  # 513^2 > DL_NOALLOC_MAX_TEXELS
    status = lib.dl_filter_bounce_window_noalloc(C.c_void_p(16), C.c_void_p(32), side, side, 0, 0, 1024, None)
    assert status == 21  # DL_INVALID_ARGUMENT
    assert b"texels" in lib.dl_last_error()
