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

MAX_TEXELS = 512 * 512  # DL_NOALLOC_MAX_TEXELS
INVALID_ARGUMENT = 21


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


@pytest.mark.gpu
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


@pytest.mark.gpu
def test_noalloc_filter_takes_a_window_of_exactly_its_limit():
    """A 512 x 512 window (DL_NOALLOC_MAX_TEXELS texels) is accepted and filtered as the oracle's
    BounceMap filters the same window (dilation and blur of bounce_map.rs:67-112)."""
    torch = pytest.importorskip("torch")
    lib = dl.load_library()
    size = 512
    rng = np.random.default_rng(7)
    n = 3000
    xs, ys = rng.integers(0, size, n), rng.integers(0, size, n)
    vals = rng.random((n, 3), dtype=np.float32)
    tex = np.concatenate([np.stack([xs, ys], 1).astype(np.float32), vals], 1).astype(np.float32)
    want = np.zeros(size * size * 3, np.float32)
    win = (C.c_uint32 * 4)()
    oracle.lib().oracle_bounce_map(size, (C.c_uint32 * 4)(4, 4, size - 5, size - 5), ptr(np.ascontiguousarray(tex)),
                                   n, ptr(want), win)
    assert list(win) == [0, 0, size - 1, size - 1]
    pre = np.zeros((size, size, 3), np.float32)
    for (x, y), v in zip(zip(xs, ys), vals):  # later texels overwrite earlier ones, as BounceMap::set
        pre[y, x] = v
    dev = torch.device("cuda:0")
    src = torch.from_numpy(pre.reshape(-1)).to(dev)
    out = torch.full((size * size * 3,), float("nan"), dtype=torch.float32, device=dev)
    status = lib.dl_filter_bounce_window_noalloc(C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()), size, size,
                                                 0, 0, size, None)
    assert status == 0, lib.dl_last_error()
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), want)


@pytest.mark.gpu
def test_noalloc_filter_rejects_one_texel_beyond_its_limit_without_launching():
    """A 1 x (DL_NOALLOC_MAX_TEXELS + 1) window in real device buffers of that size is rejected
    before any launch: the output keeps its sentinel."""
    torch = pytest.importorskip("torch")
    lib = dl.load_library()
    n = MAX_TEXELS + 1
    dev = torch.device("cuda:0")
    src = torch.zeros(n * 3, dtype=torch.float32, device=dev)
    out = torch.full((n * 3,), float("nan"), dtype=torch.float32, device=dev)
    status = lib.dl_filter_bounce_window_noalloc(C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()), 1, n,
                                                 0, 0, n, None)
    assert status == INVALID_ARGUMENT
    assert b"texels" in lib.dl_last_error()
    torch.cuda.synchronize()
    assert bool(torch.isnan(out).all())


def test_noalloc_filter_checks_its_arguments_before_any_cuda_call():
    """Size, map and overlap checks return before the library touches CUDA (so they run on a
    host without a GPU): over the limit in either shape, windows outside the map, and input and
    output ranges that overlap by any amount."""
    lib = dl.load_library()
    f = lib.dl_filter_bounce_window_noalloc
    a, b = 1 << 20, 1 << 24  # never dereferenced: every call below is rejected on the host
    assert f(C.c_void_p(a), C.c_void_p(b), 513, 513, 0, 0, 1024, None) == INVALID_ARGUMENT
    assert f(C.c_void_p(a), C.c_void_p(b), 512, 513, 0, 0, 1024, None) == INVALID_ARGUMENT
    assert f(C.c_void_p(a), C.c_void_p(b), 1, MAX_TEXELS + 1, 0, 0, MAX_TEXELS + 1, None) == INVALID_ARGUMENT
    assert b"texels" in lib.dl_last_error()
    assert f(C.c_void_p(a), C.c_void_p(b), 0, 4, 0, 0, 16, None) == INVALID_ARGUMENT
    assert f(C.c_void_p(a), C.c_void_p(b), 8, 8, 9, 0, 16, None) == INVALID_ARGUMENT
    assert b"inside the map" in lib.dl_last_error()
    window = 8 * 8 * 3 * 4  # bytes of an 8 x 8 window
    for shift in (0, 4, window - 4, -(window - 4)):
        assert f(C.c_void_p(a), C.c_void_p(a + shift), 8, 8, 0, 0, 16, None) == INVALID_ARGUMENT, shift
        assert b"overlap" in lib.dl_last_error()
    assert f(None, C.c_void_p(b), 8, 8, 0, 0, 16, None) == INVALID_ARGUMENT
