"""Failure handling on the GPU: cancellation in the middle of a bake and an exhausted device
memory budget. Neither faults, traps or hangs the GPU: the cancel flag is set from a host thread
(BakeProgress::cancel, src/bake/progress.rs:84-109) and polled by the device work queues, and
the memory failure is a cap the library enforces before it asks the driver for memory.

The reference checks its cancel flag between work items (src/bake/mesh_bake.rs:82,85,225,
src/bake/bounce.rs:57,135,171) and returns BakeError::Cancelled; an allocation failure has no
counterpart there (Rust aborts), here it is DL_OUT_OF_MEMORY.
"""
import threading
import time

import pytest

import dynlight_gb300 as dl
from dynlight_gb300 import scenes
from tests import fixtures as fx

pytestmark = pytest.mark.gpu


def timed_run(session, progress=None):
    t0 = time.perf_counter()
    session.run(progress)
    return time.perf_counter() - t0


def test_cancel_mid_bake_stops_the_device_queue_and_the_next_run_is_intact():
    """A quarter-size outdoor bake (2.6 M visibility work items): cancelled from a host thread
    15-35 ms into a run, the run reports Cancelled well before an uncancelled run would end, at
    least one cancel lands while the persistent kernels run (warps of the device queue stop on
    the flag), and the next run of the same session, and a fresh bake, equal an uncancelled bake
    byte for byte."""
    inp, opts = scenes.outdoor(grid=257, chunks=4, boxes=500, point_lights=8)
    session = dl.Session(inp, opts)
    try:
        session.run()  # the first run of a scene shape also times launch shapes
        full = min(timed_run(session) for _ in range(3))
        fresh = session.result()
        assert session.report().work_items > 1_000_000
        stops = []
        for delay in (0.015, 0.025, 0.035, 0.020):
            progress = dl.BakeProgress()
            timer = threading.Timer(delay, progress.cancel)
            t0 = time.perf_counter()
            timer.start()
            with pytest.raises(dl.BakeError) as err:
                session.run(progress)
            took = time.perf_counter() - t0
            timer.join()
            assert err.value.kind == "Cancelled", str(err.value)
            assert took < 0.75 * full + 0.005, (delay, took, full)
            stops.append(session.report().cancel_stops)
            session.run()  # no cancel: everything from the cancelled run is reset
            again = session.result()
            assert again.words_equal(fresh) and again.stats == fresh.stats, delay
        assert max(stops) > 0, stops  # the device queue saw the flag at least once
    finally:
        session.close()
    baked = dl.bake(inp, opts)
    assert baked.words_equal(fresh) and baked.stats == fresh.stats


def test_cancel_through_dl_bake_reports_the_stop():
    """dl_bake_ex with a cancel during the bake: Cancelled, and its report says how the device
    queue stopped."""
    inp, opts = scenes.outdoor(grid=257, chunks=4, boxes=500, point_lights=8)
    dl.bake(inp, opts)  # warm: launch shapes are cached per process
    for delay in (0.030, 0.040, 0.050):
        progress = dl.BakeProgress()
        report = dl._abi.DlBakeReport()
        timer = threading.Timer(delay, progress.cancel)
        timer.start()
        with pytest.raises(dl.BakeError) as err:
            dl.bake(inp, opts, progress=progress, report=report)
        timer.join()
        assert err.value.kind == "Cancelled"
        if report.cancel_stops > 0:
            return
    pytest.fail("no cancel reached the running device queue")


def test_device_memory_cap_gives_out_of_memory_and_the_next_bake_succeeds():
    """Caps from 1 MiB upwards: each capped bake either fails with DL_OUT_OF_MEMORY (in scene
    upload, BVH build or a stage's buffers) or equals the uncapped bake; after every failure an
    uncapped bake still equals it."""
    inp, opts = fx.determinism_room()
    for light in inp.lights[:2]:
        light.illumination = dl.SINGLE_BOUNCE
        light.bounce = dl.BakeBounce(samples=16)
    opts.photon_cube_resolution = 64
    report = dl._abi.DlBakeReport()
    fresh = dl.bake(inp, opts, report=report)
    need = report.device_bytes
    failures = successes = 0
    mib = 1
    while True:
        try:
            got = dl.bake(inp, opts, max_device_mib=mib)
        except dl.BakeError as e:
            assert e.status == 17 and "device memory cap" in str(e), str(e)  # DL_OUT_OF_MEMORY
            failures += 1
            again = dl.bake(inp, opts)
            assert again.words_equal(fresh) and again.stats == fresh.stats
        else:
            assert got.words_equal(fresh) and got.stats == fresh.stats
            successes += 1
            break
        mib += 1 if mib < 8 else mib // 2
        assert mib < 4 * (need >> 20) + 64, (mib, need)
    assert failures > 0 and successes == 1
