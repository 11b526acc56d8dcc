"""Benchmark: shadow rays/s and bake time of the GPU baker on a seeded synthetic workload, with
the CPU oracle (a restatement of the reference's CPU baker) timed on the host cores beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

A step is one bake of the workload. `value` is the device-resident throughput: shadow rays
(BakeStats.rays + bounce_rays) per second of device time of every bake stage, with the scene and
its BVH resident. `e2e` is the same metric through dl_bake() from host buffers: validation, BVH
build, uploads, the device pipeline, download and serialization. The L2 is flushed (a 256 MiB
write) before every timed step. Multi-GPU runs are independent replicas (the bake shards by
scene, with no exchange step): one rank per GPU, each baking the full workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from __graft_entry__ import load_package  # noqa: E402

dl = load_package()
from dynlight_gb300 import scenes  # noqa: E402

PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    # name: (generator, description)
    "outdoor": (lambda: scenes.outdoor(),
                "512x512 fBm heightfield (522k tris, 8x8 chunks) + 2000 boxes/planks = 546k tris; 0.53 deg "
                "sun, 4-bit, 5 probes + 16..32 disk samples; colored sun bounce, 128 samples; sky, 256 samples; "
                "32 point lights; 4 texels/m"),
    "room_grid": (lambda: scenes.room_grid(),
                  "6x6 rooms 8x3.5x8 m with doorways, 20 boxes/ramps each (44.5k tris); 64 point lights, "
                  "radius U[4,12]; 1-bit shadows + one bounce, 64 gather samples, 512^2 photon cubes; 16 texels/m"),
    "soft_rooms": (lambda: scenes.soft_rooms(),
                   "6x6 rooms re-meshed with log-normal triangles (106k tris), 128 lights (64 point, 32 rectangle, "
                   "32 tube), 4-bit soft shadows from 5/3 probes + 16 samples, 16 texels/m"),
    "small_room": (lambda: scenes.small_room(),
                   "10x4x10 m room + 5 cubes (72 tris), 4 point lights, 1-bit, 8 texels/m"),
    # a quarter-size outdoor scene with the same lights and samples: the case ncu captures
    "outdoor_small": (lambda: scenes.outdoor(grid=257, chunks=4, boxes=500, point_lights=8),
                      "256x256 m of the outdoor terrain (131k tris + 500 boxes), same sun/sky/bounce, 8 points"),
}
# The CPU baseline bakes a smaller instance of the same generator with the same light kinds and
# sample counts (rays/s is intensive).
CPU_SAMPLES = {
    "outdoor": (lambda: scenes.outdoor(grid=97, chunks=2, boxes=72, point_lights=2),
                "96x96 m of the same terrain generator with 72 boxes, 2 point lights, the same sun/sky/bounce"),
    "room_grid": (lambda: scenes.room_grid(rooms=2, lights=7), "2x2 rooms, 7 lights, same samples"),
    "soft_rooms": (lambda: scenes.soft_rooms(rooms=2, lights=14, boxes_per_room=20), "2x2 rooms, 14 lights"),
    "small_room": (lambda: scenes.small_room(), "the full workload"),
    "outdoor_small": (lambda: scenes.outdoor(grid=97, chunks=2, boxes=72, point_lights=2),
                      "96x96 m of the same terrain generator with 72 boxes, 2 point lights, the same sun/sky/bounce"),
}


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons}


def rank_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_baseline(name, seconds_cap=60.0):
    """The oracle, all host threads, on the bounded sample of the workload."""
    from oracle import oracle
    make, desc = CPU_SAMPLES[name]
    inp, opts = make()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    scene, burial, _ = oracle.bake(inp, opts, threads=threads)
    dt = time.perf_counter() - t0
    rays = scene.stats["rays"] + scene.stats["bounce_rays"]
    return {"value": rays / dt, "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": f"{desc}: {rays} shadow rays + {burial} burial rays in {dt:.2f} s", "seconds": dt}


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return
    name = args.workload
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(name)
    for _ in range(args.steps):
        vals.append(cpu_baseline(name))
    value = statistics.median(v["value"] for v in vals)
    last = vals[-1]
    ms = statistics.median(v["seconds"] for v in vals) * 1e3
    line = {"impl": "reference", "metric": "shadow rays/s (bake of the workload)", "value": value,
            "unit": "rays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded generator)",
            "config": {"workload": name, "description": WORKLOADS[name][1], "sample": last["sample"]},
            "cpu_baseline": {k: last[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def whole_job(rays, ms, world, device):
    """Replicas: each rank bakes its workload in `ms`; the job takes the slowest rank's time and
    processes every rank's rays. Returns (rays/s of the job, the job's ms)."""
    if world == 1:
        return rays / (ms / 1e3), ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    n = torch.tensor([float(rays)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(n.item()) / (float(t.item()) / 1e3), float(t.item())


def flush_l2(torch_mod, buf):
    buf.zero_()
    torch_mod.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="outdoor", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank, world, local = rank_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    make, desc = WORKLOADS[args.workload]
    inp, opts = make()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    # device-resident: one session, repeated runs
    session = dl.Session(inp, opts, form="batched", device=local)
    tune = None
    for _ in range(args.warmup):
        session.run()
        if tune is None:
            tune = session.report()  # the first run times candidate launch shapes (then cached)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    dev_ms, vis_ms = [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush_l2(torch, flush)
            session.run()
            r = session.report()
            dev_ms.append(r.ms_device)
            vis_ms.append(r.ms_visibility)
    torch.cuda.synchronize()
    result = session.result()
    rep = session.report()
    # the plain form (one launch per mesh), same scene, for the batched/plain ratio
    plain = dl.Session(inp, opts, form="plain", device=local)
    plain.run()
    plain_rep = plain.report()
    plain_result = plain.result()
    plain.close()
    rays = result.stats["rays"] + result.stats["bounce_rays"]
    ms = statistics.median(dev_ms)
    value, t_max = whole_job(rays, ms, world, f"cuda:{local}")

    # roofline of the dominant kernel (the persistent visibility kernel): algorithmic bytes from
    # an instrumented run of the same kernel on the same BVH (node visits x 64 B, triangle tests
    # x 48 B) plus the per-item texel/pair reads and result writes (76 B per (pair, texel) item)
    counted = dl.Session(inp, opts, form="batched", device=local, count_visits=1)
    counted.run()
    crep = counted.report()
    counted.close()
    vis = statistics.median(vis_ms)
    hbm, peak_kind = peaks()
    alg_bytes = crep.node_visits * 64 + crep.tri_tests * 48 + crep.work_items * 76
    achieved = alg_bytes / (vis / 1e3) / 1e9 if vis > 0 else 0.0
    traffic = None
    traffic_path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(traffic_path):  # DRAM bytes per launch from an ncu capture (profiles/)
        with open(traffic_path) as f:
            entry = json.load(f).get(args.workload)
        traffic = entry["bytes_per_launch"] if entry else None

    # end to end through the C ABI (dl_bake_ex) from host buffers: validation, BVH build,
    # uploads, the device pipeline and the download of every mesh's words, timed around the call
    import ctypes as C
    lib = dl.load_library()
    marshalled = dl.Marshalled(inp)
    copts = dl.marshal_options(opts)
    ccfg = dl.make_config("batched", device=local)
    e2e_ms = []
    e2e_rep = dl._abi.DlBakeReport()
    scene = None
    for i in range(max(3, args.steps // 2)):
        flush_l2(torch, flush)
        out = C.POINTER(dl._abi.DlBakedScene)()
        t0 = time.perf_counter()
        status = lib.dl_bake_ex(C.byref(marshalled.input), C.byref(copts), C.byref(ccfg), None, C.byref(out),
                                C.byref(e2e_rep))
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        assert status == 0, lib.dl_last_error()
        if scene is None:
            scene = dl.scene_from_c(out.contents)
        lib.dl_baked_scene_free(out)
    assert scene.words_equal(result) and scene.words_equal(plain_result), "forms disagree"
    e2e_value, _ = whole_job(rays, statistics.median(e2e_ms), world, f"cuda:{local}")

    if rank != 0:
        return
    line = {
        "metric": "shadow rays/s (bake of the workload, device-resident)",
        "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": args.workload, "description": desc, "form": "batched",
                   "triangles": int(inp.triangle_count()), "lights": len(inp.lights),
                   "texels": int(result.stats["texels"]), "shadow_rays": int(rays),
                   "burial_rays": int(rep.burial_rays), "pairs": int(rep.pairs),
                   "l2": "flushed (256 MiB write) before every timed step",
                   "plain_form_ms": plain_rep.ms_device, "plain_visibility_ms": plain_rep.ms_visibility,
                   "batched_visibility_ms": vis,
                   "speedup_batched_vs_plain": plain_rep.ms_device / ms if ms else None,
                   "launch_shape": {"chunk_texels": rep.tuned_chunk_texels, "sample_lanes": rep.tuned_sample_lanes,
                                    "blocks_per_sm": rep.tuned_blocks_per_sm,
                                    "stack_depth": rep.tuned_stack_depth, "launch_bound_blocks": rep.tuned_min_blocks,
                                    "autotune_trials": tune.tune_trials if tune else 0,
                                    "autotune_ms": tune.ms_tune if tune else 0.0},
                   "parallelism": f"replicas x{world}"},
        "clocks": clocks.summary(),
        "gpu_launches": int(rep.kernel_launches),
        "e2e": {"value": e2e_value, "unit": "rays/s", "ms": statistics.median(e2e_ms),
                "h2d_bytes_per_step": int(e2e_rep.h2d_bytes), "d2h_bytes_per_step": int(e2e_rep.d2h_bytes),
                "ms_validate_sort": e2e_rep.ms_host[0], "ms_bvh_build": e2e_rep.ms_host[1],
                "ms_flatten_upload": e2e_rep.ms_host[2], "ms_device": e2e_rep.ms_device,
                "ms_download_serialize": e2e_rep.ms_download},
        "roofline": {"bound": "hbm", "kernel": "k_trace_batched", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": traffic, "algorithmic_bytes_per_launch": int(alg_bytes),
                     "node_visits": int(crep.node_visits), "tri_tests": int(crep.tri_tests),
                     "items": int(crep.work_items)},
    }
    if not args.no_cpu_baseline and world == 1:  # the CPU baseline: rank 0 of a 1-GPU run
        cb = cpu_baseline(args.workload)
        cb.pop("seconds")
        line["cpu_baseline"] = cb
    print(json.dumps(line))


if __name__ == "__main__":
    main()
