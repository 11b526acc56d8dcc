"""Benchmark: shadow rays/s and bake time of the GPU baker on a seeded synthetic workload, with
the CPU oracle (a restatement of the reference's CPU baker) timed on the host cores beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

A step is one bake of the workload. `value` is the device-resident throughput: shadow rays
(BakeStats.rays + bounce_rays) per second of device time of every bake stage, with the scene and
its BVH resident. `e2e` is the same metric through dl_bake_ex() from host buffers: validation,
BVH build, uploads, the device pipeline, download and serialization. The L2 is flushed (a 256 MiB
write) before every timed step. Multi-GPU runs are independent replicas (the bake shards by
scene, with no exchange step): one rank per GPU, each baking the full workload.

The roofline of the dominant kernel (the persistent visibility kernel) divides its algorithmic
bytes (node visits x 64 B + triangle tests x 48 B + 76 B per work item, counted by the
instrumented variant) by the L2 read bandwidth measured in the same run. On a 1-GPU run the CPU
leg times the oracle once on the full workload on every host core (and checks that its words
equal the GPU's), and measures the target's bounce clause on the workload's seeded CPU sample:
the bounce maps of the bit-exact and refined forms against the FP64 oracle.

`--impl reference` times the oracle alone on the host cores, one bounded sample of the workload
per step (the same seeded sample the bounce clause uses), and prints the same metric.
"""
import argparse
import ctypes as C
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
# The headline metric, printed identically by both arms so their lines compare directly.
METRIC = "shadow rays/s & bake ms: batched vs plain GPU at bit-exact masks; CPU ref"
# The cache read-bandwidth probe behind the roofline: a buffer that fits in L2 (129 MB).
L2_PROBE_BYTES = 64 << 20

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


def cpu_baseline(name, full=None):
    """The oracle, all host threads: on the bounded sample of the workload, or on the full
    workload when `full` gives its (input, options)."""
    from oracle import oracle
    if full is not None:
        (inp, opts), desc = full, "the full workload"
    else:
        make, desc = CPU_SAMPLES[name]
        inp, opts = make()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    scene, burial, _ = oracle.bake(inp, opts, threads=threads)
    dt = time.perf_counter() - t0
    rays = scene.stats["rays"] + scene.stats["bounce_rays"]
    return {"value": rays / dt, "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": f"{desc}: {rays} shadow rays + {burial} burial rays in {dt:.2f} s", "seconds": dt,
            "scene": scene}


def precision_slice(name, device):
    """The bounce clause of the target on the workload's seeded CPU sample: the filtered bounce
    maps of the bit-exact (batched) and refined forms against the FP64 oracle's, as the maximum
    relative error (dynlight_gb300.compare.bounce_error), and the refined form's device time there.
    The oracle is the checker here."""
    from dynlight_gb300 import compare
    from oracle import oracle
    make, desc = CPU_SAMPLES[name]
    inp, opts = make()
    t0 = time.perf_counter()
    ref64 = oracle.bake_ex(inp, opts, mode=oracle.F64, threads=os.cpu_count() or 1, bounce_maps=True)
    out = {"slice": desc, "fp64_oracle_s": round(time.perf_counter() - t0, 2)}
    for form in ("batched", "refined", "bounce_refined"):
        s = dl.Session(inp, opts, form=form, device=device)
        try:
            s.run()
            scene = s.result()
            maps = compare.session_maps(s, scene)
        finally:
            s.close()
        err = compare.bounce_error(maps, ref64["maps"])
        flips = compare.bit_flips(scene, ref64["scene"])
        out[form] = {"bounce_max_rel_err_vs_fp64": err["max"], "bounce_mean_rel_err_vs_fp64": err["mean"],
                     "bounce_maps": err["maps"], "bounce_texels": err["texels"],
                     "mask_bits_differing_from_fp64": {k: v["flips"] for k, v in flips.items() if k != "bounce"}}
    return out


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
    line = {"impl": "reference", "metric": METRIC, "value": value,
            "unit": "rays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded generator)",
            "config": {"workload": name, "description": WORKLOADS[name][1],
                       "timed_sample": CPU_SAMPLES[name][1],
                       "why_a_sample": "each step bakes a bounded sample of the workload (rays/s is intensive); "
                                       "the full workload takes about 80 s per bake on 16 cores",
                       "sample": last["sample"]},
            "cpu_baseline": {"value": value, "unit": "rays/s", "cores": last["cores"], "kind": last["kind"],
                             "sample": last["sample"]},
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
    dev_ms, vis_ms, gather_ms = [], [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush_l2(torch, flush)
            session.run()
            r = session.report()
            dev_ms.append(r.ms_device)
            vis_ms.append(r.ms_visibility)
            gather_ms.append(r.ms_gather)
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
    # the roof: the L2 read bandwidth measured now, on this GPU (the BVH is L2-resident), and the
    # L1 read bandwidth beside it (most node reads hit L1)
    probe_lib = dl.load_library()
    l2_gbs, l1_gbs = C.c_double(), C.c_double()
    assert probe_lib.dl_probe_read_bandwidth(local, 2, L2_PROBE_BYTES, 100, C.byref(l2_gbs)) == 0, \
        probe_lib.dl_last_error()
    assert probe_lib.dl_probe_read_bandwidth(local, 1, L2_PROBE_BYTES, 400, C.byref(l1_gbs)) == 0, \
        probe_lib.dl_last_error()

    traffic = g_traffic = None
    traffic_path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(traffic_path):  # DRAM bytes per launch from an ncu capture (profiles/)
        with open(traffic_path) as f:
            captured = json.load(f)
        entry, g_entry = captured.get(args.workload), captured.get(args.workload + ":k_gather")
        traffic = entry["bytes_per_launch"] if entry else None
        g_traffic = g_entry["bytes_per_launch"] if g_entry else None
    # the second hot kernel, the bounce gather: node visits x 64 B + triangle tests x 48 B of the
    # instrumented gather, plus per item the texel, face and value (52 B), over its event time
    gms = statistics.median(gather_ms)
    g_bytes = crep.gather_node_visits * 64 + crep.gather_tri_tests * 48 + rep.bounce_items * 52
    roofline_gather = None
    if gms > 0 and crep.gather_node_visits:
        g_achieved = g_bytes / (gms / 1e3) / 1e9
        roofline_gather = {
            "bound": "l2", "kernel": "k_gather", "achieved": g_achieved, "peak": l2_gbs.value, "unit": "GB/s",
            "frac": g_achieved / l2_gbs.value if l2_gbs.value else None,
            "peak_source": "the same L2 read bandwidth measurement",
            "limiter": "instruction issue (ncu on the quarter-size outdoor case: issue slots 71 % busy, "
                       "SIMT efficiency 40 %, L2 throughput 8.4 % of peak)",
            "algorithmic_bytes_per_launch": int(g_bytes), "ms": gms, "traffic": g_traffic,
            "bytes_per_unit": "64 per node visit + 48 per triangle test + 52 per (bounce pair, texel) item",
            "node_visits": int(crep.gather_node_visits), "tri_tests": int(crep.gather_tri_tests),
            "items": int(rep.bounce_items)}

    # the refined form (binary64 edge re-tests, compensated sums) on the same scene
    refined = dl.Session(inp, opts, form="refined", device=local)
    refined_ms = []
    for i in range(3):
        refined.run()
        if i:
            refined_ms.append(refined.report().ms_device)
    refined_retests = int(refined.report().retests)
    refined.close()
    # the bounce-refined form: the batched form's masks with the refined form's bounce
    hybrid = dl.Session(inp, opts, form="bounce_refined", device=local)
    hybrid_ms = []
    for i in range(3):
        hybrid.run()
        if i:
            hybrid_ms.append(hybrid.report().ms_device)
    from dynlight_gb300 import compare
    hybrid_flips = compare.bit_flips(hybrid.result(), result)
    hybrid_masks_equal = all(v["flips"] == 0 for k, v in hybrid_flips.items() if k != "bounce")
    hybrid.close()

    # end to end through the C ABI (dl_bake_ex) from host buffers: validation, BVH build,
    # uploads, the device pipeline and the download of every mesh's words, timed around the call
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
        "metric": METRIC,
        "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": args.workload, "description": desc, "form": "batched",
                   "triangles": int(inp.triangle_count()), "lights": len(inp.lights),
                   "texels": int(result.stats["texels"]), "shadow_rays": int(rays),
                   "burial_rays": int(rep.burial_rays), "pairs": int(rep.pairs),
                   "l2": "flushed (256 MiB write) before every timed step",
                   "batched_ms": ms, "plain_form_ms": plain_rep.ms_device,
                   "plain_visibility_ms": plain_rep.ms_visibility, "batched_visibility_ms": vis,
                   "batched_gather_ms": statistics.median(gather_ms),
                   "speedup_batched_vs_plain": plain_rep.ms_device / ms if ms else None,
                   "masks_batched_equal_plain": True,
                   "refined_ms": statistics.median(refined_ms), "refined_retests": refined_retests,
                   "bounce_refined_ms": statistics.median(hybrid_ms),
                   "bounce_refined_masks_equal_batched": hybrid_masks_equal,
                   "launch_shape": {"chunk_texels": rep.tuned_chunk_texels, "sample_lanes": rep.tuned_sample_lanes,
                                    "blocks_per_sm": rep.tuned_blocks_per_sm,
                                    "stack_depth": rep.tuned_stack_depth, "launch_bound_blocks": rep.tuned_min_blocks,
                                    "gather_lanes": rep.tuned_gather_lanes,
                                    "gather_blocks_per_sm": rep.tuned_gather_blocks_per_sm,
                                    "gather_launch_bound_blocks": rep.tuned_gather_min_blocks,
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
        "roofline": {"bound": "l2", "kernel": "k_trace_batched", "achieved": achieved, "peak": l2_gbs.value,
                     "unit": "GB/s", "frac": achieved / l2_gbs.value if l2_gbs.value else None,
                     "peak_source": f"measured in this run: L2 read bandwidth of this GPU, a {L2_PROBE_BYTES >> 20} MiB "
                                    "buffer streamed 100 times with L1-bypassing loads (dl_probe_read_bandwidth)",
                     "l1_read_gbs": l1_gbs.value, "hbm_gbs": hbm, "hbm_source": f"{peak_kind} (MEASURED_PEAKS.json)",
                     "traffic": traffic, "traffic_frac_of_algorithmic": traffic / alg_bytes if traffic else None,
                     "limiter": "instruction issue (ncu on the quarter-size outdoor case: issue slots 74 % busy, "
                                "SIMT efficiency 54 %, L2 throughput 3.9 % of peak)",
                     "algorithmic_bytes_per_launch": int(alg_bytes),
                     "bytes_per_unit": "64 per node visit + 48 per triangle test + 76 per (pair, texel) item",
                     "node_visits": int(crep.node_visits), "tri_tests": int(crep.tri_tests),
                     "items": int(crep.work_items)},
        "roofline_gather": roofline_gather,
    }
    if not args.no_cpu_baseline and world == 1:  # the CPU baseline: rank 0 of a 1-GPU run
        # the oracle on the full workload, all host cores, once; its words are the GPU's
        cb = cpu_baseline(args.workload, full=(inp, opts))
        cb.pop("seconds")
        cpu_scene = cb.pop("scene")
        cb["words_equal_gpu"] = bool(cpu_scene.words_equal(result)) and cpu_scene.stats == result.stats
        line["cpu_baseline"] = cb
        # the target's bounce clause on the seeded CPU sample of the workload
        if args.workload in ("outdoor", "outdoor_small", "room_grid"):
            line["config"]["precision"] = precision_slice(args.workload, local)
            p = line["config"]["precision"]
            line["config"]["bounce_err_vs_fp64_bitexact"] = p["batched"]["bounce_max_rel_err_vs_fp64"]
            line["config"]["bounce_err_vs_fp64_refined"] = p["refined"]["bounce_max_rel_err_vs_fp64"]
            line["config"]["bounce_err_vs_fp64_bounce_refined"] = p["bounce_refined"]["bounce_max_rel_err_vs_fp64"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
