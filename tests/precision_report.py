"""Precision report of the precision-stress workload (needs a GPU; prints one JSON line).

    python tests/precision_report.py [--steps K] [--full-grid N]
    python tests/precision_report.py --outdoor

1. The full scene (scenes.precision_stress(): 1024x1024-vertex terrain, 200k decal quads lifted
   1e-4 m, 20k slivers of aspect up to 1e4, 256 mixed lights): device time of the bit-exact
   batched form and of the refined form, the refined form's binary64 re-tests, and the bits in
   which the refined form's output differs from the bit-exact one.
2. A slice of the same generator small enough for the oracle: each GPU form against the
   reference restatement (the binary32 oracle) and against the FP64 oracle, per output class
   (1-bit, 4-bit, 8-bit masks and bounce words), plus the bounce irradiance error against the
   FP64 oracle, for the refined form at epsilon 1e-7, 1e-6, 1e-5 and 1e-4.
With --outdoor: the full 546k-triangle outdoor scene, every GPU form against both oracles.

Test infrastructure: the oracle is what the GPU forms are compared with here, never a path of the product.
"""
import argparse
import json
import os
import statistics
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from __graft_entry__ import load_package  # noqa: E402

dl = load_package()
from dynlight_gb300 import compare, scenes  # noqa: E402
from oracle import oracle  # noqa: E402

SLICE = dict(grid=96, chunks=2, boxes=40, decals=4000, slivers=600, lights=32, sky_samples=64,
             bounce_samples=32)
EPSILONS = (1e-7, 1e-6, 1e-5, 1e-4)


def timed(inp, opts, form, steps, **tuning):
    s = dl.Session(inp, opts, form=form, **tuning)
    try:
        s.run()  # warm-up
        ms = []
        for _ in range(steps):
            s.run()
            ms.append(s.report().ms_device)
        scene = s.result()
        rep = s.report()
        return scene, statistics.median(ms), rep
    finally:
        s.close()


def gpu_with_maps(inp, opts, form, **tuning):
    s = dl.Session(inp, opts, form=form, **tuning)
    try:
        s.run()
        scene = s.result()
        return scene, compare.session_maps(s, scene), s.report()
    finally:
        s.close()


def total(flips):
    return sum(v["flips"] for v in flips.values())


def outdoor_report():
    """The 546k-triangle outdoor scene (C4) in full: the three GPU forms against the binary32
    oracle (the reference restatement) and the FP64 oracle, masks and bounce."""
    import os
    inp, opts = scenes.outdoor()
    threads = os.cpu_count() or 1
    t0 = time.time()
    ref32 = oracle.bake_ex(inp, opts, mode=oracle.F32, threads=threads, bounce_maps=True)
    t32 = time.time() - t0
    t0 = time.time()
    ref64 = oracle.bake_ex(inp, opts, mode=oracle.F64, threads=threads, bounce_maps=True)
    t64 = time.time() - t0
    out = {"report": "precision", "workload": "outdoor", "triangles": int(inp.triangle_count()),
           "texels": int(ref32["scene"].stats["texels"]), "oracle_threads": threads,
           "oracle_f32_s": round(t32, 1), "oracle_f64_s": round(t64, 1),
           "oracle_f32_vs_f64_flips": compare.bit_flips(ref32["scene"], ref64["scene"]),
           "oracle_f32_bounce_error_vs_f64": compare.bounce_error(ref32["maps"], ref64["maps"])}
    for form, tuning in (("batched", {}), ("plain", {}), ("refined", {}), ("refined eps 1e-5", {"refine_epsilon": 1e-5}),
                         ("bounce_refined", {})):
        scene, maps, rep = gpu_with_maps(inp, opts, form.split()[0], **tuning)
        out[form] = {"words_equal_reference": bool(scene.words_equal(ref32["scene"])),
                     "stats_equal_reference": scene.stats == ref32["scene"].stats,
                     "flips_vs_reference": compare.bit_flips(scene, ref32["scene"]),
                     "flips_vs_fp64": compare.bit_flips(scene, ref64["scene"]),
                     "bounce_error_vs_reference": compare.bounce_error(maps, ref32["maps"]),
                     "bounce_error_vs_fp64": compare.bounce_error(maps, ref64["maps"]),
                     "retests": int(rep.retests), "ms_device": round(rep.ms_device, 1)}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--full-grid", type=int, default=1024)
    ap.add_argument("--outdoor", action="store_true",
                    help="compare the GPU forms with both oracles on the full outdoor scene instead")
    args = ap.parse_args()
    if args.outdoor:
        return outdoor_report()
    out = {"report": "precision", "workload": "precision_stress"}

    # 1. the full scene
    t0 = time.time()
    full_kw = {} if args.full_grid == 1024 else dict(grid=args.full_grid, chunks=max(2, args.full_grid // 64))
    inp, opts = scenes.precision_stress(**full_kw)
    out["full"] = {"triangles": int(inp.triangle_count()), "meshes": len(inp.meshes), "lights": len(inp.lights),
                   "generate_s": round(time.time() - t0, 2)}
    exact, exact_ms, exact_rep = timed(inp, opts, "batched", args.steps)
    refined, refined_ms, refined_rep = timed(inp, opts, "refined", args.steps)
    hybrid, hybrid_ms, _ = timed(inp, opts, "bounce_refined", args.steps)
    rays = exact.stats["rays"] + exact.stats["bounce_rays"]
    flips = compare.bit_flips(refined, exact)
    out["full"].update({
        "texels": int(exact.stats["texels"]), "rays": int(rays),
        "batched_ms": exact_ms, "refined_ms": refined_ms,
        "batched_rays_per_s": rays / (exact_ms / 1e3), "refined_rays_per_s": rays / (refined_ms / 1e3),
        "refined_retests": int(refined_rep.retests),
        "refined_vs_exact_flips": flips, "refined_vs_exact_flip_total": total(flips),
        "bounce_refined_ms": hybrid_ms,
        "bounce_refined_vs_exact_flips": compare.bit_flips(hybrid, exact)})

    # 2. the slice against both oracles
    inp, opts = scenes.precision_stress(**SLICE)
    ref32 = oracle.bake_ex(inp, opts, mode=oracle.F32, bounce_maps=True)
    ref64 = oracle.bake_ex(inp, opts, mode=oracle.F64, bounce_maps=True)
    sl = {"config": SLICE, "triangles": int(inp.triangle_count()), "texels": int(ref32["scene"].stats["texels"]),
          "oracle_f32_vs_f64_flips": compare.bit_flips(ref32["scene"], ref64["scene"]),
          "oracle_f32_bounce_error_vs_f64": compare.bounce_error(ref32["maps"], ref64["maps"])}
    scene, maps, _ = gpu_with_maps(inp, opts, "batched")
    sl["batched"] = {"flips_vs_reference": total(compare.bit_flips(scene, ref32["scene"])),
                     "flips_vs_fp64": compare.bit_flips(scene, ref64["scene"]),
                     "bounce_error_vs_fp64": compare.bounce_error(maps, ref64["maps"])}
    scene, maps, _ = gpu_with_maps(inp, opts, "bounce_refined")
    sl["bounce_refined"] = {"flips_vs_reference": compare.bit_flips(scene, ref32["scene"]),
                            "flips_vs_fp64": compare.bit_flips(scene, ref64["scene"]),
                            "bounce_error_vs_fp64": compare.bounce_error(maps, ref64["maps"])}
    sl["refined"] = {}
    for eps in EPSILONS:
        scene, maps, rep = gpu_with_maps(inp, opts, "refined", refine_epsilon=eps)
        want = oracle.bake_ex(inp, opts, mode=oracle.REFINED, eps=eps)["scene"]
        sl["refined"][f"{eps:g}"] = {
            "retests": int(rep.retests),
            "matches_refined_oracle": bool(scene.words_equal(want)),
            "flips_vs_reference": compare.bit_flips(scene, ref32["scene"]),
            "flips_vs_fp64": compare.bit_flips(scene, ref64["scene"]),
            "bounce_error_vs_fp64": compare.bounce_error(maps, ref64["maps"])}
    out["slice"] = sl
    print(json.dumps(out))


if __name__ == "__main__":
    main()
