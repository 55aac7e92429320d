"""Benchmark of the plain FP32 progressive hemicube shooter on one GB300.

Workload (the large batched plain configuration): seeded procedural room
20 x 20 x 5 m with 40 random boxes, ~50,000 quad patches, 4 ceiling emitters,
PHYS update rule, hemicube side 512, K shooters per batch (default 128).
A step is one batch: select K shooters, render + reduce K hemicubes, update
all patches.  Metric: hemicubes/s (higher is better).

  value    device time of the timed steps (CUDA events on the solver stream),
           scene resident in HBM, one CUDA-graph replay per step
  e2e      the same steps through the C ABI with host buffers (page-locked when
           torch is importable, reused every step): per step the unshot/shot state
           is copied host->device, one batch runs, the state is copied back
           device->host, all inside the timed region
  roofline the hemicube raster + reduce kernel (the dominant kernel), timed live
           with CUDA events between stages on the solver stream
  cpu_baseline  the CPU oracle (a C port of the reference's shoot loop with a
           software rasteriser) on a bounded sample of the same workload, all host
           threads

Other configurations: ``--workload small`` (5k-patch Cornell box, W=256, K=10),
``precision`` (20k patches, 192 right-hand sides, gather to 1e-6), ``learned`` (trains the
warm-start network on 2,000 generated scenes, evaluates on 100 held-out 50k-patch rooms;
several minutes) and ``uneven`` (256 scenes under one CUDA graph, then learned + gather).

``--impl reference`` times the reference's CPU path (the oracle port: the
reference's own GL/CL path cannot run without a graphics stack) on the same
workload and prints its line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--k", type=int, default=128, help="shooters per batch")
    p.add_argument("--w", type=int, default=512, help="hemicube side")
    p.add_argument("--patches", type=int, default=50000)
    p.add_argument("--tile", type=int, default=0)
    p.add_argument("--small", type=int, default=0, help="span/warp record split in box pixels (0: default)")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-autotune", action="store_true", help="keep the default raster configuration")
    p.add_argument("--no-headline", action="store_true",
                   help="skip the time-to-residual comparison (learned + BF16 gather vs plain shooter)")
    p.add_argument("--workload", default="large", choices=["large", "small", "precision", "learned", "uneven"],
                   help="large: the headline plain configuration; the others are the other benchmark configs")
    p.add_argument("--fp64-solve", action="store_true", help="precision: also solve the full system in FP64 on CPU")
    p.add_argument("--precision-patches", type=int, default=20000, help="precision: patch count of the scene")
    p.add_argument("--uneven-tol", type=float, default=1e-4, help="uneven: unshot-fraction tolerance per scene")
    p.add_argument("--headline-patches", type=int, default=50000,
                   help="patch count of the time-to-1e-4 comparison scene in the default line")
    p.add_argument("--train-scenes", type=int, default=2000, help="learned: solver-generated training scenes")
    p.add_argument("--train-patches", default="5000,50000", help="learned: training patch range (log-uniform)")
    p.add_argument("--train-sample", type=int, default=2048, help="learned: patches kept per training scene")
    p.add_argument("--train-epochs", type=int, default=50, help="learned: training epochs")
    p.add_argument("--train-batch", type=int, default=16384, help="warm-start network: rows per Adam step")
    p.add_argument("--train-lr", type=float, default=3e-3, help="warm-start network: Adam learning rate")
    p.add_argument("--eval-scenes", type=int, default=100, help="learned: held-out room scenes")
    p.add_argument("--eval-patches", type=int, default=50000, help="learned: patch target of a held-out room")
    p.add_argument("--learned-w", type=int, default=128, help="learned: hemicube side of the training captures")
    p.add_argument("--eval-w", type=int, default=512, help="learned: hemicube side of the held-out evaluation")
    p.add_argument("--save-weights", default="", help="learned: write the trained network here (.npz)")
    p.add_argument("--gen-workers", type=int, default=8, help="learned: scene-generation processes")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x: float, world: int) -> float:
    """The largest x of all ranks (the job's time is its slowest replica's); x itself at N=1."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


RASTER_PROFILE = os.path.join("profiles", "k_raster_room50k_w512.json")


def raster_profile():
    """The committed ncu summary of the raster kernel on this workload (profiles/), with the
    commands that produced it: DRAM traffic per hemicube (one-pass metrics at K=32) and the
    SM-side utilisation of the full section set (K=8).  None when the file is absent."""
    try:
        with open(os.path.join(ROOT, RASTER_PROFILE)) as f:
            return json.load(f)
    except Exception:
        return None


def ncu_traffic(k: int):
    """DRAM bytes per raster launch: the profile's per-hemicube figure x K."""
    prof = raster_profile()
    try:
        return float(prof["traffic"]["dram_bytes_per_hemicube"]) * k
    except Exception:
        return None


def sm_side_ncu():
    """k_raster's SM-side figures and its bounding SM unit, read from the committed profile."""
    prof = raster_profile()
    if not prof or "sm_side" not in prof:
        return None
    out = dict(prof["sm_side"])
    out["source"] = RASTER_PROFILE + " (" + prof["sm_side"].get("capture", "ncu --set full") + ")"
    return out


def cpu_baseline(sc, W, K, seconds):
    """Times the CPU oracle (C port of the shoot loop) on a bounded sample of the workload."""
    from oracle import MODE_PHYS, Oracle

    orc = Oracle()
    threads = os.cpu_count() or 1
    rad = sc["radiosity"].copy()
    ill = sc["illumination"].copy()
    kk = min(K, 2 * threads)
    done = 0
    t0 = time.perf_counter()
    while True:
        rad, ill, st = orc.shoot(MODE_PHYS, W, kk, sc["vertices"], sc["color"], rad, ill, 1,
                                 rho=sc["reflectance"], threads=threads)
        done += int(st.hemicubes)
        el = time.perf_counter() - t0
        if el >= seconds or done >= 4096:
            break
    return {"value": done / el, "unit": "hemicubes/s", "cores": threads, "kind": "port",
            "sample": f"{done} hemicubes ({done // kk} batches of K={kk}) of the same scene, W={W}, "
                      f"PHYS rule, {el:.1f} s wall on {threads} host threads"}


def workload(args):
    from radiosity_gb300 import scenes

    return scenes.room_with_boxes(target=args.patches, seed=args.seed)


def config_block(args, sc, K, extra=None):
    c = {"workload": f"plain FP32 progressive shooter, procedural 20x20x5 m room with 40 boxes, "
                     f"{sc['n']} patches, hemicube {args.w}x{args.w}, K={K} shooters per batch",
         "patches": int(sc["n"]), "hemicube_side": args.w, "shooters_per_batch": K, "update_rule": "PHYS",
         "seed": args.seed, "parallelism": "replicas" if args.gpus > 1 else "single GPU",
         "l2": "per-step working set (triangle records, bin lists, 64-bit FF sums) exceeds the 129 MB L2; "
               "the 5.6 MB scene stays L2-resident as in the real loop"}
    if extra:
        c.update(extra)
    return c


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sc = workload(args)
    K = args.k
    from oracle import MODE_PHYS, Oracle

    orc = Oracle()
    threads = os.cpu_count() or 1
    kk = min(K, 2 * threads)
    rad = sc["radiosity"].copy()
    ill = sc["illumination"].copy()
    for _ in range(max(0, min(args.warmup, 1))):
        rad, ill, _ = orc.shoot(MODE_PHYS, args.w, kk, sc["vertices"], sc["color"], rad, ill, 1,
                                rho=sc["reflectance"], threads=threads)
    times, hemis = [], 0
    budget = 120.0
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rad, ill, st = orc.shoot(MODE_PHYS, args.w, kk, sc["vertices"], sc["color"], rad, ill, 1,
                                 rho=sc["reflectance"], threads=threads)
        times.append(time.perf_counter() - t0)
        hemis += int(st.hemicubes)
        if time.perf_counter() - t_all > budget:
            break
    total = sum(times)
    val = hemis / total
    line = {"metric": "hemicubes/s", "value": val, "unit": "hemicubes/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": len(times), "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural room)",
            "config": config_block(args, sc, K, {"cpu_batch": kk}),
            "cpu_baseline": {"value": val, "unit": "hemicubes/s", "cores": threads, "kind": "port",
                             "sample": f"{len(times)} steps of {kk} hemicubes (K capped at 2 x threads), "
                                       f"the reference's OpenGL/OpenCL path needs a graphics stack and is "
                                       f"unavailable on this box; timed: the C port of its CPU loop"},
            "e2e": {"value": val, "unit": "hemicubes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import radiosity_gb300 as R

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("RAD_BENCH_GLOO") is None else "gloo")
    dev = local
    sc = workload(args)
    K, W = args.k, args.w
    n = sc["n"]
    solver = R.Solver(hemicube_side=W, hemicubes_count=K, mode=R.MODE_PHYS, tile=args.tile,
                      small_tri_pixels=args.small, device=dev)
    solver.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    tuning = None
    if not args.no_autotune:  # picks the raster bin side and span/warp split (state untouched)
        t = solver.autotune(tune_k=False)
        tuning = {"tile": t.tile, "small_tri_pixels": t.small_tri_pixels, "candidates": t.candidates,
                  "us_per_hemicube": t.us_per_hemicube}
    # warm-up (graph capture happens on the first call)
    solver.shoot(args.warmup)
    # live per-stage timing (events between stages on the solver stream)
    solver.set_state(radiosity=sc["radiosity"], illumination=sc["illumination"])
    stage_ms, pst = solver.profile_stages(min(args.steps, 8))
    prof_batches = max(1, int(pst.shots_done))
    counters = {k: v / max(1.0, pst.hemicubes) for k, v in solver.raster_counters().items()}
    # timed region: device-resident state, graph replays
    solver.set_state(radiosity=sc["radiosity"], illumination=sc["illumination"])
    solver.shoot(1)
    clocks = Clocks(dev)
    clocks.start()
    barrier()
    t0 = time.perf_counter()
    st = solver.shoot(args.steps)
    wall = time.perf_counter() - t0
    barrier()
    ck = clocks.stop()
    dev_s = max_over_ranks(st.device_ms / 1000.0, world)
    hemis_local = float(st.hemicubes)
    value = hemis_local * world / dev_s
    # e2e through the C ABI with host buffers: the state lives in pinned host arrays that
    # every step copies in (rad_set_state) and reads back (rad_download)
    rad_h, ill_h, host_kind = host_state_buffers(3 * n)
    rad_h[:] = sc["radiosity"]
    ill_h[:] = sc["illumination"]
    e2e_steps = max(3, min(args.steps, 10))
    solver.set_state(radiosity=rad_h, illumination=ill_h)
    barrier()
    t0 = time.perf_counter()
    e2e_hemi = 0.0
    for _ in range(e2e_steps):
        solver.set_state(radiosity=rad_h, illumination=ill_h)
        s1 = solver.shoot(1)
        solver.download(out=(rad_h, ill_h))
        e2e_hemi += s1.hemicubes
    e2e_s = time.perf_counter() - t0
    barrier()
    if rank != 0:
        solver.close()
        return
    hbm, peak_kind = measured_peaks()
    batches = prof_batches
    raster_ms = stage_ms["raster"] / batches
    setup_ms = stage_ms["setup"] / batches
    algo_bytes = K * (48.0 * n + 4.0 * n)  # per launch: quad vertices once per hemicube + one FF row
    achieved = algo_bytes / (raster_ms / 1000.0) / 1e9
    launches_per_step = 8
    line = {
        "metric": "hemicubes/s", "value": value, "unit": "hemicubes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / max(1, st.shots_done),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural room, 40 boxes, 4 emitters)",
        "config": config_block(args, sc, K, {"tile": int(solver.cfg.tile) or "auto",
                                             "small_tri_pixels": int(solver.cfg.small_tri_pixels) or 64,
                                             "autotune": tuning, "wall_s": wall, "residual_after": st.residual}),
        "e2e": {"value": e2e_hemi / e2e_s, "unit": "hemicubes/s",
                "h2d_bytes_per_step": int(2 * 3 * 4 * n), "d2h_bytes_per_step": int(2 * 3 * 4 * n),
                "steps": e2e_steps, "host_buffers": host_kind},
        "roofline": {"bound": "hbm", "kernel": "k_raster (tile raster + fused delta-FF reduction)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "traffic": ncu_traffic(K),
                     "algorithmic_bytes_per_launch": algo_bytes, "avg_launch_ms": raster_ms,
                     # the raster is SM-bound, not DRAM-bound: its SM-side utilisation and the
                     # bounding SM unit from the committed full-section ncu capture (K=8 case
                     # of the same scene, profiles/k_raster_room50k_w512.json)
                     "sm_side_ncu": sm_side_ncu(),
                     "sm_bound": (lambda p: None if not p else {"unit": p["bounding_unit"],
                                                                 "frac": p["bounding_unit_frac"],
                                                                 "source": RASTER_PROFILE})(sm_side_ncu())},
        "stage_ms_per_step": {k: v / batches for k, v in stage_ms.items()},
        "raster_counters_per_hemicube": counters,
        "gpu_launches": int(launches_per_step * st.shots_done),
        "clocks": ck,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sc, W, K, args.cpu_seconds)
    solver.close()
    if args.headline_patches and not args.no_headline:
        # the metric's time-to-residual half: learned + BF16 gather vs the plain shooter
        try:
            line["time_to_residual"] = learned_headline(args)
        except Exception as e:  # the hemicubes/s line is still reported
            line["time_to_residual"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(line), flush=True)


def run_small(args):
    """Plain method, small: the Cornell-style box (~5,000 patches), W=256, 200 shots, K=10."""
    import radiosity_gb300 as R
    from radiosity_gb300 import scenes

    sc = scenes.cornell_box(target=5000)
    W, K, S = 256, 10, 200
    s = R.Solver(hemicube_side=W, hemicubes_count=K, mode=R.MODE_PHYS)
    s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])
    tune = s.autotune()
    s.shoot(3)
    s.set_state(radiosity=sc["radiosity"], illumination=sc["illumination"])
    t0 = time.perf_counter()
    st = s.shoot(S)
    wall = time.perf_counter() - t0
    s.close()
    line = {"metric": "hemicubes/s", "value": st.hemicubes / (st.device_ms / 1000), "unit": "hemicubes/s",
            "workload": "small", "n_gpus": 1, "steps": S, "ms_per_step": st.device_ms / S,
            "shots_per_s": S / (st.device_ms / 1000), "wall_s_200_shots": wall, "device_s_200_shots": st.device_ms / 1000,
            "residual_after": st.residual, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"Cornell-style box, {sc['n']} patches, W={W}, K={K}, {S} shots, PHYS rule",
                       "tile": tune.tile, "small_tri_pixels": tune.small_tri_pixels}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sc, W, K, args.cpu_seconds)
    print(json.dumps(line), flush=True)


def _emission_vectors(sc, n_vec, rng):
    """n_vec emission vectors (1-4 random emitter patches, U[1,20] per channel) x RGB -> 3 n_vec x N."""
    n = sc["n"]
    E = np.zeros((3 * n_vec, n), np.float32)
    for v in range(n_vec):
        em = rng.choice(n, int(rng.integers(1, 5)), replace=False)
        E[3 * v:3 * v + 3, em] = rng.uniform(1, 20, (3, len(em))).astype(np.float32)
    return E


FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def run_precision(args):
    """Precision form: dense F for N=20,000 (W=512), 64 emission vectors x RGB = 192 RHS, BF16
    tcgen05 gather with iterative refinement to 1e-6, FP64 residual check on the host."""
    import radiosity_gb300 as R
    from radiosity_gb300 import scenes

    sc = scenes.cornell_box(target=args.precision_patches)
    n, W = sc["n"], args.w
    s = R.Solver(hemicube_side=W, hemicubes_count=32, mode=R.MODE_PHYS)
    s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])
    cap_ms = s.dense_capture(keep_fp32=True)
    E = _emission_vectors(sc, 64, np.random.default_rng(args.seed))
    B, st = s.gather(E, tol=1e-6, max_outer=60, sweeps=8)
    F, _, _ = s.dense_rows(0, n)
    s.close()
    rho = sc["reflectance"].reshape(n, 3).astype(np.float64)
    FB = F.astype(np.float64) @ B.T.astype(np.float64)  # N x 192, FP64 residual of the FP32 system
    res = np.zeros(E.shape[0])
    for c in range(E.shape[0]):
        r = E[c] + rho[:, c % 3] * FB[:, c] - B[c]
        res[c] = np.linalg.norm(r) / max(np.linalg.norm(E[c]), 1e-30)
    ld = (n + 63) // 64 * 64
    flops = 2.0 * n * ld * 192 * st.sweeps
    bytes_ = 2.0 * n * ld * st.sweeps
    tf = flops / (st.sweep_ms / 1000) / 1e12 if st.sweep_ms > 0 else 0
    gbs = bytes_ / (st.sweep_ms / 1000) / 1e9 if st.sweep_ms > 0 else 0
    rflops = 2.0 * n * n * 192 * st.outer  # one FP32 residual per refinement check
    rtf = rflops / (st.resid_ms / 1000) / 1e12 if st.resid_ms > 0 else 0
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
    line = {"metric": "time-to-residual<=1e-6 (BF16 tcgen05 gather, 192 RHS)", "value": st.device_ms / 1000,
            "unit": "s", "workload": "precision", "higher_is_better": False, "n_gpus": 1, "dtype": "bf16 x bf16 -> f32",
            "capture_s": cap_ms / 1000, "capture_hemicubes_per_s": n / (cap_ms / 1000),
            "gather": {"outer": st.outer, "sweeps": st.sweeps, "initial_residual": st.initial_residual,
                       "residual": st.residual, "sweep_ms": st.sweep_ms, "resid_ms": st.resid_ms},
            "fp64_residual_max": float(res.max()),
            "roofline": {"kernel": "k_gemm_tc<192, two 128-row tiles per CTA> + k_tc_finalize (tcgen05 BF16 sweep, "
                                   "deterministic split-K)", "bound": "hbm",
                         "achieved": gbs, "peak": float(peaks["hbm_gbs"]), "unit": "GB/s",
                         "frac": gbs / float(peaks["hbm_gbs"]), "tensor_tflops": tf,
                         "tensor_frac": tf / float(peaks["bf16_tflops"]), "peak_kind": "measured"},
            "residual": {"kernel": "k_sgemm_resid + k_sgemm_resid_finalize (FP32, TwoSum-compensated, split-K)",
                         "fp32_tflops": rtf, "nominal_fp32_peak_tflops": FP32_NOMINAL_TFLOPS,
                         "frac_of_nominal": rtf / FP32_NOMINAL_TFLOPS,
                         "note": "CUDA-core FP32: 152 SMs x 128 lanes x 2 flop x 2.07 GHz, nominal (not measured)"},
            "config": {"workload": f"Cornell-style box, {n} patches, W={W}, 64 emission vectors x RGB",
                       "rhs": 192}, "data": "synthetic"}
    if args.fp64_solve:
        t0 = time.perf_counter()
        err = 0.0
        Fd = F.astype(np.float64)
        for ch in range(3):
            A = np.eye(n) - rho[:, ch][:, None] * Fd
            X = np.linalg.solve(A, E[ch::3].T.astype(np.float64))
            err = max(err, float(np.max(np.linalg.norm(B[ch::3].T - X, axis=0) / np.linalg.norm(X, axis=0))))
        line["fp64_solve_rel_error_max"] = err
        line["fp64_solve_s"] = time.perf_counter() - t0
    print(json.dumps(line), flush=True)


def host_state_buffers(count: int):
    """Two float32 host arrays of `count` for the end-to-end loop: page-locked (through torch's
    pinned allocator) when torch is importable, else ordinary numpy arrays."""
    try:
        import torch

        a = torch.empty(count, dtype=torch.float32, pin_memory=True)
        b = torch.empty(count, dtype=torch.float32, pin_memory=True)
        return a.numpy(), b.numpy(), "pinned"
    except Exception:
        return np.empty(count, np.float32), np.empty(count, np.float32), "pageable"


def train_warm_start(args, scenes_n: int = 48, epochs: int = 200, patches=(2000, 6000), kinds=("cornell",),
                     sample=None, W: int = 128, workers: int = 0):
    """Solver-generated training set (seeded scenes, W=128 by default) and the trained MLP."""
    import radiosity_gb300 as R
    from radiosity_gb300 import learned

    t0 = time.perf_counter()
    X, T = learned.training_set(scenes_n, seed=args.seed, patches=patches, W=W, kinds=kinds, sample=sample,
                                workers=workers, form=learned.FORM)
    gen_s = time.perf_counter() - t0
    order = np.random.default_rng(args.seed).permutation(X.shape[0])  # batches mix scenes
    X, T = np.ascontiguousarray(X[order]), np.ascontiguousarray(T[order])
    m = R.MLP(seed=args.seed)
    batch, lr = args.train_batch, args.train_lr
    loss, train_ms = m.train(X, T, epochs=epochs, batch=batch, lr=lr)
    # forward + backward: 3 passes of 2 * (32*128 + 3*128*128 + 128*3) flop per sample
    flop = 6.0 * sum(a * b for a, b in zip(R.MLP.DIMS[:-1], R.MLP.DIMS[1:])) * X.shape[0] * epochs
    return m, {"scenes": scenes_n, "kinds": list(kinds), "patch_range": list(patches), "W": W,
               "samples": int(X.shape[0]), "sample_per_scene": sample, "epochs": epochs, "batch": batch, "lr": lr,
               "final_loss": loss, "train_ms": train_ms, "train_tflops": flop / (train_ms * 1e9),
               "engine": "tcgen05 BF16 GEMMs", "data_gen_s": gen_s, "form": learned.FORM}


def learned_headline(args):
    """Time to residual <= 1e-4 on two 50k-patch scenes -- the large configuration's room
    (reflectance U[0.1, 0.8]) and a Cornell variant (grey walls 0.73, the harder case for a
    shooter) -- learned warm start + BF16 gather vs the plain FP32 shooter (see headline())."""
    from radiosity_gb300 import scenes

    m, training = warm_start_network(args)
    try:
        out = {}
        for name, sc in (("room", scenes.room_with_boxes(target=args.headline_patches, seed=args.seed)),
                         ("cornell", scenes.cornell_variant(args.headline_patches, seed=424242))):
            out[name] = headline(args, m, sc)
    finally:
        m.close()
    out["training"] = training
    return out


def run_learned(args):
    """Learned warm start: train the MLP on solver-generated scenes (rooms and Cornell variants,
    patch counts log-uniform in --train-patches), then, on --eval-scenes held-out seeded rooms
    of the large configuration's generator (40 boxes, 4 ceiling emitters, --eval-patches
    patches), solve to 1e-4 with rad_gather_solve from three starts: emission, emission + direct
    light, and the network's guess.  Reports refinements and device solve time per start."""
    from radiosity_gb300 import learned

    lo, hi = (int(v) for v in args.train_patches.split(","))
    W, We = args.learned_w, args.eval_w
    m, training = train_warm_start(args, scenes_n=args.train_scenes, epochs=args.train_epochs, patches=(lo, hi),
                                   kinds=("room", "cornell"), sample=args.train_sample, W=W,
                                   workers=args.gen_workers)
    if args.save_weights:
        learned.save_network(m, args.save_weights, {"training": training, "features": "learned.features",
                                                   "network": "32-128x4-3 ReLU, BF16 weights",
                                                   "form": learned.FORM})
    names = ("emission", "direct", "learned")
    rows, caps, npat = [], [], []
    t0 = time.perf_counter()
    specs = [("room", args.eval_patches, 10_000 + k, 40, 4) for k in range(args.eval_scenes)]
    for sc in learned.generated(specs, args.gen_workers):
        c0 = time.perf_counter()
        with learned.capture(sc, W=We) as s:
            caps.append(time.perf_counter() - c0)
            npat.append(sc["n"])
            E = learned.emission_block(sc)
            d = learned.direct_light(s, E)
            direct = np.ascontiguousarray((sc["radiosity"].reshape(-1, 3) + d).T, np.float32)
            guess = learned.warm_start(m, sc, d)
            res = {}
            for name, g in zip(names, (None, direct, guess)):
                _, st = s.gather(E, guess=g, tol=1e-4, max_outer=200, sweeps=4)
                res[name] = (st.outer, st.sweeps, st.device_ms, st.initial_residual, st.residual, st.sweep_ms,
                             st.resid_ms)
            rows.append(res)
    eval_s = time.perf_counter() - t0
    m.close()

    def col(k, i):
        return np.array([r[k][i] for r in rows], np.float64)

    summ = {k: {"outer_mean": float(col(k, 0).mean()), "sweeps_mean": float(col(k, 1).mean()),
                "solve_ms_mean": float(col(k, 2).mean()), "solve_ms_p50": float(np.percentile(col(k, 2), 50)),
                "solve_ms_p99": float(np.percentile(col(k, 2), 99)),
                "initial_residual_mean": float(col(k, 3).mean()), "final_residual_max": float(col(k, 4).max()),
                "sweep_ms_mean": float(col(k, 5).mean()), "resid_ms_mean": float(col(k, 6).mean())}
            for k in names}
    line = {"metric": "gather time-to-residual<=1e-4 from the learned guess", "value": summ["learned"]["solve_ms_mean"],
            "unit": "ms", "workload": "learned", "higher_is_better": False, "starts": summ,
            "learned_faster_than_direct_fraction": float(np.mean(col("learned", 2) < col("direct", 2))),
            "speedup_vs_emission": summ["emission"]["solve_ms_mean"] / summ["learned"]["solve_ms_mean"],
            "speedup_vs_direct": summ["direct"]["solve_ms_mean"] / summ["learned"]["solve_ms_mean"],
            "training": training,
            "evaluation": {"scenes": len(rows), "patches_mean": float(np.mean(npat)), "W": We,
                           "capture_s_mean": float(np.mean(caps)), "wall_s": eval_s},
            "config": {"workload": f"MLP 32-128x4-3 BF16; trained on {args.train_scenes} solver-generated scenes "
                                   f"(rooms and Cornell variants, {lo}-{hi} patches, W={W}, {args.train_sample} "
                                   f"patches sampled per scene); evaluated on {args.eval_scenes} held-out seeded "
                                   f"rooms (20x20x5 m, 40 boxes, 4 ceiling emitters, {args.eval_patches} patches, "
                                   f"W={We})"},
            "data": "synthetic"}
    print(json.dumps(line), flush=True)


def headline(args, m, sc):
    """Time to residual <= 1e-4 on one large scene: learned warm start + BF16 gather (dense capture
    included) against the plain FP32 progressive shooter, both at W=args.w on this GPU.

    Both methods solve the same discrete system and stop on its relative L2 residual on the
    captured FP32 rows: the shooter spreads power with the reciprocity form F_ji = F_ij A_i / A_j,
    so its fixed point is B = E + rho o (F^T (A o B)) / A, and the gather runs in the shoot form
    (RAD_DENSE_SHOOT_FORM), which iterates on that same system.  The shooter runs in segments of
    16 batches with its total radiosity (shot + unshot) checked after each (untimed); its own
    unshot-power rule is recorded beside it.  Final answers are checked in FP64 on the host, and
    their relative L2 difference is reported."""
    import radiosity_gb300 as R
    from radiosity_gb300 import learned

    n, W, tol = sc["n"], args.w, 1e-4
    E = learned.emission_block(sc)
    E64 = E.T.astype(np.float64)
    rho = sc["reflectance"].reshape(n, 3).astype(np.float64)
    # learned + gather
    g = R.Solver(hemicube_side=W, hemicubes_count=args.k, mode=R.MODE_PHYS)
    g.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])
    tune = g.autotune()
    cap_ms = g.dense_capture(keep_fp32=True, form=learned.FORM)
    t1 = time.perf_counter()
    d = learned.direct_light(g, E)
    guess = learned.warm_start(m, sc, d)
    t2 = time.perf_counter()
    B, st = g.gather(E, guess=guess, tol=tol, max_outer=100, sweeps=4)
    _, st0 = g.gather(E, tol=tol, max_outer=100, sweeps=4)

    def resid(Bt):  # Bt: N x 3, the shooter's own (reciprocity-form) system
        r = g.shoot_residual(E, np.ascontiguousarray(Bt.T, np.float32))
        return float(np.linalg.norm(r.astype(np.float64)) / np.linalg.norm(E64))

    # plain shooter, same raster configuration
    s = R.Solver(hemicube_side=W, hemicubes_count=args.k, mode=R.MODE_PHYS, tolerance=1e-9, tile=tune.tile,
                 small_tri_pixels=tune.small_tri_pixels)
    s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])
    s.shoot(2)
    s.set_state(radiosity=sc["radiosity"], illumination=sc["illumination"])
    dev_ms, batches, hemis, seg = 0.0, 0, 0, 16
    t_unshot = None
    res_p = 1.0
    while batches < 4000:
        stp = s.shoot(seg)
        dev_ms += stp.device_ms
        batches += stp.shots_done
        hemis += stp.hemicubes
        if t_unshot is None and stp.residual <= tol:
            t_unshot = (dev_ms / 1000, batches)
        rad, ill = s.download()
        Bp = (rad.astype(np.float64) + ill).reshape(n, 3)
        res_p = resid(Bp)
        if res_p <= tol or stp.stopped:
            break
    s.close()
    # FP64 host residuals of both answers on the FP32 rows, in row blocks
    v = sc["vertices"].reshape(n, 4, 3).astype(np.float64)
    area = 0.5 * np.linalg.norm(np.cross(v[:, 0] - v[:, 2], v[:, 1] - v[:, 3]), axis=1)
    Bg = B.T.astype(np.float64)
    FBp = np.zeros((n, 3))
    FTp = np.zeros((n, 3))
    FTg = np.zeros((n, 3))
    for r0 in range(0, n, 4096):
        F, _, _ = g.dense_rows(r0, min(4096, n - r0))
        Fd = F.astype(np.float64)
        r1 = r0 + len(F)
        FBp[r0:r1] = Fd @ Bp
        FTp += Fd.T @ (area[r0:r1, None] * Bp[r0:r1])
        FTg += Fd.T @ (area[r0:r1, None] * Bg[r0:r1])
    g.close()
    nE = np.linalg.norm(E64)
    res_p64 = float(np.linalg.norm(E64 + rho * FTp / area[:, None] - Bp) / nE)  # shooter
    res_p_gather = float(np.linalg.norm(E64 + rho * FBp - Bp) / nE)  # shooter answer, B = E + rho o (F B)
    res_g64 = float(np.linalg.norm(E64 + rho * FTg / area[:, None] - Bg) / nE)  # gather, same system
    rel_diff = float(np.linalg.norm(Bg - Bp) / np.linalg.norm(Bg))
    learned_s = (cap_ms + st.device_ms) / 1000 + (t2 - t1)
    ld = (n + 63) // 64 * 64
    sweep_gbs = 2.0 * n * ld * st.sweeps / (st.sweep_ms / 1000) / 1e9 if st.sweep_ms > 0 else 0.0
    hbm_peak, hbm_kind = measured_peaks()
    return {"patches": n, "W": W, "K": int(args.k), "tol": tol,
            "plain": {"device_s": dev_ms / 1000, "batches": batches, "hemicubes": hemis,
                      "residual": res_p, "fp64_residual": res_p64, "gather_system_residual": res_p_gather,
                      "unshot_rule_s": None if t_unshot is None else t_unshot[0],
                      "unshot_rule_batches": None if t_unshot is None else t_unshot[1]},
            "learned_gather": {"capture_s": cap_ms / 1000, "predict_host_s": t2 - t1,
                               "solve_s": st.device_ms / 1000, "outer": st.outer, "sweeps": st.sweeps,
                               "initial_residual": st.initial_residual, "residual": st.residual,
                               "fp64_residual": res_g64, "total_s": learned_s, "form": learned.FORM,
                               "sweep_ms": st.sweep_ms,
                               "sweep_roofline": {"kernel": "k_gemm_tc<16> (tcgen05 BF16 sweep, 3 RHS)",
                                                  "achieved_gbs": sweep_gbs, "peak_gbs": hbm_peak,
                                                  "peak_kind": hbm_kind, "frac": sweep_gbs / hbm_peak}},
            "gather_from_emission": {"solve_s": st0.device_ms / 1000, "outer": st0.outer, "sweeps": st0.sweeps,
                                     "initial_residual": st0.initial_residual},
            "answers_rel_l2_difference": rel_diff,
            "capture_us_per_row": cap_ms * 1000 / n, "shoot_us_per_hemicube": dev_ms * 1000 / max(1, hemis),
            "shooter_hemicubes_per_patch": hemis / n,
            "speedup_learned_gather_vs_plain": (dev_ms / 1000) / learned_s}


def warm_start_network(args):
    """The shipped network (radiosity_gb300/data) with its training record, else one trained here
    on 48 Cornell variants (2k-6k patches) with the training time reported."""
    from radiosity_gb300 import learned

    got = learned.load_network()
    if got is not None:
        m, meta = got
        if meta.get("training", {}).get("form") == learned.FORM:
            return m, dict(meta["training"], source="shipped network " + os.path.relpath(learned.WEIGHTS, ROOT))
        m.close()
    m, training = train_warm_start(args)
    return m, dict(training, source="trained in this run")


def _rel_residual(r, E):
    """max over channels of ||r_c|| / ||E_c|| (channels with E_c = 0 skipped); r, E: 3 x N."""
    nE = np.linalg.norm(E.astype(np.float64), axis=1)
    nr = np.linalg.norm(r.astype(np.float64), axis=1)
    return float(np.max(nr[nE > 0] / nE[nE > 0]))


def run_uneven(args):
    """Uneven batch: 256 Cornell-variant scenes, patches log-uniform in [500, 8000], 1-3 lights, W=128.

    Both arms run under one captured CUDA graph, and both stop each scene by the same rule: the
    relative residual max_c ||r_c|| / ||E_c|| of the shooter's discrete system
    B = E + rho o (F^T (A o B)) / A <= tol, on the scene's captured FP32 form-factor rows (the
    gather runs in the shoot form, so both arms solve that system).
      * Plain FP32 shooter (rad_multi): one replay advances every scene by one batch.  The graph
        is replayed in segments of 16 and each open scene's own-system residual (the reciprocity
        form of the shoot update) is checked after each segment, untimed; a scene's time is the
        device time to the end of the segment in which it met the rule.
      * Learned warm start + BF16 gather (rad_multi_gather): one graph launch captures every
        scene's form factors, computes its features and network guess, and runs its refinement
        loop on the device until its residual <= tol; a scene's time runs from the launch to its
        final check.
    The network's training is reported separately (the shipped network's record, or this run's)."""
    import radiosity_gb300 as R
    from radiosity_gb300 import learned, scenes

    rng = np.random.default_rng(args.seed)
    n_scenes, W, tol, seg = 256, 128, args.uneven_tol, 16
    scs = []
    for k in range(n_scenes):
        target = int(np.exp(rng.uniform(np.log(500), np.log(8000))))
        scs.append(scenes.cornell_variant(target, seed=int(rng.integers(1 << 30)), n_lights=int(rng.integers(1, 4))))
    sizes = [sc["n"] for sc in scs]
    Es = [learned.emission_block(sc) for sc in scs]
    ks = R.plan_shooters(sizes, hemicubes_per_patch=2.0 if tol >= 1e-2 else 4.5)

    def make(sc, K, **kw):
        s = R.Solver(hemicube_side=W, hemicubes_count=K, mode=R.MODE_PHYS, **kw)
        s.upload(sc["vertices"], sc["color"], sc["radiosity"], sc["illumination"], reflectance=sc["reflectance"])
        return s

    # the raster shape is tuned once, on the largest scene, and shared by every context
    big = int(np.argmax(sizes))
    probe = make(scs[big], ks[big])
    tune = probe.autotune()
    probe.close()
    shape = dict(tile=tune.tile, small_tri_pixels=tune.small_tri_pixels)
    # ---- plain shooter under one graph (device stop rule off: the residual rule stops it)
    solvers = [make(sc, K, tolerance=1e-12, **shape) for sc, K in zip(scs, ks)]
    for s in solvers:  # the FP32 rows for the residual rule (untimed)
        s.dense_capture(keep_fp32=True, form=learned.FORM)
    t_done = np.zeros(n_scenes)
    reps_done = np.zeros(n_scenes, np.int64)
    res_plain = np.ones(n_scenes)
    dev_ms, reps, t_check = 0.0, 0, 0.0
    open_ = set(range(n_scenes))
    with R.Multi(solvers) as mm:
        while open_ and reps < 4000:
            _, _, r, ms = mm.shoot(seg)
            dev_ms += ms
            reps += r
            c0 = time.perf_counter()
            for i in sorted(open_):
                rad, ill = solvers[i].download()
                B = np.ascontiguousarray((rad + ill).reshape(-1, 3).T)
                res_plain[i] = _rel_residual(solvers[i].shoot_residual(Es[i], B), Es[i])
                if res_plain[i] <= tol:
                    t_done[i], reps_done[i] = dev_ms, reps
                    open_.discard(i)
            t_check += time.perf_counter() - c0
    plain_done = np.array([i not in open_ for i in range(n_scenes)])
    for s in solvers:
        s.close()
    plain = {"scenes_per_s": float(plain_done.sum()) / (dev_ms / 1000), "device_s": dev_ms / 1000,
             "converged": int(plain_done.sum()), "replays": reps,
             "per_scene_ms": {"p50": float(np.percentile(t_done[plain_done], 50)),
                              "p99": float(np.percentile(t_done[plain_done], 99))},
             "hemicubes": int(sum(int(r) * k for r, k in zip(reps_done, ks))),
             "residual_max": float(res_plain[plain_done].max()), "check_wall_s_untimed": t_check,
             "K_per_scene": [int(min(ks)), int(max(ks))]}
    # ---- learned warm start + BF16 gather under one graph
    m, training = warm_start_network(args)
    ctxs = [make(sc, 16, **shape) for sc in scs]
    try:
        t0 = time.perf_counter()
        mg = R.MultiGather(ctxs, mlp=m, tol=tol, max_outer=100, sweeps=4, form=learned.FORM)
        build_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        out = mg.run()
        wall = time.perf_counter() - t0
        fp64 = []
        for i in range(4):  # FP64 residual of the shooter's system on the FP32 rows
            n = sizes[i]
            F, _, _ = ctxs[i].dense_rows(0, n)
            B = mg.result(i).T.astype(np.float64)
            E64 = Es[i].T.astype(np.float64)
            rho = scs[i]["reflectance"].reshape(n, 3).astype(np.float64)
            a = learned.patch_geometry(scs[i]["vertices"])[2][:, None]
            FT = F.astype(np.float64).T @ (a * B)
            fp64.append(_rel_residual((E64 + rho * FT / a - B).T, Es[i]))
        mg.close()
    finally:
        for c in ctxs:
            c.close()
        m.close()
    ok = out["status"] == 1
    gather = {"scenes_per_s": float(ok.sum()) / (out["device_ms"] / 1000), "device_s": out["device_ms"] / 1000,
              "wall_s": wall, "graph_build_s": build_s, "converged": int(ok.sum()),
              "per_scene_ms": {"p50": float(np.percentile(out["scene_ms"], 50)),
                               "p99": float(np.percentile(out["scene_ms"], 99))},
              "refinements_mean": float(np.mean(out["outer"]) - 1), "residual_max": float(out["residual"].max()),
              "initial_residual_mean": float(np.mean(out["initial_residual"])),
              "fp64_residual_max_checked": max(fp64), "fp64_checked_scenes": len(fp64),
              "hemicubes": int(sum(sizes)), "training": training}
    line = {"metric": f"scenes/s to own-system relative residual <= {tol:g} (256 uneven scenes, one CUDA graph each arm)",
            "value": gather["scenes_per_s"], "unit": "scenes/s", "workload": "uneven", "higher_is_better": True,
            "scenes": n_scenes, "patches": {"min": int(min(sizes)), "max": int(max(sizes)), "total": int(sum(sizes))},
            "learned_gather": gather, "plain_shooter": plain,
            "speedup_learned_gather_vs_plain": gather["scenes_per_s"] / plain["scenes_per_s"],
            "config": {"workload": f"{n_scenes} Cornell-variant scenes, 500-8000 patches (log-uniform), 1-3 lights, "
                                   f"W={W}, tol={tol:g}", "tile_from_autotune": tune.tile,
                       "small_tri_pixels_from_autotune": tune.small_tri_pixels},
            "data": "synthetic"}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "small":
        run_small(args)
    elif args.workload == "precision":
        run_precision(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.workload == "uneven":
        run_uneven(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
