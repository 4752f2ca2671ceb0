"""Benchmark of the annihilation sky-map projection on GB300.

Headline metric: particles/s at Nside 2048 for the
compensated-FP32 form, with the plain FP64-accumulate GPU form and the
per-pixel error against FP64 reported beside it.  Workload: the 16,777,216-
particle NFW host + 100 subhalos set (seeded synthetic stand-in for the
reference's simulation data), one observer at 8 kpc, HEALPix Nside 2048.

A step renders the whole particle set into one map.  ``value`` times steps
with inputs resident in HBM; ``e2e`` times the public API with pinned host
inputs and a host map (H2D of the particles and D2H of the 403 MB map inside
every step).  Inputs (403 MB) plus the map and the accumulation plane (805 MB)
exceed the 126 MB L2, so no explicit L2 flush is done between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "dm-annihilation-cxx_gb300", "pywrapper"))

import numpy as np  # noqa: E402

METRIC = "particles/s at Nside 2048: comp-FP32 vs plain GPU form; px err vs FP64"
UNIT = "particles/s"
WORKLOAD = "nfw16m_sub100_ns2048"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--scale", type=float, default=1.0, help="generate a halo with this fraction of "
                    "the particles (particles get fatter: same halo mass)")
    ap.add_argument("--subset", type=int, default=0, help="render only the first N particles of the "
                    "full (shuffled) workload: same per-particle disc statistics")
    ap.add_argument("--nside", type=int, default=0, help="render at this Nside instead of the "
                    "workload's (the overlap density, deposits per pixel, does not depend on it)")
    ap.add_argument("--plain-scale", type=float, default=1.0 / 64)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=60.0, help="reference arm: timed CPU seconds "
                    "over all steps")
    ap.add_argument("--no-extras", action="store_true", help="skip plain form, e2e and CPU legs")
    ap.add_argument("--no-tune", action="store_true", help="keep the default tuning (no autotuner)")
    return ap.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, v, device=None):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        busy = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """Per-deposit DRAM bytes of the deposit kernel from the committed ncu summary."""
    p = os.path.join(REPO, "profiles", "disc_seg_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def measure_l2_red(device, plane_floats):
    """Live L2 reduction rates (operations/s) of the library's own sweep
    microbenchmark: FP32 red (the compensated form's deposit) over an array
    the size of the FP32 deposit plane (the footprint the deposits land
    in), and for reference FP32 and FP64 red over 400 MB."""
    import ctypes as C
    from annmap import _lib
    L = _lib.load()
    out = {}
    plane = max(1 << 20, 4 * int(plane_floats))
    for name, kind, nbytes in (("red_f32", 0, plane), ("red_f32_400mb", 0, 400_000_000),
                               ("red_f64_400mb", 1, 400_000_000)):
        v = C.c_double()
        st = L.dmann_measure_l2_red(int(device), kind, int(nbytes), 20, C.byref(v))
        out[name] = v.value if st == 0 else None
    out["plane_bytes"] = plane
    return out


FP32_FLOPS_PER_WEIGHT = 12   # x (FMA), y = x^2, 4 Horner FMAs, the sum: 2 + 1 + 8 + 1


def roofline(device, deposits, pass1_ms, pass2_ms, npix):
    """The deposit pass's roofline on its binding resource, the L2 reduction
    units: each algorithmic deposit is one FP32 reduction (4 B) into the
    map's FP32 plane, against the library's live red.global.add.f32 sweep.
    Beside it the same bytes against measured HBM, and pass 1 (weight sums:
    FP32 arithmetic, no memory traffic to speak of) against the nominal FP32
    rate of the FMA pipes."""
    l2 = measure_l2_red(device, npix)
    hbm, hbm_src = measured_peaks()
    red_bytes = 4.0 * deposits
    s2, s1 = pass2_ms / 1e3, pass1_ms / 1e3
    achieved = red_bytes / s2 / 1e9
    peak = (l2["red_f32"] or 0.0) * 4.0 / 1e9
    traffic = profile_traffic()
    nominal_fp32 = 152 * 128 * 2 * 2.07e9 / 1e12
    p1_tflops = deposits * FP32_FLOPS_PER_WEIGHT / s1 / 1e12
    return {"bound": "l2_red", "kernel": "k_seg_dep (deposit segments)", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak if peak else None,
            "peak_source": (f"measured here: red.global.add.f32 sweep over the deposit plane's "
                            f"{l2['plane_bytes'] / 1e6:.0f} MB ({l2['red_f32']:.3e} reductions/s)")
            if l2["red_f32"] else "unavailable",
            "traffic": (traffic["dram_bytes_per_deposit"] * deposits) if traffic else None,
            "traffic_source": traffic.get("capture") if traffic else None,
            "algorithmic_bytes": red_bytes,
            "basis": "4 B FP32 reduction per algorithmic deposit / deposit-pass time (CUDA events)",
            "hbm": {"achieved": achieved, "peak": hbm, "frac": achieved / hbm,
                    "peak_source": hbm_src + " (MEASURED_PEAKS hbm_gbs)"},
            "sweeps_400mb": {"red_f32": l2["red_f32_400mb"], "red_f64": l2["red_f64_400mb"]},
            "pass1": {"kernel": "k_seg_norm (weight sums)", "ms": pass1_ms, "weights_per_s": deposits / s1,
                      "fp32_flops_per_weight": FP32_FLOPS_PER_WEIGHT, "achieved_tflops": p1_tflops,
                      "peak_tflops": nominal_fp32,
                      "peak_source": "nominal: 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz",
                      "frac": p1_tflops / nominal_fp32}}


def rel_err(got, ref):
    mask = ref > 1e-6 * ref.max()
    r = np.abs(got[mask] - ref[mask]) / ref[mask]
    return float(np.median(r)), float(r.max())


def cpu_oracle_run(P, nside, seconds, threads=None):
    """Times the FP64 oracle (CPU restatement of the reference map path) on a
    bounded prefix of the (shuffled, hence i.i.d.) particle set."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    threads = threads or os.cpu_count() or 1
    o = O.make_params(nside=nside, obs_pos=P.obs_pos, centerpos=P.centerpos, align_vec=P.align_vec,
                      particle_masses=(P.particle_mass,))
    # calibrate on a small prefix, then size the sample to ~`seconds`
    n0 = min(len(P), 64 * threads)
    t0 = time.perf_counter()
    O.render(o, P.subset(slice(0, n0)).as_dict(), nthreads=threads, finalize=False)
    dt0 = max(time.perf_counter() - t0, 1e-3)
    n = int(min(len(P), max(n0, n0 * seconds / dt0)))
    sub = P.subset(slice(0, n))
    t0 = time.perf_counter()
    mp, st, tot = O.render(o, sub.as_dict(), nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": threads, "seconds": dt, "particles": n,
            "deposits": st["deposits"], "deposits_per_s": st["deposits"] / dt}, sub, mp, tot


def bench_config(args, n, nside):
    """The workload description both arms print (identical in the two lines)."""
    return {"workload": args.workload + (f" (first {n} particles)" if args.subset else "")
            + (f" at Nside {nside}" if args.nside else ""),
            "particles": n, "nside": nside,
            "l2": f"no flush: inputs {24 * n / 1e6:.0f} MB + map/planes "
                  f"{16 * 12 * nside * nside / 1e6:.0f} MB > 126 MB L2"}


def run_reference(args, ws, rank):
    """The reference arm: the CPU restatement of the reference's own map path
    (src/genmap.cpp) on every host thread, on the same workload.  Each step
    renders a different slice of the shuffled (hence i.i.d.) particle set,
    sized so that the timed steps take about --ref-seconds (60 s) together; particles/s and
    deposits/s are totals over the timed slices, and ms_per_step is the time
    the whole set would take at that rate (an extrapolation)."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    from annmap import synth
    P, nside = synth.workload(args.workload, scale=args.scale)
    nside = args.nside or nside
    if args.subset:
        P = P.subset(slice(0, args.subset))
    n = len(P)
    threads = os.cpu_count() or 1
    o = O.make_params(nside=nside, obs_pos=P.obs_pos, centerpos=P.centerpos, align_vec=P.align_vec,
                      particle_masses=(P.particle_mass,))
    # a calibration slice, then slices of about `per_step` seconds (warm-up
    # steps a tenth of that)
    per_step = min(20.0, max(min(3.0, args.ref_seconds), args.ref_seconds / max(1, args.steps)))
    k0 = min(n, 64 * threads)
    t0 = time.perf_counter()
    O.render(o, P.subset(slice(0, k0)).as_dict(), nthreads=threads, finalize=False)
    rate0 = k0 / max(time.perf_counter() - t0, 1e-3)
    pos = k0
    parts = dep = secs = 0.0
    for i in range(args.warmup + args.steps):
        k = max(threads, int(rate0 * per_step * (0.1 if i < args.warmup else 1.0)))
        k = min(k, n)
        if pos + k > n:
            pos = 0
        sub = P.subset(slice(pos, pos + k))
        pos += k
        t0 = time.perf_counter()
        _, st, _ = O.render(o, sub.as_dict(), nthreads=threads, finalize=False)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            parts += k
            dep += st["deposits"]
            secs += dt
    v = parts / secs
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / v,
            "ms_per_step_basis": "extrapolated: whole-set particles / the timed slices' rate",
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded NFW host + subhalos)",
            "config": bench_config(args, n, nside),
            "form": "reference CPU map path (FP64), restated; all host threads",
            "deposits_per_s": dep / secs, "timed_seconds": secs,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{int(parts)} of {n} particles over {args.steps} timed steps, "
                                       f"a different slice of the shuffled (i.i.d.) set per step, "
                                       f"{secs:.1f} s on all {threads} host threads"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args, ws, rank, local):
    import torch
    import annmap
    from annmap import synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    P, nside = synth.workload(args.workload, scale=args.scale)
    nside = args.nside or nside
    if args.subset:
        P = P.subset(slice(0, args.subset))
    n = len(P)
    npix = 12 * nside * nside
    par = annmap.Parameters.for_synthetic(P, nside)
    host = P.as_dict()
    dparts = {k: torch.from_numpy(v).to(dev) for k, v in host.items()}
    dmap = torch.zeros(npix, dtype=torch.float64, device=dev)
    r = annmap.Renderer(local)
    r.set_params(par)
    stream = torch.cuda.current_stream(dev)
    r.set_stream(stream)

    # footprint bins and block shape for this Nside, measured on a sample
    from annmap import autotune
    if args.no_tune:
        tuned = {"best": r.get_tuning(), "seconds": 0.0, "cached": False}
    else:
        # on the whole set up to 16M particles: how many discs overlap while
        # rendered (the density, which a prefix sample lowers) decides the
        # block shape; beyond that a 16M prefix keeps tuning within a minute
        tuned = autotune.tune(r, dparts, nside, annmap.COMP_F32, sample=min(n, 1 << 24), reps=1,
                              out=dmap)

    disc_ms, step_ms, step_stats = [], [], None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the clock sampler starts before the warm-up so its start-up is not timed
    with ClockSampler(local) as clk:
        for _ in range(args.warmup):
            r.render(dparts, nside, annmap.COMP_F32, out=dmap)
        torch.cuda.synchronize()
        clk.lines.clear()
        barrier(ws)
        torch.cuda.synchronize()
        e0.record(stream)
        launches = 0
        p1_ms, p2_ms = [], []
        for _ in range(args.steps):
            r.render(dparts, nside, annmap.COMP_F32, out=dmap)
            step_stats = r.stats()
            disc_ms.append(step_stats["disc_ms"])
            step_ms.append(step_stats["kernel_ms"])
            p1_ms.append(step_stats["pass1_ms"])
            p2_ms.append(step_stats["pass2_ms"])
            launches += step_stats["launches"]
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
    ms = e0.elapsed_time(e1) / args.steps
    ms = allmax(ws, ms, dev)
    value = ws * n / (ms / 1e3)
    clocks = clk.summary()
    comp_map = dmap.cpu().numpy()

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded NFW host + 100 subhalos; reference data unavailable)",
            "config": bench_config(args, n, nside),
            "form": "compensated FP32 (FP64 geometry, FP32 weights, two-float sums)",
            "parallelism": f"replicas x{ws}",
            "tuning": dict(tuned["best"], autotune_s=round(tuned["seconds"], 2), cached=tuned["cached"]),
            "clocks": clocks, "gpu_launches": launches,
            "deposits_per_step": step_stats["deposits"],
            "deposits_per_s": step_stats["deposits"] / (ms / 1e3),
            # the map's total (sum x dOmega) against the kept particles' flux
            "flux_conservation_rel": abs(float(comp_map.sum()) * (4 * math.pi / npix) - step_stats["total_flux"])
                                     / step_stats["total_flux"],
            "stage_ms": {"step": ms, "disc_kernels": statistics.mean(disc_ms),
                         "disc_block": step_stats["disc_block_ms"], "disc_warp": step_stats["disc_warp_ms"],
                         "per_step": [round(x, 2) for x in step_ms]}}

    line["stage_ms"].update({"pass1": statistics.mean(p1_ms), "pass2": statistics.mean(p2_ms)})
    line["roofline"] = roofline(local, step_stats["deposits"], statistics.mean(p1_ms),
                                statistics.mean(p2_ms), npix)

    if not args.no_extras and rank == 0:
        # plain FP64 form on a prefix (the plain form is FP64-throughput bound)
        # (the shuffled set's prefix is an i.i.d. sample, so particles/s carries
        # over to the whole set; both forms are timed with CUDA events on it)
        k = max(1024, int(n * args.plain_scale))
        sub = {kk: v[:k] for kk, v in dparts.items()}
        pmap = torch.zeros_like(dmap)
        cmap = torch.zeros_like(dmap)

        def timed(prec, out, reps=3):
            r.render(sub, nside, prec, out=out)
            t = []
            for _ in range(reps):
                a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a0.record(stream)
                r.render(sub, nside, prec, out=out)
                a1.record(stream)
                torch.cuda.synchronize()
                t.append(a0.elapsed_time(a1))
            return statistics.median(t), r.stats()

        tp, pst = timed(annmap.PLAIN_F64, pmap)
        tc, cst = timed(annmap.COMP_F32, cmap)
        pm, cm = pmap.cpu().numpy(), cmap.cpu().numpy()
        med, mx = rel_err(cm, pm)
        plain_value = k / (tp / 1e3)
        line["plain_form"] = {"value": plain_value, "unit": UNIT, "particles": k,
                              "ms_per_step": tp, "deposits_per_s": pst["deposits"] / (tp / 1e3),
                              "timing": f"CUDA events, median of 3 renders of the first {k} particles "
                                        f"(1/{round(n / k)} of the set, i.i.d.)",
                              "comp_same_particles": {"value": k / (tc / 1e3), "ms_per_step": tc}}
        # the two forms on the same particles
        line["speedup_vs_plain"] = tp / tc
        line["px_err"] = {"vs": "GPU plain FP64 form, same particles", "particles": k,
                          "median": med, "max": mx, "floor": "pixels > 1e-6 max",
                          "total_flux_rel": abs(cm.sum() - pm.sum()) / pm.sum(),
                          "nonzero_sets_equal": bool(np.array_equal(cm != 0, pm != 0))}
        # e2e through the public API: pinned host inputs -> host map
        pin = {kk: torch.from_numpy(v).pin_memory() for kk, v in host.items()}
        hmap = torch.zeros(npix, dtype=torch.float64).pin_memory()
        hmap_np = hmap.numpy()
        r.set_stream(None)
        r.render({kk: v.numpy() for kk, v in pin.items()}, nside, annmap.COMP_F32, out=hmap_np)
        ke = max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        for _ in range(ke):
            r.render({kk: v.numpy() for kk, v in pin.items()}, nside, annmap.COMP_F32, out=hmap_np)
        te = (time.perf_counter() - t0) / ke
        line["e2e"] = {"value": n / te, "unit": UNIT, "h2d_bytes_per_step": 24 * n,
                       "d2h_bytes_per_step": 8 * npix, "ms_per_step": te * 1e3, "steps": ke}
        dev_vs_host = rel_err(hmap_np, comp_map)
        line["e2e"]["max_rel_diff_vs_device_run"] = dev_vs_host[1]
        # CPU baseline (rank 0, N = 1): the oracle on a bounded sample, and
        # the GPU map of the same sample against it
        if ws == 1:
            cpu, csub, omap, otot = cpu_oracle_run(P, nside, args.cpu_seconds)
            line["cpu_baseline"] = {"value": cpu["value"], "unit": UNIT, "cores": cpu["cores"],
                                    "kind": "port",
                                    "sample": f"{cpu['particles']} of {n} particles (shuffled prefix, "
                                              f"i.i.d.), {cpu['seconds']:.1f} s on {cpu['cores']} threads"}
            # the reference's own loop is single-threaded (genmap.cpp:67-156)
            cpu1, _, _, _ = cpu_oracle_run(P, nside, min(8.0, args.cpu_seconds), threads=1)
            line["cpu_baseline_1thread"] = {"value": cpu1["value"], "unit": UNIT, "cores": 1,
                                            "kind": "port", "sample": f"{cpu1['particles']} particles, "
                                            f"{cpu1['seconds']:.1f} s on 1 thread"}
            r.set_stream(None)
            g = r.render(csub.as_dict(), nside, annmap.COMP_F32)
            med2, mx2 = rel_err(g, omap)
            dom = 4 * math.pi / npix
            line["px_err_vs_oracle"] = {"particles": cpu["particles"], "median": med2, "max": mx2,
                                        "total_flux_rel": abs(g.sum() * dom - otot) / otot}
    r.close()
    if not args.no_extras and rank == 0:
        del dparts, dmap
        torch.cuda.empty_cache()
        line["small_map"] = bench_small(dev, args)
        line["batched"] = bench_batched(dev)
        line["adjoint"] = bench_adjoint(dev)
        line["large_map"] = bench_large(dev)
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_small(dev, args):
    """The plain method's own configuration: 1,048,576 NFW particles at Nside
    512, rendered whole by both GPU forms (CUDA events after a warm-up: one
    plain render, the median of three compensated ones; inputs resident),
    each against the FP64 oracle on a sample, and the oracle (the restated
    reference CPU path) timed on the host cores."""
    import torch
    import annmap
    from annmap import synth
    P, nside = synth.workload("nfw1m_ns512")
    n, npix = len(P), 12 * nside * nside
    r = annmap.Renderer(dev.index or 0)
    r.set_params(annmap.Parameters.for_synthetic(P, nside))
    dparts = {k: torch.from_numpy(v).to(dev) for k, v in P.as_dict().items()}
    out = torch.empty(npix, dtype=torch.float64, device=dev)
    res = {"workload": "nfw1m_ns512", "particles": n, "nside": nside}
    for name, prec, reps in (("plain_f64", annmap.PLAIN_F64, 1), ("comp_f32", annmap.COMP_F32, 3)):
        r.render(dparts, nside, prec, out=out)   # warm-up
        ms = []
        for _ in range(reps):
            r.render(dparts, nside, prec, out=out)
            torch.cuda.synchronize()
            ms.append(r.stats()["kernel_ms"])
        t = statistics.median(ms)
        st = r.stats()
        res[name] = {"ms": t, "particles_per_s": n / (t / 1e3), "deposits": st["deposits"],
                     "deposits_per_s": st["deposits"] / (t / 1e3)}
    cpu, csub, omap, otot = cpu_oracle_run(P, nside, min(10.0, args.cpu_seconds))
    res["cpu_baseline"] = {"value": cpu["value"], "unit": UNIT, "cores": cpu["cores"], "kind": "port",
                           "deposits_per_s": cpu["deposits_per_s"],
                           "sample": f"{cpu['particles']} particles, {cpu['seconds']:.1f} s"}
    dom = 4 * math.pi / npix
    for name, prec in (("plain_f64", annmap.PLAIN_F64), ("comp_f32", annmap.COMP_F32)):
        g = r.render(csub.as_dict(), nside, prec)
        med, mx = rel_err(g, omap)
        res[name]["px_err_vs_oracle"] = {"particles": cpu["particles"], "median": med, "max": mx,
                                         "total_flux_rel": abs(g.sum() * dom - otot) / otot}
    r.close()
    return res


def bench_batched(dev):
    """64 observers on the 8 kpc sphere, Nside cycling 256/512/1024, all maps
    of the 8,388,608-particle set rendered by one dmann_render_batch call
    (one CUDA graph, captured by the warm-up call and relaunched by the timed
    one; inputs and maps on the device), against the same 64 maps rendered
    one dmann_render call at a time."""
    import torch
    import annmap
    from annmap import synth
    P, _ = synth.workload("nfw8m_sub50_batched")
    obs = synth.batched_observers(64)
    par = annmap.Parameters.for_synthetic(P, 1024)
    dparts = {k: torch.from_numpy(v).to(dev) for k, v in P.as_dict().items()}
    frames, nsides = [], []
    for opos, ns in obs:
        par.set_observer(opos)
        frames.append((np.array(par.rot_flat()), opos))
        nsides.append(ns)
    outs = [torch.empty(12 * ns * ns, dtype=torch.float64, device=dev) for ns in nsides]
    r = annmap.Renderer(dev.index or 0)
    r.set_params(par)
    from annmap import autotune
    tuned = autotune.tune_nsides(r, dparts, nsides, annmap.COMP_F32, sample=1 << 20, reps=1)
    t0 = time.perf_counter()
    r.render_batch(dparts, frames, nsides, annmap.COMP_F32, outs=outs)   # warm-up: captures the graph
    torch.cuda.synchronize()
    t_capture = time.perf_counter() - t0
    t0 = time.perf_counter()
    r.render_batch(dparts, frames, nsides, annmap.COMP_F32, outs=outs)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    st = r.stats()
    # the same maps one render call each (same tuning, device inputs and maps)
    singles = []
    for (rot, opos), ns, out in zip(frames, nsides, outs):
        r.set_frame(rot, opos)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r.render(dparts, ns, annmap.COMP_F32, out=out)
        torch.cuda.synchronize()
        singles.append(time.perf_counter() - t1)
    r.close()
    return {"workload": "nfw8m_sub50_batched", "particles": len(P), "observers": len(obs),
            "nsides": sorted(set(nsides)), "form": "compensated FP32", "seconds": dt,
            "maps_per_s": len(obs) / dt, "particle_maps_per_s": len(P) * len(obs) / dt,
            "deposits": st["deposits"], "deposits_per_s": st["deposits"] / dt,
            "graph_ms": st["kernel_ms"], "launches": st["launches"],
            "first_call_seconds": t_capture,
            "sum_of_single_renders_seconds": sum(singles),
            "speedup_vs_single_renders": sum(singles) / dt,
            "launch": "one CUDA graph (dmann_render_batch, device maps), kept across calls",
            "tuning": {str(k): v["best"] for k, v in tuned.items()}}


def bench_large(dev):
    """The large-map configuration: 134,217,728 particles (NFW + 500 subhalos,
    10,000 of them within 0.5 kpc of the observer, whose discs reach whole
    hemispheres or the whole sky) at Nside 4096 (201,326,592 pixels): one
    warm-up and one timed render of the compensated form (CUDA events, inputs
    resident), flux conservation, and the per-pixel error against the oracle
    on a sample of the first 32,768 particles of the shuffled set plus 16 of
    the near-observer particles."""
    import torch
    import annmap
    from annmap import synth
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    t0 = time.perf_counter()
    P, nside = synth.workload("nfw134m_sub500_ns4096")
    gen_s = time.perf_counter() - t0
    n, npix = len(P), 12 * nside * nside
    dparts = {k: torch.from_numpy(v).to(dev) for k, v in P.as_dict().items()}
    out = torch.empty(npix, dtype=torch.float64, device=dev)
    r = annmap.Renderer(dev.index or 0)
    r.set_params(annmap.Parameters.for_synthetic(P, nside))
    stream = torch.cuda.current_stream(dev)
    r.set_stream(stream)
    r.render(dparts, nside, annmap.COMP_F32, out=out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    r.render(dparts, nside, annmap.COMP_F32, out=out)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    st = r.stats()
    total = float(out.sum()) * 4 * math.pi / npix
    del dparts, out
    torch.cuda.empty_cache()
    # the oracle on a sample that includes near-observer (large) discs
    pos = np.stack([P.x, P.y, P.z], 1).astype(np.float64) - np.array(P.obs_pos)
    near = np.flatnonzero(np.linalg.norm(pos, axis=1) < 0.5)
    pick = np.random.default_rng(5).choice(near, min(16, len(near)), replace=False)
    idx = np.random.default_rng(6).permutation(np.unique(np.concatenate([np.arange(1 << 15), pick])))
    sub = P.subset(idx)
    o = O.make_params(nside=nside, obs_pos=P.obs_pos, centerpos=P.centerpos, align_vec=P.align_vec,
                      particle_masses=(P.particle_mass,))
    t1 = time.perf_counter()
    ref, ost, otot = O.render(o, sub.as_dict(), nthreads=os.cpu_count() or 1)
    o_s = time.perf_counter() - t1
    r.set_stream(None)
    got = r.render(sub.as_dict(), nside, annmap.COMP_F32)
    r.close()
    med, mx = rel_err(got, ref)
    return {"workload": "nfw134m_sub500_ns4096", "particles": n, "nside": nside,
            "form": "compensated FP32", "ms": ms, "particles_per_s": n / (ms / 1e3),
            "deposits": st["deposits"], "deposits_per_s": st["deposits"] / (ms / 1e3),
            "pass1_ms": st["pass1_ms"], "pass2_ms": st["pass2_ms"],
            "flux_conservation_rel": abs(total - st["total_flux"]) / st["total_flux"],
            "generation_s": gen_s,
            "px_err_vs_oracle": {"particles": len(sub), "near_observer": int(len(pick)),
                                 "median": med, "max": mx,
                                 "total_flux_rel": abs(got.sum() * 4 * math.pi / npix - otot) / otot,
                                 "nonzero_sets_equal": bool(np.array_equal(got != 0, ref != 0)),
                                 "oracle_s": o_s}}


def bench_adjoint(dev):
    """dmann_adjoint on the 4,194,304-particle set at Nside 512 (device
    inputs, device gradient), after one warm-up call."""
    import torch
    import annmap
    from annmap import synth
    P, nside = synth.workload("nfw4m_sub20_adjoint")
    par = annmap.Parameters.for_synthetic(P, nside)
    dparts = {k: torch.from_numpy(v).to(dev) for k, v in P.as_dict().items()}
    G = torch.randn(12 * nside * nside, dtype=torch.float64, device=dev,
                    generator=torch.Generator(device=dev).manual_seed(7))
    out = torch.empty((6, len(P)), dtype=torch.float64, device=dev)
    r = annmap.Renderer(dev.index or 0)
    r.set_observer(P.obs_pos, P.centerpos, P.align_vec)
    r.set_units(par.unit_factor, par.hires_threshold)
    r.set_stream(torch.cuda.current_stream(dev))
    r.adjoint(dparts, nside, G, out=out)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r.adjoint(dparts, nside, G, out=out)
    dt = time.perf_counter() - t0
    st = r.stats()
    # the compensated-FP32 adjoint of the same loss, and its distance to the FP64 one
    out_c = torch.empty_like(out)
    r.adjoint(dparts, nside, G, out=out_c, precision=annmap.COMP_F32)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    r.adjoint(dparts, nside, G, out=out_c, precision=annmap.COMP_F32)
    dtc = time.perf_counter() - t1
    stc = r.stats()
    rel = [float(torch.linalg.vector_norm(out_c[k] - out[k]) / torch.linalg.vector_norm(out[k]))
           for k in range(6)]
    fwd = torch.empty(12 * nside * nside, dtype=torch.float64, device=dev)
    r.render(dparts, nside, annmap.PLAIN_F64, out=fwd)
    fst = r.stats()
    r.close()
    return {"workload": "nfw4m_sub20_adjoint", "particles": len(P), "nside": nside,
            "ms": dt * 1e3, "kernel_ms": st["kernel_ms"], "particles_per_s": len(P) / dt,
            "deposits": st["deposits"], "plain_forward_kernel_ms": fst["kernel_ms"],
            "form": "FP64 adjoint of the plain form (two passes per disc)",
            "comp_f32": {"ms": dtc * 1e3, "kernel_ms": stc["kernel_ms"], "particles_per_s": len(P) / dtc,
                         "normwise_rel_diff_vs_fp64": dict(zip(["x", "y", "z", "m", "rho", "h"], rel))}}


def main():
    args = parse()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gb300(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
