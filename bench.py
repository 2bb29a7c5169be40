#!/usr/bin/env python
"""Benchmark: gradient evaluations per second of the matchgate-brickwall fit at L=16.

Workload (seeded, synthetic): the spinful 1-D Fermi-Hubbard model on 8 sites x 2 spins
(interleaved, Jordan-Wigner, open chain), J=1, U=4, total time t=0.25, as a
second-order Trotter circuit of 64 steps built from matchgates (3336 gates); the fitted
circuit is a 5-layer periodic brickwall initialised at identity plus 1e-2 seeded noise.
One step = one gradient evaluation: f = -tr(U^dagger W) and the gate gradients, traced
over all 2^16 basis columns, target applied per column (nothing cached between steps).

The timed arm (default) runs the float-float ("mixed") engine; the FP64 engine is timed on
a column sample beside it and the mixed result's relative error against FP64 is reported.
--impl reference times the oracle port (the reference's CPU algorithm restated in C,
OpenMP over basis columns) on the host's cores on a bounded column sample.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "rqcopt_hpc-matchgate_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "grad evals/s at L=16 (mixed vs FP64 GPU, rel err<=1e-9); serving p50/p99 ms"
UNIT = "grad evals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--L", type=int, default=16)
    ap.add_argument("--layers", type=int, default=5)
    ap.add_argument("--trotter-steps", type=int, default=64)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp32"])
    ap.add_argument("--fp64-steps", type=int, default=1, help="timed FP64 evaluations over the full trace")
    ap.add_argument("--no-fp64", action="store_true", help="leave the FP64 comparison out")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--config", default="grad16", choices=["grad16", "grad18", "hess14", "batch64", "serve", "published", "hostmap"],
                    help="grad16: the headline (L=16 gradient, 5 layers); grad18: L=18 gradient, 7 layers, on a "
                         "column sample; hess14: L=14 full Hessian, 9 layers; batch64: 64 instances of uneven size "
                         "in one batched launch sequence; serve: a seeded Poisson request stream through the "
                         "request server; published: one trust-region iteration of the reference's published "
                         "benchmark (L=16, 5 layers, 601-layer target); hostmap: L=14 with the target as a host map")
    ap.add_argument("--published-hessian", default="both", choices=["plain", "ti", "both"])
    ap.add_argument("--published-precision", default="both", choices=["mixed", "fp64", "both"])
    ap.add_argument("--resident", action="store_true", help="--config published: make the target resident before the fit")
    ap.add_argument("--published-sweep", action="store_true",
                    help="--config published: sweep the target in every evaluation (MG_OPT_FIT_RESIDENT 1), as the "
                         "reference applies its target map each time")
    ap.add_argument("--serve-requests", type=int, default=60,
                    help="--config serve: the first this many requests of the seeded stream (a time-bounded prefix)")
    ap.add_argument("--serve-hess-max-L", type=int, default=12, help="largest L of Hessian and trust-region-step requests")
    ap.add_argument("--no-serve", action="store_true", help="leave the short serving stream out of the headline line")
    ap.add_argument("--serve-max-L", type=int, default=18)
    ap.add_argument("--sample-columns", type=int, default=4096, help="column sample of --config grad18")
    ap.add_argument("--profile-columns", type=int, default=0,
                    help="small case for ncu: one evaluation over this many columns, no timing, then exit")
    ap.add_argument("--hessian", default="per-gate", choices=["per-gate", "layer", "ti"],
                    help="--config hess14: per-gate blocks (504 parameters), per-layer blocks "
                         "(matchgate_brickwall_unitary_target_gradient_hessian, 72 parameters) or its "
                         "translation-invariant variant")
    ap.add_argument("--profile-hessian", type=int, default=0,
                    help="with --config hess14, for ncu: one mixed evaluation launched in chunks of this many "
                         "columns (each chunk one k_hessian launch), no FP64 arm, no timing, then exit")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """barrier / max over ranks on the host (gloo); no data-path collective: replicas"""

    def __init__(self, world):
        self.world = world
        if world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())


def workload(L, nlayers, nsteps, seed=3):
    import targets as T
    import numpy as np
    g, w, _ = T.hubbard_trotter_circuit(L // 2, 1.0, 4.0, 0.25, nsteps)
    rng = np.random.default_rng(seed)
    v = T.near_identity_brickwall(nlayers, rng)
    perms = T.brickwall_perms(L, nlayers)
    return g, w, v, perms


def headline_config(L, nl, gu, trotter_steps):
    """the workload description both arms print (identical dicts, so the two lines compare)"""
    return {"workload": f"L={L} spinful Hubbard Trotter target ({gu} gates, {trotter_steps} second-order steps), "
                        f"{nl}-layer brickwall fit ({nl * (L // 2)} gates), f + Riemannian gradient over all 2^{L} "
                        f"basis columns",
            "L": L, "nlayers": nl, "target_gates": gu, "trotter_steps": trotter_steps,
            "l2": "per-step working set larger than L2; the GPU arm also writes a 512 MiB buffer between timed steps"}


# DRAM bytes (read + write) of the target-sweep kernel per basis column: ncu
# dram__bytes_read.sum + dram__bytes_write.sum of one k_target_w<PrecX> launch over 912 columns
# of this workload (L=16, float-float, two columns per resident block).  The kernel's traffic
# is its output columns plus the tile round trips that miss L2, both proportional to the
# columns, so per-launch traffic = this x columns per launch.
TARGET_DRAM_BYTES_PER_COLUMN = {16: (23.944726e9 + 20.012690e9) / 912}


def hbm_view(traffic, launch_s):
    """the dominant kernel against the measured HBM copy bandwidth (MEASURED_PEAKS.json,
    else the 6800 GB/s fallback): DRAM bytes per launch over the launch time"""
    if not traffic:
        return None
    peak, src = 6800.0, "fallback"
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peak, src = float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        pass
    gbs = traffic / launch_s / 1e9
    return {"achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak, "peak_source": src}


def alg_flops(L, gu, gw, ncols):
    """algorithmic real flops of target+gradient over ncols columns, counted on the parity
    sector S = 2^(L-1): 14 per amplitude and forward gate, 44 per amplitude and fitted gate
    (forward 14 + backward 30), 8 per amplitude for the overlap"""
    return float(ncols) * (1 << (L - 1)) * (14 * gu + 44 * gw + 8)


class Clocks:
    """nvidia-smi samples during the timed region"""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1])); smax = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(g, w, v, perms, L, budget_s, nthreads=0):
    """the oracle port (reference algorithm, full vectors, OpenMP over basis columns) on a
    bounded column sample; returns (evals/s, threads, columns, seconds, f, grad_vec) with f
    and the Riemannian gradient traced over the sample's columns"""
    import oracle
    nthreads = nthreads or os.cpu_count()
    t = oracle.Target("circuit", L, gates=g, wires=w)
    ncols = nthreads
    t0 = time.perf_counter()
    oracle.brickwall_projected_gradient(t, v, perms, L, nthreads=nthreads, col_range=(0, ncols))
    dt = time.perf_counter() - t0
    reps = max(1, min(64, int(budget_s / max(dt, 1e-3))))
    ncols = min(1 << L, nthreads * reps)
    t0 = time.perf_counter()
    f, gv = oracle.brickwall_projected_gradient(t, v, perms, L, nthreads=nthreads, col_range=(0, ncols))
    dt = time.perf_counter() - t0
    return (ncols / float(1 << L)) / dt, nthreads, ncols, dt, f, gv


def cpu_baseline_line(g, w, v, perms, L, budget_s, ncols, gpu_columns=None):
    """the bench line's cpu_baseline: the port on all host cores (OpenMP over basis columns,
    as the reference's parallel drivers split the trace), and beside it on one core (the
    reference's gradient path is serial as shipped, src/matchgate_target.c:212-302).  The
    all-core sample's f and gradient double as the oracle check of the GPU result:
    gpu_columns(b0, b1) -> (f, grad_vec) of the timed precision over the same columns."""
    import numpy as np
    cv, cores, cc, cs, f_o, g_o = cpu_baseline(g, w, v, perms, L, budget_s)
    c1, _, n1, s1, _, _ = cpu_baseline(g, w, v, perms, L, budget_s / 4, nthreads=1)
    out = {"value": cv, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{cc} of {ncols} basis columns in {cs:.1f} s, scaled to one full evaluation",
           "single_core": {"value": c1, "unit": UNIT, "cores": 1,
                           "sample": f"{n1} of {ncols} basis columns in {s1:.1f} s, scaled to one full evaluation"}}
    if gpu_columns is not None:
        f_x, g_x = gpu_columns(0, cc)
        out["oracle_check"] = {"columns": [0, cc],
                               "rel_err_f_vs_oracle": float(abs(f_x - f_o) / abs(f_o)),
                               "rel_err_grad_vs_oracle": float(np.linalg.norm(g_x - g_o) / np.linalg.norm(g_o))}
    return out


def run_reference(a):
    """the reference arm: the oracle port (the reference's algorithm restated in C; the
    reference's own sources are not on the GPU machine) on all host cores, OpenMP over basis
    columns.  Each step traces a fixed column sample (a few seconds of host work);
    ms_per_step is that step's wall time, value the evaluations/s it extrapolates to."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    g, w, v, perms = workload(a.L, a.layers, a.trotter_steps)
    import oracle
    nthreads = os.cpu_count()
    t = oracle.Target("circuit", a.L, gates=g, wires=w)
    # size the per-step column sample to a few seconds of host work
    t0 = time.perf_counter()
    oracle.brickwall_projected_gradient(t, v, perms, a.L, nthreads=nthreads, col_range=(0, nthreads))
    d1 = time.perf_counter() - t0
    ncols = min(1 << a.L, nthreads * max(1, min(64, int(2.5 / max(d1, 1e-3)))))
    for _ in range(max(0, a.warmup - 1)):
        oracle.brickwall_projected_gradient(t, v, perms, a.L, nthreads=nthreads, col_range=(0, nthreads))
    times = []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        oracle.brickwall_projected_gradient(t, v, perms, a.L, nthreads=nthreads, col_range=(0, ncols))
        times.append(time.perf_counter() - t0)
    step_s = statistics.mean(times)
    value = (ncols / float(1 << a.L)) / step_s
    sample = f"{ncols} of {1 << a.L} basis columns per step ({step_s:.2f} s wall), scaled to one full gradient evaluation"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": step_s * 1e3, "columns_per_step": ncols,
        "value_is": "evaluations/s extrapolated from the per-step column sample (the per-column cost is uniform)",
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded Hubbard Trotter target, seeded near-identity fit)",
        "config": headline_config(a.L, a.layers, len(g), a.trotter_steps),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_gb300(a):
    import numpy as np
    rank, world, local = dist_env()
    os.environ["MG_DEVICE"] = str(local)
    dist = Dist(world)
    import mgcu
    lib = mgcu.default_lib()
    prec = {"mixed": mgcu.PREC_MIXED, "fp64": mgcu.PREC_FP64, "fp32": mgcu.PREC_FP32}[a.precision]
    L, nl = a.L, a.layers
    g, w, v, perms = workload(L, nl, a.trotter_steps)
    gu, gw = len(g), nl * (L // 2)
    ncols = 1 << L
    fp32_peak = lib.lib.mg_measure_fp32_peak_gflops()
    fp64_peak = lib.lib.mg_measure_fp64_peak_gflops()

    target = lib.target_circuit(g, w, L)
    lib.set_precision(prec)
    if a.profile_columns:
        lib.brickwall_columns(lib.mg_target_apply, target, v, perms, L, 0, min(304, a.profile_columns))
        rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, target, v, perms, L, 0, a.profile_columns)
        assert rc == 0, lib.last_error()
        lib.target_free(target)
        if rank == 0:
            print(json.dumps({"profile_columns": a.profile_columns, "L": L, "precision": a.precision, "f": [f.real, f.imag]}))
        return
    plan = lib.plan_brickwall(lib.mg_target_apply, target, v, perms, L, mgcu.EVAL_GRADIENT)
    for _ in range(a.warmup):
        assert lib.lib.mg_plan_run(mgcu.P(plan)) == 0, lib.last_error()
    dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    n0 = lib.launch_count()
    total_ms = lib.lib.mg_plan_time_ms(mgcu.P(plan), a.steps, 1)
    launches = lib.launch_count() - n0
    clk = clocks.stop()
    tk_ms, tk_n = lib.plan_target_kernel_ms(plan)
    dist.barrier()
    assert total_ms > 0, lib.last_error()
    f_dev, dv_dev, _, gvec_dev, _ = lib.plan_results(plan, nl, grad=True, proj=True)
    total_s = dist.max(total_ms / 1e3)
    value = world * a.steps / total_s
    ms_per_step = total_s * 1e3 / a.steps

    # end to end through the reference-facing C call, host buffers in and out
    for _ in range(1):
        lib.brickwall_projected_gradient(lib.mg_target_apply, target, v, perms, L)
    dist.barrier()
    e2e_t = []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        rc, f_e2e, g_e2e = lib.brickwall_projected_gradient(lib.mg_target_apply, target, v, perms, L)
        e2e_t.append(time.perf_counter() - t0)
        assert rc == 0, lib.last_error()
    e2e_s = dist.max(sum(e2e_t))
    tsize = 16 if prec != mgcu.PREC_FP32 else 8
    h2d = gu * 0 + (nl * (L // 2)) * 8 * tsize + nl * 128      # gate matrices + gates for the projection
    d2h = 16 + nl * 8 * 8                                      # f + projected gradient

    # FP64 over the full trace, timed by the same CUDA-event timer as the headline: the
    # speed-up of the timed precision, and its error over all 2^L columns
    fp64 = None
    if a.precision != "fp64" and not a.no_fp64:
        lib.set_precision(mgcu.PREC_FP64)
        plan64 = lib.plan_brickwall(lib.mg_target_apply, target, v, perms, L, mgcu.EVAL_GRADIENT)
        lib.set_precision(prec)
        assert lib.lib.mg_plan_run(mgcu.P(plan64)) == 0, lib.last_error()
        ms64 = lib.lib.mg_plan_time_ms(mgcu.P(plan64), a.fp64_steps, 1)
        assert ms64 > 0, lib.last_error()
        f64, dv64, _, g64, _ = lib.plan_results(plan64, nl, grad=True, proj=True)
        lib.lib.mg_plan_free(mgcu.P(plan64))
        s64 = ms64 / 1e3 / a.fp64_steps
        fp64 = {"value": 1.0 / s64, "unit": UNIT, "ms_per_step": s64 * 1e3, "steps": a.fp64_steps, "columns": ncols,
                "extrapolated_from_sample": False, "timer": "CUDA events on the library stream (mg_plan_time_ms), as the headline",
                "speedup_of_timed_precision": s64 / (ms_per_step / 1e3)}
        accuracy = {"columns": ncols,
                    "rel_err_f_vs_fp64": float(abs(f_dev - f64) / abs(f64)),
                    "rel_err_grad_vs_fp64": float(np.linalg.norm(gvec_dev - g64) / np.linalg.norm(g64)),
                    "rel_err_layer_gradients_vs_fp64": float(np.linalg.norm(dv_dev - dv64) / np.linalg.norm(dv64)),
                    "f": [float(np.real(f_dev)), float(np.imag(f_dev))], "f_fp64": [float(np.real(f64)), float(np.imag(f64))]}
    else:
        accuracy = {"columns": ncols, "f": [float(np.real(f_dev)), float(np.imag(f_dev))]}

    def gpu_columns(b0, b1):
        """f and Riemannian gradient of the timed precision over columns [b0, b1)"""
        lib.set_precision(prec)
        rc, fx, dvx = lib.brickwall_columns(lib.mg_target_apply, target, v, perms, L, b0, b1)
        assert rc == 0, lib.last_error()
        return fx, lib.project_gradient(v, dvx)

    # optimiser steady state: the target's columns kept resident on the GPU after one sweep
    # (reported beside the headline, which sweeps the target in every evaluation)
    resident = None
    if world == 1:
        lib.set_precision(prec)
        lib.target_set_resident(target, True)
        plan_r = lib.plan_brickwall(lib.mg_target_apply, target, v, perms, L, mgcu.EVAL_GRADIENT)
        t0 = time.perf_counter()
        assert lib.lib.mg_plan_run(mgcu.P(plan_r)) == 0, lib.last_error()   # fills the resident columns
        lib.plan_results(plan_r, nl, grad=True)                              # (waits for the GPU)
        fill_s = time.perf_counter() - t0
        ms_r = lib.lib.mg_plan_time_ms(mgcu.P(plan_r), a.steps, 1)
        f_r, _, _, gvec_r, _ = lib.plan_results(plan_r, nl, grad=True, proj=True)
        lib.lib.mg_plan_free(mgcu.P(plan_r))
        lib.target_set_resident(target, False)
        resident = {"value": a.steps / (ms_r / 1e3), "unit": UNIT, "first_evaluation_s": fill_s,
                    "device_bytes": (1 << L) * (1 << (L - 1)) * (16 if prec != mgcu.PREC_FP32 else 8),
                    "same_result": bool(abs(f_r - f_dev) <= 1e-12 * abs(f_dev)),
                    "note": "the target's -conj(U e_b) columns stay on the GPU after the first evaluation "
                            "(mg_target_set_resident); later evaluations with new fitted gates run only the "
                            "fitted circuit; not the headline, which sweeps the target every evaluation"}

    # the metric's serving part: a short version of the seeded request stream (the full one:
    # --config serve); skipped with --no-serve
    serving = None
    if world == 1 and not a.no_serve:
        serving = serve_stream(lib, 100, 14)
        serving["note"] = "100 requests, L up to 14; the 200-request stream with L up to 16 is --config serve"
        lib.set_precision(prec)

    flops = alg_flops(L, gu, gw, ncols)
    achieved_step = flops / (ms_per_step / 1e3) / 1e12
    # dominant kernel: the target sweep (k_target), timed by CUDA events around each launch
    cols_per_launch = ncols * a.steps / tk_n
    gu_run = lib.lib.mg_target_sweep_gates(mgcu.P(target))   # gates the sweep applies (fermionic swaps relabelled away)
    # amplitude-columns the sweep visits per launch: the whole parity sector of every column,
    # or (Hamming-weight-conserving target) the amplitudes of the column's weight only:
    # sum_b C(L, |b|) = C(2L, L) over all 2^L columns
    weight = bool(lib.lib.mg_target_conserves_weight(mgcu.P(target)))
    sector_units = float(cols_per_launch) * (1 << (L - 1))
    live_units = float(math.comb(2 * L, L)) * cols_per_launch / ncols if weight else sector_units
    tk_avg_s = tk_ms / 1e3 / tk_n
    achieved = live_units * 14 * gu_run / tk_avg_s / 1e12
    bpc = TARGET_DRAM_BYTES_PER_COLUMN.get(L) if a.precision == "mixed" else None
    traffic = bpc * cols_per_launch if bpc else None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"mixed": "f32 float-float pairs (about 48-bit significands), f64 final sums",
                  "fp64": "f64", "fp32": "f32, compensated f32 sums"}[a.precision],
        "data": "synthetic (seeded Hubbard Trotter target, seeded near-identity fit)",
        "config": headline_config(L, nl, gu, a.trotter_steps),
        "precision": a.precision, "parallelism": f"replicas x{world}", "columns_per_step": ncols,
        "gpu_launches": launches,
        "clocks": clk,
        "e2e": {"value": world * a.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "timer": "host clock around matchgate_brickwall_unitary_target_and_projected_gradient (synchronous C call)"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak / 1e3, "unit": "TFLOP/s",
                     "frac": achieved / (fp32_peak / 1e3), "traffic": traffic,
                     "kernel": "k_target (target sweep)", "kernel_launches": tk_n,
                     "kernel_config": lib.plan_target_config(plan),
                     "kernel_ms_per_launch": tk_avg_s * 1e3, "kernel_share_of_step": tk_ms / total_ms,
                     "columns_per_launch": cols_per_launch,
                     "achieved_is": "algorithmic complex-arithmetic flops of the target sweep (14 per visited "
                                    "amplitude and applied gate) per second of k_target; the target conserves the "
                                    "Hamming weight, so the sweep visits C(2L, L) amplitude-columns per trace, the "
                                    "nonzero ones, not the 2^(2L-1) of the parity sectors" if weight else
                                    "algorithmic complex-arithmetic flops of the target sweep (14 per parity-sector "
                                    "amplitude and applied gate) per second of k_target",
                     "visited_amplitudes_per_launch": live_units,
                     "parity_sector_equivalent_tflops": sector_units * 14 * gu_run / tk_avg_s / 1e12,
                     "target_gates_applied": gu_run,
                     "step_achieved": achieved_step,
                     "peak_source": "FP32 FMA microkernel of this library, measured in this run "
                                    "(MEASURED_PEAKS.json holds HBM and bf16 tensor peaks only)",
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_target_w launch over "
                                       "912 columns of this workload, per column, x columns per launch",
                     "fp64_peak_tflops": fp64_peak / 1e3,
                     "hbm": hbm_view(traffic, tk_avg_s)},
        "fp64_gpu": fp64,
        "accuracy": accuracy,
        "serving": serving,
        "resident_target": resident,
    }
    if rank == 0 and world == 1 and not a.no_cpu:
        out["cpu_baseline"] = cpu_baseline_line(g, w, v, perms, L, a.cpu_seconds, ncols, gpu_columns)
    lib.lib.mg_plan_free(mgcu.P(plan))
    lib.target_free(target)
    if rank == 0:
        print(json.dumps(out))


def run_secondary(a):
    """the other Hubbard configurations: L=18 gradient with 7 layers (column sample,
    extrapolated) and L=14 gradient + full Hessian with 9 layers (504 real parameters),
    mixed precision against FP64 on the GPU"""
    import numpy as np
    import mgcu
    lib = mgcu.default_lib()
    L, nl = (18, 7) if a.config == "grad18" else (14, 9)
    g, w, v, perms = workload(L, nl, a.trotter_steps)
    target = lib.target_circuit(g, w, L)
    ncols = 1 << L
    if a.config == "hess14" and a.profile_hessian:
        lib.set_precision(mgcu.PREC_MIXED)
        lib.set_option(mgcu.OPT_CHUNK_COLUMNS, a.profile_hessian)
        if a.hessian == "layer":   # the per-layer Hessian: grouped items, one per layer and entry
            rc, f, dg, H = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, target, v, perms, L)
        else:
            cg = np.array([v[l] for l in range(nl) for _ in range(L // 2)])
            cw = np.array([[perms[l][2 * i], perms[l][2 * i + 1]] for l in range(nl) for i in range(L // 2)], np.int32)
            rc, f, dg, H = lib.circuit_target_gradient_hessian(lib.mg_target_apply, target, cg, cw, L)
        assert rc == 0, lib.last_error()
        lib.set_option(mgcu.OPT_CHUNK_COLUMNS, 0)
        lib.target_free(target)
        print(json.dumps({"profile_hessian": a.profile_hessian, "hessian": a.hessian, "L": L, "f": [f.real, f.imag]}))
        return
    res = {}
    for name, prec in (("mixed", mgcu.PREC_MIXED), ("fp64", mgcu.PREC_FP64)):
        lib.set_precision(prec)
        if a.config == "grad18":
            c = min(a.sample_columns, ncols)
            lib.brickwall_columns(lib.mg_target_apply, target, v, perms, L, 0, min(304, c))
            t0 = time.perf_counter()
            rc, f, dv = lib.brickwall_columns(lib.mg_target_apply, target, v, perms, L, 0, c)
            dt = time.perf_counter() - t0
            assert rc == 0, lib.last_error()
            res[name] = {"evals_per_s": (c / ncols) / dt, "s_per_eval": dt * ncols / c, "f": f, "g": dv.reshape(-1)}
        elif a.hessian != "per-gate":
            # one block per layer (the reference's brickwall Hessian, 8 * nl real parameters),
            # or its translation-invariant variant (one placement per layer, weighted)
            ti = a.hessian == "ti"
            lib.brickwall_target_gradient_hessian(lib.mg_target_apply, target, v[:1], perms[:1], L, ti=ti)   # warm-up
            t0 = time.perf_counter()
            rc, f, dv, H = lib.brickwall_target_gradient_hessian(lib.mg_target_apply, target, v, perms, L, ti=ti)
            dt = time.perf_counter() - t0
            assert rc == 0, lib.last_error()
            res[name] = {"evals_per_s": 1 / dt, "s_per_eval": dt, "f": f, "g": dv.reshape(-1), "H": np.asarray(H)}
        else:
            # every gate of the brickwall its own parameter block: 8 * nl * L/2 real parameters
            cg = np.array([v[l] for l in range(nl) for _ in range(L // 2)])
            cw = np.array([[perms[l][2 * i], perms[l][2 * i + 1]] for l in range(nl) for i in range(L // 2)], np.int32)
            lib.circuit_target_gradient_hessian(lib.mg_target_apply, target, cg[:1], cw[:1], L)   # warm-up
            t0 = time.perf_counter()
            rc, f, dg, H = lib.circuit_target_gradient_hessian(lib.mg_target_apply, target, cg, cw, L)
            dt = time.perf_counter() - t0
            assert rc == 0, lib.last_error()
            res[name] = {"evals_per_s": 1 / dt, "s_per_eval": dt, "f": f, "g": dg.reshape(-1), "H": np.asarray(H)}
    lib.target_free(target)
    mx, fp = res["mixed"], res["fp64"]
    rel = lambda x, y: float(np.linalg.norm(np.asarray(x) - np.asarray(y)) / np.linalg.norm(np.asarray(y)))
    acc = {"rel_err_f_vs_fp64": abs(mx["f"] - fp["f"]) / abs(fp["f"]), "rel_err_grad_vs_fp64": rel(mx["g"], fp["g"])}
    if "H" in mx:
        acc["rel_err_hessian_vs_fp64"] = rel(mx["H"], fp["H"])
    what = "gradient" if a.config == "grad18" else {"per-gate": "gradient + per-gate Hessian",
                                                     "layer": "gradient + per-layer Hessian",
                                                     "ti": "gradient + translation-invariant per-layer Hessian"}[a.hessian]
    out = {"metric": f"{what} evals/s at L={L} (mixed vs FP64 GPU)", "value": mx["evals_per_s"], "unit": "evals/s",
           "n_gpus": 1, "higher_is_better": True, "dtype": "f32 float-float pairs, f64 final sums",
           "data": "synthetic (seeded Hubbard Trotter target, seeded near-identity fit)",
           "config": {"workload": f"L={L} spinful Hubbard Trotter target ({len(g)} gates), {nl}-layer brickwall fit "
                                  f"({nl * (L // 2)} gates), {what} over all 2^{L} columns",
                      "real_parameters": 8 * nl * (L // 2) if a.config == "hess14" and a.hessian == "per-gate" else 8 * nl,
                      "L": L, "nlayers": nl, "target_gates": len(g)},
           "s_per_eval": {"mixed": mx["s_per_eval"], "fp64": fp["s_per_eval"]},
           "speedup_mixed_vs_fp64": fp["s_per_eval"] / mx["s_per_eval"], "accuracy": acc,
           "extrapolated_from_sample": a.config == "grad18",
           "sample_columns": min(a.sample_columns, ncols) if a.config == "grad18" else ncols}
    print(json.dumps(out))


# the reference's published wall times of one trust-region iteration at L=16, 5 fitted layers,
# 601-layer target, 112 OpenMP threads of one CoolMUC-4 node
# (benchmark_hpc/bench_out/q16/plots/n5_q16_u601_invariance_scaling.txt:10-11)
PUBLISHED_S = {"plain": 4134.93143864, "ti": 1438.426814181}


def published_workload(L=16):
    """the reference's benchmark inputs (benchmark_hpc/spl_hubbard1d_bench_init.py:24-118, with
    the step counts its published runs used): spinless Hubbard J=1, g=1.5, t=1; target = 12
    steps of the 6th-order Suzuki rule (601 layers); fit = 2 steps of the 2nd-order rule (5
    layers), each layer one matchgate on all L/2 pairs of its periodic brickwall wiring"""
    import targets as T
    ul, up = T.spinless_hubbard_brickwall(L, 1.0, 1.5, 1.0, 12, 6)
    v, perms = T.spinless_hubbard_brickwall(L, 1.0, 1.5, 1.0, 2, 2)
    return ul, up, v, perms


def run_published(a):
    """config published: one trust-region iteration of the reference's published benchmark
    (benchmark_hpc/benchmark_threads.c:121-135: optimize_matchgate_brickwall_circuit_hmat with
    niter = 1 and set_rtr_default_params(16 nlayers), i.e. f + Riemannian gradient + Hessian,
    tCG, retraction, f at the trial point, f at the final point; src/trust_region.c:235-306),
    on this library's native trust-region driver, plain and translation-invariant Hessian, in
    float-float and in complex128; wall time of the synchronous call.  By default the native
    fit keeps the target's columns on the GPU after the first evaluation (the target is fixed
    within a fit; MG_OPT_FIT_RESIDENT 0), which the reference does not do; --published-sweep
    sweeps the target in every evaluation as the reference does."""
    import numpy as np
    import mgcu
    lib = mgcu.default_lib()
    L = 16
    lib.set_option(mgcu.OPT_FIT_RESIDENT, 1 if a.published_sweep else 0)
    ul, up, v, perms = published_workload(L)
    target = lib.target_brickwall(ul, up, L)
    rows = {}
    hess = [h for h in ("plain", "ti") if a.published_hessian in (h, "both")]
    precs = [p for p in ("mixed", "fp64") if a.published_precision in (p, "both")]
    for h in hess:
        lib.set_option(mgcu.OPT_TRANSLATIONAL_INVARIANCE, 1 if h == "ti" else 0)
        for pname in precs:
            refine = 1e-300 if pname == "mixed" else 0.0   # float-float throughout, or complex128
            lib.target_set_resident(target, bool(a.resident))
            t0 = time.perf_counter()
            f_iter, prec_iter, vout = lib.optimize_native(target, v, perms, L, 1, refine_gnorm=refine)
            dt = time.perf_counter() - t0
            lib.target_set_resident(target, False)
            rows[f"{h}_{pname}"] = {"s_per_tr_iteration": dt, "published_s": PUBLISHED_S[h],
                                    "speedup_vs_published": PUBLISHED_S[h] / dt,
                                    "f_iter": [float(x) for x in f_iter], "gates_out": vout}
    lib.set_option(mgcu.OPT_TRANSLATIONAL_INVARIANCE, 0)
    lib.set_option(mgcu.OPT_FIT_RESIDENT, 0)
    lib.target_free(target)
    acc = {}
    for h in hess:
        if f"{h}_mixed" in rows and f"{h}_fp64" in rows:
            m, d = rows[f"{h}_mixed"], rows[f"{h}_fp64"]
            acc[h] = {"rel_err_f_iter_vs_fp64": [abs(x - y) / abs(y) for x, y in zip(m["f_iter"], d["f_iter"])],
                      "max_abs_gate_diff_vs_fp64": float(np.max(np.abs(m["gates_out"] - d["gates_out"])))}
    for r in rows.values():
        del r["gates_out"]
    head = rows.get("plain_mixed") or next(iter(rows.values()))
    print(json.dumps({
        "metric": "wall time of one trust-region iteration, L=16, 5 layers, 601-layer target (the reference's published benchmark)",
        "value": head["s_per_tr_iteration"], "unit": "s", "higher_is_better": False, "n_gpus": 1,
        "vs_baseline": head["s_per_tr_iteration"] / PUBLISHED_S["plain" if "plain_mixed" in rows else next(iter(rows)).split("_")[0]],
        "dtype": "f32 float-float pairs (f64 sums, projection, tCG) / f64",
        "data": "the reference's benchmark inputs rebuilt analytically (spinless Hubbard J=1, g=1.5, t=1; Suzuki order 6 x 12 "
                "steps target, order 2 x 2 steps fit)",
        "config": {"workload": "optimize_matchgate_brickwall_circuit_hmat, niter=1: f + Riemannian gradient + Hessian, tCG "
                               "(maxiter 160), retraction, 2 f", "L": L, "nlayers": len(v), "target_layers": len(ul),
                   "target_gates": len(ul) * (L // 2),
                   "target_columns": ("swept in every evaluation (MG_OPT_FIT_RESIDENT 1)" if a.published_sweep else
                                      "kept on the GPU after the first evaluation of the fit (MG_OPT_FIT_RESIDENT 0)"),
                   "resident_target": bool(a.resident)},
        "published": {"plain_s": PUBLISHED_S["plain"], "ti_s": PUBLISHED_S["ti"],
                      "hardware": "LRZ CoolMUC-4 node, 112 OpenMP threads",
                      "source": "benchmark_hpc/bench_out/q16/plots/n5_q16_u601_invariance_scaling.txt:10-11"},
        "runs": rows, "accuracy": acc}))


def run_hostmap(a):
    """config hostmap: a target given as a caller's host map, the pattern of the reference's
    drivers (benchmark_hpc/benchmark_threads.c:24-33 pass a host brickwall apply as `ufunc`):
    L=14, 5-layer fit against a 16-layer random brickwall applied on the host (a plain C map
    from tests/helpers), one projected-gradient evaluation with the map called from all host
    threads and from one (the latter on a column sample, scaled), beside the same brickwall
    as a GPU target and the oracle port on all host cores"""
    import ctypes as C
    import numpy as np
    import mgcu
    import targets as T
    lib = mgcu.default_lib()
    helpers = C.CDLL(os.path.join(ROOT, "tests", "_build", "libmgtest.so"))
    L, nl, nu = 14, 5, 16
    rng = np.random.default_rng(14)
    ul, up = T.haar_matchgates(nu, rng), T.brickwall_perms(L, nu)
    v, perms = T.near_identity_brickwall(nl, rng), T.brickwall_perms(L, nl)
    g = np.ascontiguousarray(ul.reshape(-1, 8)); pp = np.ascontiguousarray(up.astype(np.int32))

    class HB(C.Structure):
        _fields_ = [("gates", C.c_void_p), ("perms", C.c_void_p), ("nlayers", C.c_int)]
    hb = HB(g.ctypes.data, pp.ctypes.data, nu)
    uf, ud = mgcu.ufunc_address(helpers.mgt_brickwall_ufunc), C.addressof(hb)
    lib.set_precision(mgcu.PREC_FP64)
    ncols = 1 << L
    lib.brickwall_columns(uf, ud, v, perms, L, 0, 64)   # plans and module loading
    t0 = time.perf_counter()
    rc, f_all, g_all = lib.brickwall_projected_gradient(uf, ud, v, perms, L)
    s_all = time.perf_counter() - t0
    assert rc == 0, lib.last_error()
    threads = os.cpu_count()
    lib.set_option(mgcu.OPT_HOST_THREADS, 1)
    sample = 512
    t0 = time.perf_counter()
    rc, _, _ = lib.brickwall_columns(uf, ud, v, perms, L, 0, sample)
    s_one = (time.perf_counter() - t0) * ncols / sample
    lib.set_option(mgcu.OPT_HOST_THREADS, 0)
    t = lib.target_brickwall(ul, up, L)
    lib.brickwall_projected_gradient(lib.mg_target_apply, t, v, perms, L)
    t0 = time.perf_counter()
    rc, f_gpu, g_gpu = lib.brickwall_projected_gradient(lib.mg_target_apply, t, v, perms, L)
    s_gpu = time.perf_counter() - t0
    lib.target_free(t)
    out = {"metric": "projected-gradient evaluation with a host-map target, L=14 (seconds)", "value": s_all, "unit": "s",
           "higher_is_better": False, "n_gpus": 1, "dtype": "f64",
           "data": "synthetic (seed 14: 16-layer Haar brickwall target applied by a host C map; 5-layer near-identity fit)",
           "config": {"workload": "matchgate_brickwall_unitary_target_and_projected_gradient with a host linear_func",
                      "L": L, "nlayers": nl, "target_layers": nu},
           "host_threads": threads, "host_map_all_threads_s": s_all,
           "host_map_one_thread_s": s_one, "one_thread_sample": f"{sample} of {ncols} columns, scaled",
           "gpu_target_s": s_gpu,
           "rel_diff_host_map_vs_gpu_target": float(abs(f_all - f_gpu) / abs(f_gpu))}
    if not a.no_cpu:
        import oracle
        tt = oracle.Target("brickwall", L, ulist=ul, uperms=up)
        nc = threads * 32
        t0 = time.perf_counter()
        oracle.brickwall_projected_gradient(tt, v, perms, L, nthreads=threads, col_range=(0, nc))
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": cs * ncols / nc, "unit": "s", "cores": threads, "kind": "port",
                               "sample": f"{nc} of {ncols} columns in {cs:.1f} s, scaled to one evaluation"}
    print(json.dumps(out))


def batch_workload(n=64, seed=4):
    """64 instances: L ~ U{10,12,14,16}, fitted depth ~ U{3..9} (Haar-random layers),
    target = a random matchgate brickwall of twice the depth; seeded"""
    import numpy as np
    import targets as T
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.choice([10, 12, 14, 16]))
        nl = int(rng.integers(3, 10))
        out.append({"L": L, "nl": nl, "ul": T.haar_matchgates(2 * nl, rng), "uperms": T.brickwall_perms(L, 2 * nl),
                    "v": T.haar_matchgates(nl, rng), "perms": T.brickwall_perms(L, nl)})
    return out


def _batch_eval(lib, mgcu, inst, prec, steps, warmup):
    lib.set_precision(prec)
    args = ([x["t"] for x in inst], [x["v"] for x in inst], [x["perms"] for x in inst], [x["L"] for x in inst])
    b = lib.batch_create(*args)
    for _ in range(warmup):
        assert lib.batch_run(b) == 0, lib.last_error()
    n1 = lib.launch_count()
    ms = lib.batch_time_ms(b, steps, True)
    assert ms > 0, lib.last_error()
    launches = (lib.launch_count() - n1) / steps
    res = [lib.batch_results(b, i) for i in range(len(inst))]
    info = [lib.batch_info(b, i) for i in range(len(inst))]
    lib.batch_free(b)
    return {"s": ms / 1e3 / steps, "res": res, "info": info, "launches": launches}


def _one_at_a_time(lib, mgcu, inst, prec):
    lib.set_precision(prec)
    tot = 0.0
    for x in inst:
        plan = lib.plan_brickwall(lib.mg_target_apply, x["t"], x["v"], x["perms"], x["L"], mgcu.EVAL_GRADIENT)
        assert lib.lib.mg_plan_run(mgcu.P(plan)) == 0
        tot += lib.lib.mg_plan_time_ms(mgcu.P(plan), 1, 0)
        lib.lib.mg_plan_free(mgcu.P(plan))
    return tot / 1e3


def run_batch(a):
    """config batch64: one batch of 64 uneven instances (f + gradient each), against the
    same instances one device-resident plan at a time; FP64 on the L<=14 instances"""
    import numpy as np
    import mgcu
    lib = mgcu.default_lib()
    inst = batch_workload()
    for x in inst:
        x["t"] = lib.target_brickwall(x["ul"], x["uperms"], x["L"])
    mx = _batch_eval(lib, mgcu, inst, mgcu.PREC_MIXED, a.steps, a.warmup)
    seq = _one_at_a_time(lib, mgcu, inst, mgcu.PREC_MIXED)
    small = [x for x in inst if x["L"] <= 12]
    mx_small = _batch_eval(lib, mgcu, small, mgcu.PREC_MIXED, 3, 1)
    seq_small = _one_at_a_time(lib, mgcu, small, mgcu.PREC_MIXED)
    sub = [i for i, x in enumerate(inst) if x["L"] <= 14]
    fp = _batch_eval(lib, mgcu, [inst[i] for i in sub], mgcu.PREC_FP64, 1, 1)
    mx_sub = _batch_eval(lib, mgcu, [inst[i] for i in sub], mgcu.PREC_MIXED, 1, 1)
    lib.set_precision(mgcu.PREC_MIXED)
    for x in inst:
        lib.target_free(x["t"])
    ef = max(abs(mx["res"][i][0] - f[0]) / max(abs(f[0]), 1e-300) for i, f in zip(sub, fp["res"]))
    eg = max(float(np.linalg.norm(mx["res"][i][2] - f[2]) / max(np.linalg.norm(f[2]), 1e-300)) for i, f in zip(sub, fp["res"]))
    Ls = [x["L"] for x in inst]
    tiles = {}
    for x, (kt, npass, items) in zip(inst, mx["info"]):
        tiles.setdefault(x["L"], set()).add(kt)
    print(json.dumps({
        "metric": "batch evaluations/s (64 uneven instances, f + Riemannian gradient each)",
        "value": 1.0 / mx["s"], "unit": "batches/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": mx["s"] * 1e3, "higher_is_better": True, "dtype": "f32 float-float pairs, f64 sums",
        "data": "synthetic (seed 4: L ~ U{10,12,14,16}, depth ~ U{3..9}, Haar layers; random brickwall targets of twice the depth)",
        "config": {"workload": "64 instances in one batch: one persistent fused launch (target sweep + fitted circuit per "
                               "column, work items largest first), captured CUDA graph",
                   "instances_per_L": {str(L): Ls.count(L) for L in sorted(set(Ls))},
                   "tuned_target_tile_bits_per_L": {str(L): sorted(v) for L, v in sorted(tiles.items())},
                   "l2": "a 512 MiB buffer is written between timed replays"},
        "gpu_launches": mx["launches"],
        "one_plan_at_a_time_s": seq, "speedup_batch_vs_one_at_a_time": seq / mx["s"],
        "small_instances": {"instances": len(small), "L": "10, 12", "batch_s": mx_small["s"], "one_plan_at_a_time_s": seq_small,
                            "speedup": seq_small / mx_small["s"]},
        "fp64_subset": {"instances": len(sub), "L": "<= 14", "fp64_batch_s": fp["s"], "mixed_batch_s": mx_sub["s"],
                        "speedup_mixed_vs_fp64": fp["s"] / mx_sub["s"]},
        "accuracy": {"max_rel_err_f_vs_fp64": ef, "max_rel_err_grad_vs_fp64": eg, "instances": len(sub)}}))


def serve_stream(lib, n, Lmax, seed=5, hess_max_L=12):
    """a seeded Poisson stream (200 requests/s) of f / gradient / Hessian / trust-region-step
    requests (40/40/10/10 %) through the request server in float-float, HBM budget 120 GiB;
    returns the latency summary (completion - submission per request)"""
    import threading
    import numpy as np
    import mgcu
    import targets as T
    lib.set_precision(mgcu.PREC_MIXED)
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1 / 200.0, size=n))
    kinds = rng.choice([mgcu.REQ_TARGET, mgcu.REQ_GRADIENT, mgcu.REQ_HESSIAN, mgcu.REQ_TRSTEP], size=n, p=[0.4, 0.4, 0.1, 0.1])
    reqs = []
    for k in kinds:
        # Hessians and trust-region steps (G^2 work per column) on L <= hess_max_L
        L = int(rng.choice([x for x in range(10, (Lmax if k <= mgcu.REQ_GRADIENT else hess_max_L) + 1, 2)]))
        nl = int(rng.integers(3, 10))
        ul = T.haar_matchgates(2 * nl, rng)
        reqs.append({"kind": int(k), "L": L, "nl": nl, "t": lib.target_brickwall(ul, T.brickwall_perms(L, 2 * nl), L),
                     "v": T.near_identity_brickwall(nl, rng), "perms": T.brickwall_perms(L, nl)})
    sv = lib.server_create(120 << 30)
    # warm-up outside the measured stream: module loading and the first plans
    for x in reqs[:10]:
        lib.server_result(sv, lib.server_submit(sv, x["kind"], x["t"], x["v"], x["perms"], x["L"], 0.05), x["nl"])
    steps0, batched0, _ = lib.server_stats(sv)
    ids = [None] * n
    t0 = time.perf_counter()

    def producer():
        for i, x in enumerate(reqs):
            dt = t0 + arrivals[i] - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            ids[i] = lib.server_submit(sv, x["kind"], x["t"], x["v"], x["perms"], x["L"], 0.05)
    th = threading.Thread(target=producer)
    th.start()
    th.join()
    res = [lib.server_result(sv, ids[i], x["nl"]) for i, x in enumerate(reqs)]
    steps1, batched1, peak = lib.server_stats(sv)
    lib.server_free(sv)
    for x in reqs:
        lib.target_free(x["t"])
    assert all(r["status"] == 0 for r in res)
    lat = np.array([(r["times"][2] - r["times"][0]) * 1e3 for r in res])
    span = max(r["times"][2] for r in res) - min(r["times"][0] for r in res)
    by_kind = {}
    for name, k in (("target", 0), ("gradient", 1), ("hessian", 2), ("trstep", 3)):
        l = lat[[i for i, x in enumerate(reqs) if x["kind"] == k]]
        if len(l):
            by_kind[name] = {"n": int(len(l)), "p50_ms": float(np.percentile(l, 50)), "p99_ms": float(np.percentile(l, 99))}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)), "throughput_rps": n / span,
            "requests": n, "offered_rate_rps": 200.0, "stream_s": float(arrivals[-1]),
            "data": f"seed {seed}: Poisson arrivals at 200/s, mix 40/40/10/10 target/gradient/Hessian/TR step, depth U{{3..9}}, "
                    f"random brickwall targets of twice the depth; L U{{10..{Lmax}}} even (Hessian and TR step: L even "
                    f"U{{10..{hess_max_L}}}); the first {n} requests of the stream",
            "steps": steps1 - steps0, "requests_batched": batched1 - batched0, "peak_step_budget_bytes": peak,
            "by_kind": by_kind}


def run_serve(a):
    """config serve: the seeded request stream through the request server"""
    import mgcu
    lib = mgcu.default_lib()
    r = serve_stream(lib, a.serve_requests, a.serve_max_L, hess_max_L=a.serve_hess_max_L)
    print(json.dumps({
        "metric": "serving p50/p99 latency (ms) and throughput (requests/s)", "value": r["p50_ms"],
        "unit": "ms (p50)", "p99_ms": r["p99_ms"], "throughput_rps": r["throughput_rps"], "n_gpus": 1,
        "higher_is_better": False, "dtype": "f32 float-float pairs, f64 sums", "data": "synthetic (" + r["data"] + ")",
        "config": {"workload": "request server, continuous batching (a step's Hessian and trust-region requests on a "
                               "second stream beside its f / gradient batch), HBM budget 120 GiB", "steps": r["steps"],
                   "requests_batched": r["requests_batched"], "peak_step_budget_bytes": r["peak_step_budget_bytes"],
                   "offered_rate_rps": 200.0, "stream_s": r["stream_s"], "requests": r["requests"]},
        "by_kind": r["by_kind"]}))


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.config == "batch64":
        run_batch(a)
    elif a.config == "serve":
        run_serve(a)
    elif a.config == "published":
        run_published(a)
    elif a.config == "hostmap":
        run_hostmap(a)
    elif a.config != "grad16":
        run_secondary(a)
    else:
        run_gb300(a)


if __name__ == "__main__":
    main()
