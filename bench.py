#!/usr/bin/env python
"""Benchmark: orbit-steps/s of gala's orbit-integration hot path on one GB300.

Headline workload (``uneven_batch``): 262,144 orbits in the Milky-Way-like
composite (nucleus Hernquist 1.7e9/0.07 + bulge Hernquist 5e9/1 +
Miyamoto-Nagai 6.8e10/3/0.28 + NFW 5.4e11/15.6), R ~ U[2, 30] kpc, |z| < 2 kpc,
v = v_c(R) + N(0, 30 km/s); per-orbit n_steps log-uniform in [100, 20000], dt
from {0.1, 0.5, 1.0} Myr, Leapfrog for half the orbits and Ruth4 for the other
half.  One step = one integration of every orbit (9.83e8 orbit-steps).
``value`` is the FP32-compensated persistent-queue kernel replayed as one CUDA
graph (inputs resident in HBM); the line also carries the plain FP64 GPU form
of the same workload (gala's per-orbit arithmetic), the ratio between them, the
FP32 form's energy drift and its final-position error against the FP64 form.
``e2e`` runs the public call ``integrate_batch`` with pinned host arrays in and
out, host<->device copies inside the timed region.

Variants in the same line (compact; ``--detail FILE`` writes every figure):
  mw_dop853           DOP853 rtol 1e-10 atol 1e-12 FP64 on 100,000 orbits x
                      10,000 steps through integrate_orbit (the plain drop-in)
  hernquist_leapfrog  Leapfrog on Hernquist, 1,024 orbits x 1,000 steps, every
                      snapshot stored (HBM snapshot stream)
  scf_surrogate       SCF nmax 12 lmax 8 host, 262,144 orbits x 5,000 Leapfrog
                      steps: learned surrogate vs analytic FP32 / FP64
  mock_streams        512 progenitors x 2,000 releases, DOP853 release systems;
                      the animate mode (one growing system per stream, 152
                      streams x 1,000 steps, snapshots every 10 steps)
  orbit_reductions    peri/apo/zmax over 100,000 orbits x 2,001 snapshots

Arms
  default           the CUDA library.
  --impl reference  gala's Leapfrog / Ruth4 loops (leapfrog.pyx:99-116,
                    ruth4.pyx:98-108) over gala's gradient, restated in C and
                    built with gala's flags (-Ofast), on every host thread, over
                    a bounded seeded sample of the headline workload.

Multi-GPU (torchrun): orbits are independent, so every rank integrates its own
shard of the same size (weak scaling, no data-path collective); the time is the
max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "orbit-steps/s on 1 GB300: FP32+surrogate vs plain FP64 at ΔE/E≤1e-6"
UNIT = "orbit-steps/s"

# Algorithmic work, every add, multiply, divide, sqrt, log and pow counted as
# one flop (an FMA as two).
F_RHS_MW = 2 * 17 + 21 + 26 + 6   # MW composite gradient (Hernquist x2, MN, NFW) + Hamiltonian copy/negate
F_FORCE_MW = F_RHS_MW - 6         # the gradient alone
F_LEAPFROG = 21                   # kick-drift-kick per step, besides the force
F_RUTH4 = 72                      # four kicks and four drifts per step, besides the forces
F_RUTH4_SKIP = 63                 # the same without the kick of the d = 0 sub-step
F_DOP_STEP = 6 * 159              # DOP853 attempted step per orbit: 12 stages, 8th-order update, error terms
F_DOP_DENSE = 6 * 153             # dense-output coefficients and the stage sums of the 3 extra stages
F_DOP_OUTPUT = 6 * 14 + 2         # one contd8 evaluation of 6 components
F_HERNQUIST = 17

# DRAM bytes per launch measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum),
# per orbit of the launch, scaled to the benched launch by its orbit count (the inputs are
# read once; the outputs are still in the 129 MB L2 when a launch ends):
#   batch_fp32c  18,895,872 B for 262,144 orbits (full size)  profiles/batch_fp32_kernel_uneven.md
#   dop853       1,700,864 B for 30,000 orbits                profiles/dop853_fp64_mw_composite.md
TRAFFIC_PER_ORBIT = {"batch_fp32c": (18_925_568 + 256) / 262_144, "dop853": 1_700_864 / 30_000}


def sig(x, n=4):
    """x rounded to n significant digits (compact JSON)."""
    if x is None or not isinstance(x, (int, float)) or isinstance(x, bool) or not math.isfinite(x) or x == 0:
        return x
    return float(f"{x:.{n}g}")


def measured_peak(key, fallback):
    """(value, source) of a MEASURED_PEAKS.json entry; without the file or the
    key, the fallback figure (an earlier measurement on a GB300) and 'fallback'."""
    try:
        v = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())[key]
        if isinstance(v, (int, float)) and v > 0:
            return float(v), "measured"
    except (OSError, ValueError, KeyError, TypeError):
        pass
    return float(fallback), "fallback"


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gx", choices=["gx", "reference"])
    p.add_argument("--workload", default="all",
                   choices=["all", "uneven_batch", "mw_dop853", "mw_dop853_fp32", "hernquist_leapfrog",
                            "scf_surrogate", "mock_streams", "orbit_reductions"],
                   help="all: the headline line with every variant; otherwise that workload alone "
                        "(profiling), printed as its detailed record")
    p.add_argument("--detail", default=None, help="write the detailed record of every workload to this file")
    p.add_argument("--batch-orbits", type=int, default=262_144)
    p.add_argument("--batch-step-scale", type=float, default=1.0, help="multiply the batch step counts")
    p.add_argument("--batch-precision", default="both", choices=["both", "fp32c", "fp64"])
    p.add_argument("--no-autotune", action="store_true", help="use the cached or default launch shape")
    p.add_argument("--surrogate-steps", type=int, default=30000, help="training steps of the SCF surrogate")
    p.add_argument("--surrogate-split", type=int, default=3, choices=[1, 2, 3],
                   help="tensor-core operands: 1 BF16, 2 BF16 hi+lo activations, 3 FP16")
    p.add_argument("--surrogate-orbits", type=int, default=262_144)
    p.add_argument("--surrogate-nsteps", type=int, default=5000)
    p.add_argument("--skip", default="", help="comma-separated variants to leave out")
    p.add_argument("--reduce-orbits", type=int, default=100_000)
    p.add_argument("--reduce-nsteps", type=int, default=2000)
    p.add_argument("--stream-progenitors", type=int, default=512)
    p.add_argument("--stream-nsteps", type=int, default=2000)
    p.add_argument("--stream-cpu-streams", type=int, default=8, help="streams in the CPU-baseline sample")
    p.add_argument("--animate-streams", type=int, default=152, help="streams of the animate-mode measurement")
    p.add_argument("--animate-nsteps", type=int, default=1000, help="grid steps of the animate-mode measurement")
    p.add_argument("--orbits", type=int, default=100_000, help="DOP853 variant: orbits per GPU")
    p.add_argument("--nsteps", type=int, default=10_000, help="DOP853 variant: steps")
    p.add_argument("--dop-reps", type=int, default=3, help="DOP853 variant: timed runs")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=6.0, help="target CPU time of one reference step")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi samples (every 200 ms) of SM clock and throttle reasons."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measure_fma_peak(torch, stream, fp64=True):
    """FP64 (or FP32) multiply-add throughput (TFLOP/s) from the library's FMA-chain probe."""
    from gala_gb300 import _abi

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096 if fp64 else 65536
    sink = torch.zeros(blocks * threads, dtype=torch.float64 if fp64 else torch.float32, device="cuda")
    h = int(stream.cuda_stream)
    f = 1 if fp64 else 0
    for _ in range(2):
        _abi.call("gx_calibrate_fma", f, blocks, threads, iters, int(sink.data_ptr()), h)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = None
    for _ in range(3):
        e0.record(stream)
        _abi.call("gx_calibrate_fma", f, blocks, threads, iters, int(sink.data_ptr()), h)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    flops = 16.0 * iters * blocks * threads
    return flops / (best * 1e-3) / 1e12


_PEAKS = {}


def fma_peak(torch, stream, fp64):
    key = "fp64" if fp64 else "fp32"
    if key not in _PEAKS:
        _PEAKS[key] = measure_fma_peak(torch, stream, fp64)
    return _PEAKS[key]


def event_time(torch, stream, fn, reps, flush=None):
    """Mean device time (ms) of fn() over reps calls, CUDA events on `stream`,
    L2 evicted before each call when `flush` (a >L2 buffer) is given."""
    times = []
    for _ in range(reps):
        if flush is not None:
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return float(np.mean(times))


# --------------------------------------------------------------------------
# Headline workload: the uneven batch (FP32 compensated vs plain FP64)
# --------------------------------------------------------------------------
def uneven_workload(n, scale=1.0):
    from gala_gb300 import workloads as W

    pot = W.mw_composite()
    w0 = W.mw_ics(n, seed=W.SEED_BASE + 3)
    nsteps, dt, method = W.uneven_steps(n)
    if scale != 1.0:
        nsteps = np.maximum(1, np.round(nsteps * scale)).astype(np.int64)
    return pot, w0, nsteps, dt, method


def uneven_flops(nsteps, method, skip_d0=False):
    """Flops of the uneven batch.  gala's Ruth4 step evaluates four gradients;
    the first sub-step's kick coefficient is zero, and the FP32 form
    (skip_d0) neither evaluates that gradient nor applies that kick, so it is
    charged three gradients; the FP64 form keeps gala's four."""
    is_ruth4 = np.asarray(method) == 1
    r4 = F_RUTH4_SKIP + 3 * F_FORCE_MW if skip_d0 else F_RUTH4 + 4 * F_FORCE_MW
    return float(np.sum(nsteps * np.where(is_ruth4, r4, F_LEAPFROG + F_FORCE_MW)))


def cpu_uneven_run(pot, w0, nsteps, dt, method, target_s, steps, warmup, nthreads=None):
    """gala's Leapfrog / Ruth4 loops (restated, -Ofast) on the host threads over
    a seeded random sample of the workload's orbits sized to ~target_s seconds
    per step; the rate is the sample's orbit-steps per second."""
    from oracle import Oracle
    from oracle.oracle import host_threads

    fast = Oracle("fast")
    nth = nthreads or host_threads()
    n = w0.shape[1]
    rng = np.random.default_rng(12345)
    perm = rng.permutation(n)
    # single-thread probe on 64 orbits of the same mix
    probe = np.sort(perm[:64])
    t0 = time.perf_counter()
    fast.batch_fixed(pot, w0[:, probe], nsteps[probe], dt[probe], method[probe], nthreads=1)
    one = time.perf_counter() - t0
    probe_rate = float(np.sum(nsteps[probe])) / one
    mean_steps = float(np.mean(nsteps))
    ns = int(target_s * probe_rate * nth / mean_steps)
    ns = max(nth, min(n, ns))
    idx = np.sort(perm[:ns])
    w0s, ns_s, dt_s, m_s = (np.ascontiguousarray(a) for a in (w0[:, idx], nsteps[idx], dt[idx], method[idx]))
    times, out = [], None
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        out = fast.batch_fixed(pot, w0s, ns_s, dt_s, m_s, nthreads=nth)
        if i >= warmup:
            times.append(time.perf_counter() - t0)
    per = float(np.mean(times))
    work = float(np.sum(ns_s))
    return {
        "value": work / per, "unit": UNIT, "cores": nth, "kind": "port",
        "sample": f"seeded {ns} of {n} orbits ({work:.3g} orbit-steps), gala's Leapfrog/Ruth4 in C, -Ofast",
        "seconds_per_step": per, "single_thread_value": probe_rate,
    }, idx, out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pot, w0, nsteps, dt, method = uneven_workload(args.batch_orbits, args.batch_step_scale)
    base, idx, _ = cpu_uneven_run(pot, w0, nsteps, dt, method, args.cpu_seconds, args.steps, args.warmup)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": base["value"],
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": base["seconds_per_step"] * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": f"uneven_batch: {args.batch_orbits} MW orbits, n_steps logU[100,20000], "
                               "dt {0.1,0.5,1}, Leapfrog/Ruth4 half each",
                   "orbits": args.batch_orbits, "sample_orbits": int(len(idx))},
        "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample", "single_thread_value")},
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_uneven_batch(args, torch, stream, timed_steps, warmup, world=1, clocks=None):
    """FP32-compensated and plain FP64 forms of the uneven batch, each as one
    CUDA-graph replay (queue reset, persistent kernel, FP64 energy diagnostic);
    e2e through integrate_batch with pinned host arrays; CPU baseline."""
    from gala_gb300.batch import BatchIntegrator, integrate_batch
    from gala_gb300.shard import max_over_ranks

    n = args.batch_orbits
    pot, w0, nsteps, dt, method = uneven_workload(n, args.batch_step_scale)
    total = float(nsteps.sum())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    res = {"workload": f"uneven_batch: {n} MW orbits, n_steps logU[100,20000]x{args.batch_step_scale:g}, "
                       "dt {0.1,0.5,1}, Leapfrog/Ruth4 half each",
           "orbits": n, "orbit_steps": total}
    outs = {}
    precs = ["fp32c", "fp64"] if args.batch_precision == "both" else [args.batch_precision]
    for prec in precs:
        b = BatchIntegrator(pot, w0, nsteps, dt, method, precision=prec)
        if not args.no_autotune:
            b.autotune(work_fraction=0.05 if prec == "fp32c" else 0.004, reps=2)
        b.capture()
        reps = timed_steps if prec == "fp32c" else 2
        for _ in range(max(1, warmup if prec == "fp32c" else 1)):
            b.run()
        torch.cuda.synchronize()
        if prec == "fp32c" and clocks is not None:
            with clocks:
                wall0 = time.perf_counter()
                ms = event_time(torch, stream, b.run, reps, flush)
                res["wall_s_timed_region"] = time.perf_counter() - wall0
        else:
            ms = event_time(torch, stream, b.run, reps, flush)
        ms = max_over_ranks(ms) if world > 1 else ms
        # the persistent kernel alone (the roofline's kernel), eager launches
        from gala_gb300._device import stream_handle

        ms_k = event_time(torch, stream, lambda: b._launch_integrator(stream_handle(stream)), max(2, min(reps, 5)),
                          flush)
        dE = b.energy_drift().cpu().numpy()
        outs[prec] = b.w_out.cpu().numpy()
        peak = fma_peak(torch, stream, prec == "fp64")
        ach = uneven_flops(nsteps, method, skip_d0=prec == "fp32c") / (ms_k * 1e-3) / 1e12
        res[prec] = {"value": total * world / (ms * 1e-3), "ms": ms, "kernel_ms": ms_k, "config": b.config,
                     "dE_over_E_median": float(np.median(dE)), "dE_over_E_p99": float(np.percentile(dE, 99)),
                     "roofline": {"bound": "fp32" if prec == "fp32c" else "fp64", "achieved": ach, "peak": peak,
                                  "unit": "TFLOP/s", "frac": ach / peak,
                                  "traffic": (TRAFFIC_PER_ORBIT.get(f"batch_{prec}", 0) * n) or None}}
    if len(outs) == 2:
        err = np.linalg.norm(outs["fp32c"][:3] - outs["fp64"][:3], axis=0) / np.linalg.norm(outs["fp64"][:3], axis=0)
        res["position_error_vs_fp64"] = {"median": float(np.median(err)), "p99": float(np.percentile(err, 99)),
                                         "max": float(np.max(err)), "frac_le_1e-4": float(np.mean(err <= 1e-4))}
        res["speedup_fp32c_vs_fp64"] = res["fp32c"]["value"] / res["fp64"]["value"]

    if "fp32c" in precs:
        # end to end: pinned host inputs -> integrate_batch -> pinned host outputs
        hw0 = torch.from_numpy(w0).pin_memory()
        hns = torch.from_numpy(nsteps).pin_memory()
        hdt = torch.from_numpy(dt).pin_memory()
        hm = torch.from_numpy(method).pin_memory()
        out = (torch.empty((6, n), dtype=torch.float64).pin_memory(), torch.empty(n, dtype=torch.float64).pin_memory())
        e2e = []
        for i in range(warmup + timed_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            w_host, dE_host = integrate_batch(pot, hw0, hns, hdt, hm, precision="fp32c", out=out)
            if i >= warmup:
                e2e.append((time.perf_counter() - t0) * 1e3)
        e2e_ms = max_over_ranks(float(np.mean(e2e))) if world > 1 else float(np.mean(e2e))
        res["e2e"] = {"value": total * world / (e2e_ms * 1e-3), "unit": UNIT,
                      "h2d_bytes_per_step": int(w0.nbytes + nsteps.nbytes + dt.nbytes + method.nbytes),
                      "d2h_bytes_per_step": int(out[0].numel() * 8 + out[1].numel() * 8), "ms_per_step": e2e_ms,
                      "matches_device_run": bool(np.array_equal(w_host, outs["fp32c"]))}

    if world == 1 and not args.no_cpu_baseline:
        base, idx, cpu_out = cpu_uneven_run(pot, w0, nsteps, dt, method, args.cpu_seconds, 1, 0)
        cb = {k: base[k] for k in ("value", "unit", "cores", "kind", "sample", "single_thread_value")}
        for prec, o in outs.items():
            rel = (np.linalg.norm(o[:, idx] - cpu_out, axis=0) / np.linalg.norm(cpu_out, axis=0))
            cb[f"{prec}_vs_cpu_max_rel"] = float(np.max(rel))
            if prec == "fp32c":
                pe = (np.linalg.norm(o[:3, idx] - cpu_out[:3], axis=0) / np.linalg.norm(cpu_out[:3], axis=0))
                cb["fp32c_position_error_vs_cpu_median"] = float(np.median(pe))
        res["cpu_baseline"] = cb
    return res


# --------------------------------------------------------------------------
# Variant: DOP853 FP64 through integrate_orbit (config 2)
# --------------------------------------------------------------------------
def run_mw_dop853(args, torch, stream, reps, warmup, world=1, rank=0):
    import gala_gb300 as g
    from gala_gb300 import _abi
    from gala_gb300 import workloads as W
    from gala_gb300.shard import max_over_ranks, shard_range

    mw = W.mw_composite()
    nsteps, stride, nbatch = args.nsteps, 100, 100
    n_global = args.orbits * world
    lo, hi = shard_range(n_global, rank, world, nbatch)
    n = hi - lo
    w0 = np.ascontiguousarray(W.mw_ics(n_global, seed=W.SEED_BASE + 2)[:, lo:hi])
    t = g.parse_time_specification(dt=0.5, n_steps=nsteps)
    ntimes = len(t)
    n_out = (ntimes - 1) // stride + 1
    nb = (n + nbatch - 1) // nbatch
    dev = torch.device("cuda", torch.cuda.current_device())
    w0d = torch.from_numpy(w0).to(dev)
    td = torch.from_numpy(t).to(dev)
    out = torch.empty((6, n_out, n), dtype=torch.float64, device=dev)
    status = torch.zeros(nb, dtype=torch.int32, device=dev)
    stats = torch.zeros((nb, 4), dtype=torch.int64, device=dev)
    desc = mw.packed().for_device()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    sh = int(stream.cuda_stream)

    def launch():
        _abi.call("gx_dop853_integrate_hamiltonian", desc, None, int(w0d.data_ptr()), n, int(td.data_ptr()),
                  ntimes, 1e-12, 1e-10, 0, 0.0, 0, 1, nbatch, stride, int(out.data_ptr()), int(status.data_ptr()),
                  int(stats.data_ptr()), sh)

    for _ in range(warmup):
        launch()
    torch.cuda.synchronize()
    ms = event_time(torch, stream, launch, reps, flush)
    ms = max_over_ranks(ms) if world > 1 else ms
    st = status.cpu().numpy()
    if np.any(st != 1):
        raise RuntimeError(f"integration failed in {int(np.sum(st != 1))} batches: {np.unique(st)}")
    stt = stats.cpu().numpy()
    nb_sizes = np.full(nb, nbatch, dtype=np.int64)
    nb_sizes[-1] = n - nbatch * (nb - 1)
    # dense-output preparations from the counters: nfcn = 2 + 11 nstep + naccpt + 3 n_dense
    n_dense = (stt[:, 0] - 2 - 11 * stt[:, 1] - stt[:, 2]) // 3
    flops = float(np.sum(nb_sizes * (stt[:, 0] * F_RHS_MW + stt[:, 1] * F_DOP_STEP + n_dense * F_DOP_DENSE))
                  + n * n_out * F_DOP_OUTPUT)
    H = g.Hamiltonian(mw)
    E0 = H.energy(out[:, 0, :].cpu().numpy())
    E1 = H.energy(out[:, -1, :].cpu().numpy())
    dE = np.abs((E1 - E0) / E0)

    e2e = []
    for i in range(1 + max(1, reps - 1)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        orbit = mw.integrate_orbit(w0, dt=0.5, n_steps=nsteps, Integrator="dop853",
                                   Integrator_kwargs=dict(atol=1e-12, rtol=1e-10, out_stride=stride))
        wout = orbit.w()
        if i >= 1:
            e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = max_over_ranks(float(np.mean(e2e))) if world > 1 else float(np.mean(e2e))
    f32 = run_dop853_fp32(args, torch, stream, mw, w0d, td, ntimes, stride, n, flush, out.cpu().numpy(), H, E0)
    peak = fma_peak(torch, stream, True)
    ach = flops / (ms * 1e-3) / 1e12
    res = {"workload": f"mw_dop853: MW composite, DOP853 rtol 1e-10 atol 1e-12 FP64, {args.orbits} orbits, "
                       f"dt 0.5 Myr, {nsteps} steps, every {stride}th output kept",
           "value": n_global * nsteps / (ms * 1e-3), "ms": ms,
           "e2e": {"value": n_global * nsteps / (e2e_ms * 1e-3), "ms": e2e_ms,
                   "h2d_bytes": int(w0.nbytes + t.nbytes), "d2h_bytes": int(wout.nbytes + status.numel() * 4),
                   "matches_device_run": bool(np.array_equal(wout, out.cpu().numpy()))},
           "roofline": {"bound": "fp64", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                        "flops_per_orbit": flops / n,
                        "traffic": (TRAFFIC_PER_ORBIT.get("dop853", 0) * n) or None},
           "dE_over_E_median": float(np.median(dE)), "dE_over_E_p99": float(np.percentile(dE, 99)),
           "counters_per_orbit": {"nfcn": float(np.mean(stt[:, 0])), "attempted": float(np.mean(stt[:, 1])),
                                  "accepted": float(np.mean(stt[:, 2])), "dense": float(np.mean(n_dense))},
           "fp32": f32}
    f32["speedup_vs_fp64"] = f32["value"] / res["value"]
    if world == 1 and not args.no_cpu_baseline:
        base, sample, cpu_out = cpu_dop853_run(mw, w0, t, args.cpu_seconds)
        gpu_sample = out[:, :, : sample.shape[1]].cpu().numpy()
        rel = np.linalg.norm(gpu_sample - cpu_out, axis=0) / np.linalg.norm(cpu_out, axis=0)
        base["gpu_vs_cpu_max_rel"] = float(np.max(rel))
        res["cpu_baseline"] = base
    return res


DOP32_ATOL, DOP32_RTOL = 1e-10, 1e-8


def run_dop853_fp32(args, torch, stream, mw, w0d, td, ntimes, stride, n, flush, ref=None, H=None, E0=None):
    """The FP32-stage / FP64-control DOP853 (per-orbit step control) on the same
    orbits at atol 1e-10, rtol 1e-8 (FP32 stages resolve ~1e-8 relative per
    step), against the FP64 form's outputs when given."""
    from gala_gb300 import _abi

    n_out = (ntimes - 1) // stride + 1
    out = torch.empty((6, n_out, n), dtype=torch.float64, device="cuda")
    status = torch.zeros(n, dtype=torch.int32, device="cuda")
    stats = torch.zeros((n, 4), dtype=torch.int64, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    desc = mw.packed().for_device()
    sh = int(stream.cuda_stream)

    from gala_gb300.hamiltonian import cost_order

    order = cost_order(mw, w0d, sh)

    def launch():
        _abi.call("gx_dop853_fp32", desc, None, int(w0d.data_ptr()), n, int(td.data_ptr()), ntimes, DOP32_ATOL,
                  DOP32_RTOL, 0, 0.0, 0, 1, stride, int(order.data_ptr()), int(out.data_ptr()),
                  int(status.data_ptr()), int(stats.data_ptr()), int(cnt.data_ptr()), sh)

    launch()
    torch.cuda.synchronize()
    ms = event_time(torch, stream, launch, max(2, args.dop_reps), flush)
    stt = stats.cpu().numpy()
    nsteps = ntimes - 1
    n_dense = (stt[:, 0] - 2 - 11 * stt[:, 1] - stt[:, 2]) // 3
    flops = float(np.sum(stt[:, 0] * F_RHS_MW + stt[:, 1] * F_DOP_STEP + n_dense * F_DOP_DENSE)
                  + n * n_out * F_DOP_OUTPUT)
    peak = fma_peak(torch, stream, False)
    res = {"value": n * nsteps / (ms * 1e-3), "ms": ms, "atol": DOP32_ATOL, "rtol": DOP32_RTOL,
           "status_ok_fraction": float(np.mean(status.cpu().numpy() == 1)),
           "roofline": {"bound": "fp32", "achieved": flops / (ms * 1e-3) / 1e12, "peak": peak, "unit": "TFLOP/s",
                        "frac": flops / (ms * 1e-3) / 1e12 / peak},
           "counters_per_orbit": {"nfcn": float(np.mean(stt[:, 0])), "attempted": float(np.mean(stt[:, 1])),
                                  "accepted": float(np.mean(stt[:, 2]))}}
    if ref is not None:
        w = out.cpu().numpy()
        pe = np.linalg.norm(w[:3, -1] - ref[:3, -1], axis=0) / np.linalg.norm(ref[:3, -1], axis=0)
        dE = np.abs((H.energy(w[:, -1]) - E0) / E0)
        res.update({"position_error_vs_fp64_median": float(np.median(pe)),
                    "position_error_vs_fp64_p99": float(np.percentile(pe, 99)),
                    "position_error_vs_fp64_max": float(np.max(pe)),
                    "dE_over_E_median": float(np.median(dE)), "dE_over_E_p99": float(np.percentile(dE, 99))})
    return res


def cpu_dop853_run(mw, w0_all, t, target_s):
    """gala's DOP853 (restated, -Ofast) on the host threads over whole 100-orbit
    batches of the workload, sized to ~target_s seconds."""
    from oracle import Oracle
    from oracle.oracle import host_threads

    fast = Oracle("fast")
    nthreads = host_threads()
    nsteps = len(t) - 1
    probe = w0_all[:, :100]
    t0 = time.perf_counter()
    fast.dop853(mw, probe, t, atol=1e-12, rtol=1e-10, out_stride=100, nthreads=1)
    one = time.perf_counter() - t0
    nb = int(round(target_s * nthreads / max(one, 1e-3)))
    nb = max(nthreads, (nb // nthreads) * nthreads)
    nb = max(1, min(nb, w0_all.shape[1] // 100))
    nthreads = min(nthreads, nb)
    sample = np.ascontiguousarray(w0_all[:, : nb * 100])
    t0 = time.perf_counter()
    out, _, _ = fast.dop853(mw, sample, t, atol=1e-12, rtol=1e-10, out_stride=100, nthreads=nthreads)
    per = time.perf_counter() - t0
    return {"value": sample.shape[1] * nsteps / per, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{nb} batches x 100 orbits x {nsteps} steps, gala's DOP853 restated in C, -Ofast, "
                      f"{nthreads} threads",
            "single_thread_value": probe.shape[1] * nsteps / one}, sample, out


# --------------------------------------------------------------------------
# Variant: Leapfrog on Hernquist, every snapshot stored (config 1)
# --------------------------------------------------------------------------
def run_hernquist_leapfrog(args, torch, stream):
    import gala_gb300 as g
    from gala_gb300 import _abi
    from gala_gb300 import workloads as W

    pot = W.hernquist_potential()
    n, nsteps = 1024, 1000
    w0 = W.hernquist_ics(n)
    t = g.parse_time_specification(dt=1.0, n_steps=nsteps)
    ntimes = len(t)
    w0d = torch.from_numpy(w0).cuda()
    td = torch.from_numpy(t).cuda()
    out = torch.empty((6, ntimes, n), dtype=torch.float64, device="cuda")
    desc = pot.packed().for_device()
    sh = int(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def launch():
        _abi.call("gx_leapfrog_integrate_hamiltonian", desc, None, int(w0d.data_ptr()), n, int(td.data_ptr()),
                  ntimes, 1, int(out.data_ptr()), sh)

    for _ in range(3):
        launch()
    ms = event_time(torch, stream, launch, 10, flush)
    algo_bytes = 48.0 * n * ntimes + 48.0 * n + 8.0 * ntimes
    hbm, hbm_src = measured_peak("hbm_gbs", 6800.0)
    fl = float(n * nsteps * (F_LEAPFROG + F_HERNQUIST))
    peak64 = fma_peak(torch, stream, True)
    e2e = []
    for i in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        o = pot.integrate_orbit(w0, dt=1.0, n_steps=nsteps, Integrator="leapfrog")
        wout = o.w()
        if i:
            e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = float(np.mean(e2e))
    res = {"workload": "hernquist_leapfrog: Hernquist m=1e11 c=1, 1024 orbits, dt 1 Myr, 1000 steps, all snapshots",
           "value": n * nsteps / (ms * 1e-3), "ms": ms,
           "roofline": {"bound": "hbm (snapshot stream)", "achieved": algo_bytes / (ms * 1e-3) / 1e9, "peak": hbm,
                        "unit": "GB/s", "frac": algo_bytes / (ms * 1e-3) / 1e9 / hbm, "bytes_per_launch": algo_bytes,
                        "peak_source": hbm_src, "fp64_frac": fl / (ms * 1e-3) / 1e12 / peak64},
           "e2e": {"value": n * nsteps / (e2e_ms * 1e-3), "ms": e2e_ms, "h2d_bytes": int(w0.nbytes + t.nbytes),
                   "d2h_bytes": int(wout.nbytes)}}
    if not args.no_cpu_baseline:
        from oracle import Oracle
        from oracle.oracle import host_threads

        fast = Oracle("fast")
        nth = host_threads()
        ref = None
        for th in (1, nth):
            t0 = time.perf_counter()
            ref = fast.fixed(pot, w0, t, "leapfrog", save_all=True, nthreads=th)
            s = time.perf_counter() - t0
            res.setdefault("cpu_baseline", {})["value" if th == nth else "single_thread_value"] = n * nsteps / s
        res["cpu_baseline"].update({"unit": UNIT, "cores": nth, "kind": "port",
                                    "sample": "the whole workload, gala's Leapfrog loop restated in C, -Ofast",
                                    "gpu_vs_cpu_max_rel": float(np.max(np.abs(out.cpu().numpy() - ref) /
                                                                       np.maximum(np.abs(ref), 1e-300)))})
    return res


# --------------------------------------------------------------------------
# Variant: SCF host and its learned surrogate (config 4)
# --------------------------------------------------------------------------
def run_scf_surrogate(args, torch, stream):
    """SCF(m=1e12, r_s=20, nmax=12, lmax=8) with random coefficients, 262,144
    orbits, dt = 1 Myr, 5,000 Leapfrog steps.  A surrogate is trained on 16M
    analytic samples (timed separately), then the same FP32 leapfrog runs with
    (a) the tensor-core surrogate, (b) the analytic SCF force in FP32; the plain
    FP64 form (gala's arithmetic, analytic SCF) is timed on a 20-step run of all
    orbits.  Accuracy: force and potential error on 50k held-out points; orbit
    position error and energy change against the FP64 form on 2,048 orbits over
    1,000 steps (the energy change minus the FP64 orbit's own, which carries
    Leapfrog's truncation oscillation).  Gain at equal accuracy: the analytic
    SCF cut at the lowest degree L whose force error does not exceed the
    surrogate's, timed the same way."""
    import gala_gb300 as g
    from gala_gb300 import surrogate as S
    from gala_gb300 import workloads as W

    n_orbits, n_steps = args.surrogate_orbits, args.surrogate_nsteps
    scf = W.scf_potential()
    sp = S.SurrogatePotential(scf, seed=0, split=args.surrogate_split)
    t0 = time.perf_counter()
    sp.make_dataset(n_samples=16 << 20)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    hist = sp.train(steps=args.surrogate_steps, batch=8192, lr=1e-3, log_every=max(1, args.surrogate_steps // 4))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    x = sp.sample_positions(50000, seed=99)
    xh = x.cpu().numpy()
    ref = scf.gradient(xh)
    pref = scf.energy(xh)

    def ferr(gr):
        return np.linalg.norm(gr - ref, axis=0) / np.linalg.norm(ref, axis=0)

    grad, phi = sp.gradient_and_energy(x)
    fe = ferr(grad.cpu().numpy())
    pe = np.abs(phi.cpu().numpy() - pref) / np.abs(pref)
    w0 = W.scf_ics(n_orbits)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), out

    ms_sur, (wsur, fb) = timed(lambda: sp.integrate_leapfrog(w0, 1.0, n_steps, engine="tcgen05"))
    n32 = min(65536, n_orbits)
    ms_f32, _ = timed(lambda: sp.integrate_leapfrog(w0[:, :n32], 1.0, 200, analytic=True))
    ms_f64, _ = timed(lambda: scf.integrate_orbit(w0, dt=1.0, n_steps=20, Integrator="leapfrog", save_all=False,
                                                  return_device=True))
    v_sur = n_orbits * n_steps / (ms_sur * 1e-3)
    flops_run = float(n_orbits * (n_steps + 1)) * 6 * 2 * 256 * 256 * (2 if sp.split == 2 else 1)
    bf16_peak, bf16_src = measured_peak("bf16_tflops_sustained", 1700.0)
    v_f32 = n32 * 200 / (ms_f32 * 1e-3)
    v_f64 = n_orbits * 20 / (ms_f64 * 1e-3)

    # the analytic SCF cut to the surrogate's force accuracy
    trunc = None
    for L in range(0, int(scf.parameters["Snlm"].shape[1])):
        sc = S.truncated_scf(scf, L)
        e_L = ferr(sc.gradient(xh))
        if np.median(e_L) <= np.median(fe):
            sp_L = S.SurrogatePotential(sc, seed=0)
            ms_L, _ = timed(lambda: sp_L.integrate_leapfrog(w0[:, :n32], 1.0, 200, analytic=True))
            trunc = {"lmax": L, "force_error_median": float(np.median(e_L)), "value": n32 * 200 / (ms_L * 1e-3)}
            break

    sub = w0[:, :min(2048, n_orbits)]
    o64 = scf.integrate_orbit(sub, dt=1.0, n_steps=1000, Integrator="leapfrog", save_all=False).w().reshape(6, -1)
    osur = sp.integrate_leapfrog(sub, 1.0, 1000)[0].cpu().numpy()
    o32 = sp.integrate_leapfrog(sub, 1.0, 1000, analytic=True)[0].cpu().numpy()
    H = g.Hamiltonian(scf)
    E0 = H.energy(sub)
    dE64 = (H.energy(o64) - E0) / E0

    def errs(o):
        pe_ = np.linalg.norm(o[:3] - o64[:3], axis=0) / np.linalg.norm(o64[:3], axis=0)
        dE = (H.energy(o) - E0) / E0
        return {"position_error_median": float(np.median(pe_)), "position_error_p90": float(np.percentile(pe_, 90)),
                "dE_over_E_median": float(np.median(np.abs(dE))),
                "dE_over_E_vs_fp64_median": float(np.median(np.abs(dE - dE64)))}

    return {
        "workload": f"scf_surrogate: SCF m=1e12 r_s=20 nmax=12 lmax=8, {n_orbits} orbits, dt 1 Myr, "
                    f"{n_steps} Leapfrog steps",
        "surrogate": {"value": v_sur, "ms": ms_sur, "operands": {1: "BF16", 2: "BF16 hi+lo", 3: "FP16"}[sp.split],
                      "fallback_force_evaluations": int(fb.item()),
                      "roofline": {"bound": "tensor", "unit": "TFLOP/s",
                                   "achieved": flops_run / (ms_sur * 1e-3) / 1e12, "peak": bf16_peak,
                                   "frac": flops_run / (ms_sur * 1e-3) / 1e12 / bf16_peak,
                                   "peak_source": f"{bf16_src}, cuBLAS BF16 sustained"}},
        "fp32_analytic": {"value": v_f32, "sample": f"{n32} orbits x 200 steps"},
        "fp64_analytic_plain": {"value": v_f64, "sample": f"{n_orbits} orbits x 20 steps"},
        "equal_accuracy_analytic": trunc,
        "speedup_surrogate_vs_fp64": v_sur / v_f64,
        "speedup_surrogate_vs_fp32_analytic": v_sur / v_f32,
        "speedup_at_equal_accuracy": (v_sur / trunc["value"]) if trunc else None,
        "training": {"samples": int(sp.X.shape[0]), "steps": args.surrogate_steps, "dataset_s": t_data,
                     "train_s": t_train, "loss_history": hist},
        "force_error": {"median": float(np.median(fe)), "p90": float(np.percentile(fe, 90)),
                        "p99": float(np.percentile(fe, 99))},
        "potential_error": {"median": float(np.median(pe)), "p90": float(np.percentile(pe, 90))},
        "orbits_vs_fp64_2048x1000": {"surrogate": errs(osur), "fp32_analytic": errs(o32),
                                     "fp64_leapfrog_own_dE_median": float(np.median(np.abs(dE64)))},
    }


# --------------------------------------------------------------------------
# Variant: mock streams (config 5)
# --------------------------------------------------------------------------
F_PLUMMER_PULL = 3 + 17 + 3
F_STIFF_PER_COMP = 6


def run_mock_streams(args, torch, stream):
    """512 Plummer progenitors (m ~ U[1e4, 1e6] Msun, b ~ U[5, 20] pc) on
    MW-composite disk orbits, FardalStreamDF releasing 1 particle per tail at
    every one of the 2001 times of dt = 1 Myr; DOPRI853 with gala's defaults and
    err_if_fail = 0.  Metric: particle-steps/s.  Timed: the whole pipeline and
    the release-system kernel alone; end to end through run_batch."""
    import gala_gb300 as g
    from gala_gb300 import _abi
    from gala_gb300 import workloads as W
    from gala_gb300._device import ptr
    from gala_gb300.mockstream import FardalStreamDF, MockStreamGenerator
    from gala_gb300.nbody import bodies_to_device, integrate_systems, integrate_systems_leapfrog, pack_bodies

    S, nsteps = args.stream_progenitors, args.stream_nsteps
    pot = W.mw_composite()
    w0, m, b = W.stream_progenitors(S)
    pots = W.stream_progenitor_potentials(m, b)
    kw = dict(err_if_fail=0)

    def gen(seed=1):
        return MockStreamGenerator(FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(seed)),
                                   pot)

    gen().run_batch(w0[:, :16], m[:16], progenitor_potentials=pots[:16], dt=1.0, n_steps=min(nsteps, 200),
                    Integrator_kwargs=kw)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    res = gen().run_batch(w0, m, progenitor_potentials=pots, dt=1.0, n_steps=nsteps, Integrator_kwargs=kw,
                          return_stats=True)
    e1.record(stream)
    e1.synchronize()
    ms_pipe = e0.elapsed_time(e1)
    n_rows = int(res.stream_w.shape[1])
    t_final = float(res.t[-1])
    particle_steps = S * float(np.sum(np.round(t_final - res.release_time)))
    status = res.status.cpu().numpy()
    stats = res.stats.cpu().numpy()

    t = g.parse_time_specification(dt=1.0, n_steps=nsteps)
    bodies = pack_bodies([[p] for p in pots]).reshape(S, 1)
    orbit, _ = integrate_systems(pot, bodies, np.ascontiguousarray(w0.T.reshape(S, 1, 6)), t, nstiff=-1)
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(1))
    counts = df.release_counts(len(t))
    sw0, _, _, _ = df.sample_device(pot, orbit.reshape(S, len(t), 6), t, np.repeat(m[:, None], len(t), 1), counts)
    off = torch.from_numpy(np.concatenate([[0], np.cumsum(2 * counts)]).astype(np.int64)).cuda()
    td = torch.from_numpy(t).cuda()
    bd = bodies_to_device(bodies, "cuda")
    out = torch.empty_like(sw0)
    nb_out = torch.empty((S, 1, 6), dtype=torch.float64, device="cuda")
    st_k = torch.zeros((S, len(t)), dtype=torch.int32, device="cuda")
    counter = torch.zeros(1, dtype=torch.int64, device="cuda")
    H = g.Hamiltonian(pot)
    desc = pot.packed().for_device()

    def release_kernel():
        _abi.call("gx_mockstream_dop853", desc, H._frame_ref(), S, 1, ptr(bd), ptr(orbit), len(t), ptr(td), ptr(off),
                  2, ptr(sw0), n_rows, t_final, 1.0, 1e-10, 1e-10, 0, ptr(out), ptr(nb_out), ptr(st_k), None,
                  ptr(counter), int(stream.cuda_stream))

    e0.record(stream)
    release_kernel()
    e1.record(stream)
    e1.synchronize()
    ms_rel = e0.elapsed_time(e1)
    same = bool(torch.equal(out, res.stream_w))

    # the FP32-stage / FP64-control form of the same release systems (rtol 1e-8)
    out32 = torch.empty_like(sw0)
    st32 = torch.zeros((S, len(t)), dtype=torch.int32, device="cuda")
    stats32 = torch.zeros((S, len(t), 4), dtype=torch.int64, device="cuda")

    def release_kernel_fp32():
        _abi.call("gx_mockstream_dop853_fp32", desc, S, 1, ptr(bd), ptr(orbit), len(t), ptr(td), ptr(off), 2,
                  ptr(sw0), n_rows, t_final, 1.0, DOP32_ATOL, DOP32_RTOL, 0, ptr(out32), ptr(nb_out), ptr(st32),
                  ptr(stats32), ptr(counter), int(stream.cuda_stream))

    release_kernel_fp32()
    torch.cuda.synchronize()
    e0.record(stream)
    release_kernel_fp32()
    e1.record(stream)
    e1.synchronize()
    ms_rel32 = e0.elapsed_time(e1)
    o64, o32_ = out.cpu().numpy(), out32.cpu().numpy()
    okm = np.repeat((st_k.cpu().numpy() == 1) & (st32.cpu().numpy() == 1), 2, axis=1)[:, :n_rows]
    perr32 = (np.linalg.norm(o32_[..., :3] - o64[..., :3], axis=-1) / np.linalg.norm(o64[..., :3], axis=-1))[okm]
    stt32 = stats32.cpu().numpy()
    flops32 = float(np.sum(stt32[..., 0]) * (F_RHS_MW * 3 + F_PLUMMER_PULL * 2) + np.sum(stt32[..., 1]) * 3 * F_DOP_STEP)
    nsys_p = 2
    flops = float(np.sum(stats[..., 0]) * (F_RHS_MW * (1 + nsys_p) + F_PLUMMER_PULL * nsys_p) +
                  np.sum(stats[..., 1]) * (1 + nsys_p) * F_DOP_STEP +
                  np.sum(stats[..., 2]) * 6 * (1 + nsys_p) * F_STIFF_PER_COMP)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r2 = gen().run_batch(w0, m, progenitor_potentials=pots, dt=1.0, n_steps=nsteps, Integrator_kwargs=kw)
    host_stream = r2.stream_w.cpu().numpy()
    host_nbody = r2.nbody_w.cpu().numpy()
    e2e_ms = (time.perf_counter() - t0) * 1e3

    orbit_lf = integrate_systems_leapfrog(pot, bodies, np.ascontiguousarray(w0.T.reshape(S, 1, 6)), t)
    df = FardalStreamDF(gala_modified=True, random_state=np.random.RandomState(1))
    sw_lf, _, _, _ = df.sample_device(pot, orbit_lf.reshape(S, len(t), 6), t, np.repeat(m[:, None], len(t), 1),
                                      counts)
    lf_out, lf_ms = {}, {}
    for name in ("gx_mockstream_leapfrog", "gx_mockstream_leapfrog_fp32"):
        o = torch.empty_like(sw_lf)
        st_lf = torch.zeros((S, len(t)), dtype=torch.int32, device="cuda")

        def lf_call():
            _abi.call(name, desc, S, 1, ptr(bd), ptr(orbit_lf), len(t), ptr(td), ptr(off), 2, ptr(sw_lf), n_rows,
                      t_final, 1.0, ptr(o), ptr(nb_out), ptr(st_lf), int(stream.cuda_stream))

        lf_call()
        torch.cuda.synchronize()
        e0.record(stream)
        lf_call()
        e1.record(stream)
        e1.synchronize()
        lf_ms[name] = e0.elapsed_time(e1)
        lf_out[name] = o.cpu().numpy()
    o64, o32 = lf_out["gx_mockstream_leapfrog"], lf_out["gx_mockstream_leapfrog_fp32"]
    perr = (np.linalg.norm(o32[..., :3] - o64[..., :3], axis=-1) / np.linalg.norm(o64[..., :3], axis=-1)).ravel()

    # animate mode (output_every): one growing shared-step system per stream over
    # the first args.animate_nsteps grid steps, a snapshot every 10 steps
    sa, na = min(S, args.animate_streams), min(nsteps, args.animate_nsteps) + 1
    rows_a = int(2 * counts[:na].sum())
    nd_a = torch.from_numpy((2 * counts[:na]).astype(np.int32)).cuda()
    sw_a = sw0[:sa, :rows_a].contiguous()
    nb0_a = orbit[:sa, 0].contiguous()
    td_a = td[:na].contiguous()
    Ma = 1 + rows_a
    lib = _abi.load()
    n_out_a = int(lib.gx_mockstream_animate_snapshots(na, 10))
    nbytes_a = int(lib.gx_mockstream_wide_scratch_bytes(sa, Ma))
    scratch_a = torch.empty(nbytes_a // 8, dtype=torch.float64, device="cuda")
    snap_a = torch.empty((sa, 6, n_out_a, Ma), dtype=torch.float64, device="cuda")
    w_a = torch.empty((sa, Ma, 6), dtype=torch.float64, device="cuda")
    st_a = torch.zeros((sa, na), dtype=torch.int32, device="cuda")
    stats_a = torch.zeros((sa, 4), dtype=torch.int64, device="cuda")

    def animate_call():
        _abi.call("gx_mockstream_dop853_animate", desc, H._frame_ref(), sa, 1, ptr(bd), ptr(nb0_a), na, ptr(td_a),
                  1.0, ptr(nd_a), ptr(sw_a), rows_a, 10, 1e-10, 1e-10, 0, ptr(scratch_a), nbytes_a, ptr(snap_a),
                  ptr(w_a), ptr(st_a), ptr(stats_a), int(stream.cuda_stream))

    e0.record(stream)
    animate_call()
    e1.record(stream)
    e1.synchronize()
    ms_anim = e0.elapsed_time(e1)
    # particle-steps: every particle from its release time to the end of the grid
    live = np.cumsum(2 * counts[:na])[:-1]
    anim_particle_steps = sa * float(live.sum())
    st_anim = st_a.cpu().numpy()
    # the same streams with FP32 stages and forces and FP64 step control (rtol 1e-8)
    snap_a32 = torch.empty_like(snap_a)
    w_a32 = torch.empty_like(w_a)
    st_a32 = torch.zeros_like(st_a)

    def animate_call_fp32():
        _abi.call("gx_mockstream_dop853_animate_fp32", desc, sa, 1, ptr(bd), ptr(nb0_a), na, ptr(td_a), 1.0,
                  ptr(nd_a), ptr(sw_a), rows_a, 10, DOP32_ATOL, DOP32_RTOL, 0, ptr(scratch_a), nbytes_a,
                  ptr(snap_a32), ptr(w_a32), ptr(st_a32), None, int(stream.cuda_stream))

    e0.record(stream)
    animate_call_fp32()
    e1.record(stream)
    e1.synchronize()
    ms_anim32 = e0.elapsed_time(e1)
    wa64, wa32 = w_a.cpu().numpy(), w_a32.cpu().numpy()
    perr_a = (np.linalg.norm(wa32[..., :3] - wa64[..., :3], axis=-1) / np.linalg.norm(wa64[..., :3], axis=-1)).ravel()
    lf_flops = S * float(np.sum(np.round(t_final - t))) * (3 * (F_FORCE_MW + 18) + 2 * F_PLUMMER_PULL)
    fp64_peak = fma_peak(torch, stream, True)
    result = {
        "workload": f"mock_streams: {S} Plummer progenitors on MW disk orbits, Fardal 1 particle per tail per step, "
                    f"dt 1 Myr, {nsteps} steps, DOPRI853 atol=rtol=1e-10, err_if_fail=0",
        "particle_steps": particle_steps,
        "pipeline": {"value": particle_steps / (ms_pipe * 1e-3), "unit": "particle-steps/s", "ms": ms_pipe},
        "release_kernel": {"value": particle_steps / (ms_rel * 1e-3), "ms": ms_rel, "matches_pipeline_output": same,
                           "roofline": {"bound": "fp64", "achieved": flops / (ms_rel * 1e-3) / 1e12,
                                        "peak": fp64_peak, "frac": flops / (ms_rel * 1e-3) / 1e12 / fp64_peak,
                                        "unit": "TFLOP/s"}},
        "e2e": {"value": particle_steps / (e2e_ms * 1e-3), "ms": e2e_ms,
                "h2d_bytes": int(w0.nbytes + m.nbytes + S * n_rows * 4 * 8),
                "d2h_bytes": int(host_stream.nbytes + host_nbody.nbytes)},
        "release_kernel_fp32": {"value": particle_steps / (ms_rel32 * 1e-3), "ms": ms_rel32, "atol": DOP32_ATOL,
                                "rtol": DOP32_RTOL, "speedup_vs_fp64": ms_rel / ms_rel32,
                                "position_error_vs_fp64_median": float(np.median(perr32)),
                                "position_error_vs_fp64_p99": float(np.percentile(perr32, 99)),
                                "frac_fp32": flops32 / (ms_rel32 * 1e-3) / 1e12 / fma_peak(torch, stream, False)},
        "stiff_exit_fraction": float(np.mean(status[status != 0] == -4)),
        "leapfrog_fp64": {"value": particle_steps / (lf_ms["gx_mockstream_leapfrog"] * 1e-3),
                          "frac": lf_flops / (lf_ms["gx_mockstream_leapfrog"] * 1e-3) / 1e12 / fp64_peak},
        "leapfrog_fp32c": {"value": particle_steps / (lf_ms["gx_mockstream_leapfrog_fp32"] * 1e-3),
                           "position_error_vs_fp64_median": float(np.median(perr)),
                           "position_error_vs_fp64_p99": float(np.percentile(perr, 99))},
        "animate": {"workload": f"{sa} streams, {na - 1} steps, one growing DOP853 system per stream "
                                f"(up to {Ma} members), snapshot every 10 steps ({n_out_a} snapshots)",
                    "value": anim_particle_steps / (ms_anim * 1e-3), "unit": "particle-steps/s", "ms": ms_anim,
                    "intervals_ok": float(np.mean(st_anim[:, 1:] == 1)),
                    "snapshot_bytes": int(snap_a.numel() * 8),
                    "fp32": {"value": anim_particle_steps / (ms_anim32 * 1e-3), "ms": ms_anim32, "atol": DOP32_ATOL,
                             "rtol": DOP32_RTOL, "speedup_vs_fp64": ms_anim / ms_anim32,
                             "intervals_ok": float(np.mean(st_a32.cpu().numpy()[:, 1:] == 1)),
                             "final_position_error_vs_fp64_median": float(np.median(perr_a)),
                             "final_position_error_vs_fp64_p99": float(np.percentile(perr_a, 99))}},
    }
    if not args.no_cpu_baseline:
        from oracle import Oracle
        from oracle.oracle import host_threads

        ns = min(args.stream_cpu_streams, S)
        fast = Oracle("fast")
        nth = host_threads()
        nbody_w = orbit[:ns].cpu().numpy()
        sw_host = sw0[:ns].cpu().numpy()
        t0 = time.perf_counter()
        cpu_out, _, cpu_status, _ = fast.mockstream_systems(pot, bodies[:ns], nbody_w, t, 2 * counts, sw_host,
                                                            t_final, 1.0, nthreads=nth)
        cpu_s = time.perf_counter() - t0
        gpu_o = out[:ns].cpu().numpy()
        gpu_st = st_k[:ns].cpu().numpy()
        ok = np.repeat((gpu_st == 1) & (cpu_status == 1), 2, axis=1)
        pe = np.linalg.norm(gpu_o[..., :3] - cpu_out[..., :3], axis=-1)[ok]
        result["cpu_baseline"] = {
            "value": ns * float(np.sum(np.round(t_final - res.release_time))) / cpu_s,
            "unit": "particle-steps/s", "cores": nth, "kind": "port",
            "sample": f"release systems of {ns} of the {S} streams, gala's dop853_step loop restated in C, -Ofast",
            "status_agreement": float(np.mean(gpu_st == cpu_status)),
            "position_diff_kpc_p99": float(np.percentile(pe, 99)) if pe.size else None,
        }
        # the animate mode's CPU baseline: gala's interval loop restated in C, one
        # stream per host thread (ctypes releases the GIL), a bounded sample of streams
        from concurrent.futures import ThreadPoolExecutor

        na_cpu = min(sa, nth)
        bodies_np = bodies[:na_cpu]
        nb0_np, sw_np, t_np = nb0_a[:na_cpu].cpu().numpy(), sw_a[:na_cpu].cpu().numpy(), t[:na]

        def one(k):
            return fast.mockstream_animate(pot, bodies_np[k], nb0_np[k], t_np, sw_np[k], 2 * counts[:na],
                                           output_every=10)

        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=nth) as ex:
            outs = list(ex.map(one, range(na_cpu)))
        cpu_anim_s = time.perf_counter() - t0
        w_gpu = w_a[:na_cpu].cpu().numpy()
        diff = max(float(np.abs(w_gpu[k] - outs[k][2]).max() / np.abs(outs[k][2]).max()) for k in range(na_cpu))
        result["animate"]["cpu_baseline"] = {
            "value": na_cpu * float(live.sum()) / cpu_anim_s, "unit": "particle-steps/s", "cores": nth,
            "kind": "port", "sample": f"{na_cpu} of the {sa} streams, gala's mockstream_dop853_animate loop "
                                      "restated in C, -Ofast, one stream per thread",
            "gpu_vs_cpu_max_rel": diff}
    return result


# --------------------------------------------------------------------------
# Variant: orbit reductions (peri / apo / zmax)
# --------------------------------------------------------------------------
def run_orbit_reductions(args, torch, stream):
    """Pericentre, apocentre and z-maximum statistics (gala's Orbit.pericenter /
    apocenter / zmax) over 100,000 MW-composite orbits x 2,001 Leapfrog
    snapshots (9.6 GB resident in HBM), one fused pass reading x, y, z.  L2
    flushed before each timed pass.  CPU baseline: gala's numpy algorithm."""
    from gala_gb300 import _abi
    from gala_gb300 import workloads as W
    from gala_gb300._device import ptr

    n, nsteps = args.reduce_orbits, args.reduce_nsteps
    mw = W.mw_composite()
    w0 = W.mw_ics(n, seed=W.SEED_BASE + 7)
    orbit = mw.integrate_orbit(w0, dt=1.0, n_steps=nsteps, Integrator="leapfrog", return_device=True)
    wd = orbit.w_device.contiguous()
    td = torch.from_numpy(np.ascontiguousarray(orbit.t)).cuda()
    nt = int(wd.shape[1])
    count = torch.zeros((3, n), dtype=torch.int32, device="cuda")
    sm, mn, mx = (torch.zeros((3, n), dtype=torch.float64, device="cuda") for _ in range(3))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def call():
        _abi.call("gx_orbit_extrema", ptr(wd), ptr(td), nt, n, 0, 0, ptr(count), ptr(sm), ptr(mn), ptr(mx), None,
                  None, int(stream.cuda_stream))

    for _ in range(3):
        call()
    times = []
    for _ in range(5):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    algo_bytes = 3 * nt * n * 8 + nt * 8 + 3 * n * (4 + 3 * 8)
    hbm, hbm_src = measured_peak("hbm_gbs", 6800.0)
    res = {
        "workload": f"orbit_reductions: {n} MW orbits x {nt} Leapfrog snapshots, peri/apo/zmax in one pass",
        "value": n * nt / (ms * 1e-3), "unit": "orbit-snapshots/s", "ms": ms,
        "roofline": {"bound": "hbm", "achieved": algo_bytes / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": algo_bytes / (ms * 1e-3) / 1e9 / hbm, "bytes_per_launch": algo_bytes,
                     "peak_source": hbm_src},
    }
    if not args.no_cpu_baseline:
        from oracle import orbit_oracle as OO

        ns = 200
        wh = wd[:, :, :ns].cpu().numpy()
        t0 = time.perf_counter()
        ref = np.stack([OO.reduce(wh, orbit.t, k) for k in ("peri", "apo", "zmax")])
        cpu_s = time.perf_counter() - t0
        gpu_mean = (sm / count)[:, :ns].cpu().numpy()
        res["cpu_baseline"] = {"value": ns * nt / cpu_s, "unit": "orbit-snapshots/s", "cores": 1, "kind": "port",
                               "sample": f"{ns} orbits, gala's _max_helper (scipy argrelmax + numpy polyfit)",
                               "gpu_vs_cpu_max_rel": float(np.nanmax(np.abs(gpu_mean - ref) / np.abs(ref)))}
    return res


# --------------------------------------------------------------------------
# Compact summaries of the variants (the JSON line stays short)
# --------------------------------------------------------------------------
def compact(name, r):
    cb = r.get("cpu_baseline", {})
    if name == "mw_dop853":
        f = r["fp32"]
        return {"value": sig(r["value"]), "e2e": sig(r["e2e"]["value"]), "frac_fp64": sig(r["roofline"]["frac"], 3),
                "dE_over_E_median": sig(r["dE_over_E_median"], 2), "cpu_16c": sig(cb.get("value")),
                "gpu_vs_cpu_max_rel": sig(cb.get("gpu_vs_cpu_max_rel"), 2),
                "fp32_rtol1e-8": {"value": sig(f["value"]), "speedup": sig(f["speedup_vs_fp64"], 3),
                                  "frac_fp32": sig(f["roofline"]["frac"], 3),
                                  "pos_err_median": sig(f["position_error_vs_fp64_median"], 2),
                                  "pos_err_p99": sig(f["position_error_vs_fp64_p99"], 2),
                                  "dE_median": sig(f["dE_over_E_median"], 2)}}
    if name == "hernquist_leapfrog":
        return {"value": sig(r["value"]), "hbm_gbs": sig(r["roofline"]["achieved"]),
                "frac_hbm": sig(r["roofline"]["frac"], 3), "e2e": sig(r["e2e"]["value"]), "cpu": sig(cb.get("value")),
                "gpu_vs_cpu_max_rel": sig(cb.get("gpu_vs_cpu_max_rel"), 2)}
    if name == "scf_surrogate":
        o = r["orbits_vs_fp64_2048x1000"]
        t = r["equal_accuracy_analytic"] or {}
        return {"surrogate": sig(r["surrogate"]["value"]), "operands": r["surrogate"]["operands"],
                "fp32_analytic": sig(r["fp32_analytic"]["value"]), "fp64_plain": sig(r["fp64_analytic_plain"]["value"]),
                "force_err_median": sig(r["force_error"]["median"], 2),
                "sur_pos_err_median": sig(o["surrogate"]["position_error_median"], 2),
                "sur_dE_vs_fp64_median": sig(o["surrogate"]["dE_over_E_vs_fp64_median"], 2),
                "fp32_pos_err_median": sig(o["fp32_analytic"]["position_error_median"], 2),
                "fp32_dE_vs_fp64_median": sig(o["fp32_analytic"]["dE_over_E_vs_fp64_median"], 2),
                "equal_acc_lmax": t.get("lmax"), "speedup_at_equal_accuracy": sig(r["speedup_at_equal_accuracy"], 3),
                "frac_tensor": sig(r["surrogate"]["roofline"]["frac"], 3)}
    if name == "mock_streams":
        return {"unit": "particle-steps/s", "pipeline": sig(r["pipeline"]["value"]),
                "release_kernel": sig(r["release_kernel"]["value"]),
                "frac_fp64": sig(r["release_kernel"]["roofline"]["frac"], 3), "e2e": sig(r["e2e"]["value"]),
                "release_fp32": sig(r["release_kernel_fp32"]["value"]),
                "release_fp32_pos_err_median": sig(r["release_kernel_fp32"]["position_error_vs_fp64_median"], 2),
                "leapfrog_fp32c": sig(r["leapfrog_fp32c"]["value"]), "cpu_16c": sig(cb.get("value")),
                "status_agreement": sig(cb.get("status_agreement"), 5),
                "animate": sig(r["animate"]["value"]), "animate_fp32": sig(r["animate"]["fp32"]["value"]),
                "animate_fp32_pos_err_median": sig(r["animate"]["fp32"]["final_position_error_vs_fp64_median"], 2),
                "animate_cpu": sig(r["animate"].get("cpu_baseline", {}).get("value")),
                "animate_vs_cpu_max_rel": sig(r["animate"].get("cpu_baseline", {}).get("gpu_vs_cpu_max_rel"), 2)}
    if name == "orbit_reductions":
        return {"unit": "orbit-snapshots/s", "value": sig(r["value"]), "frac_hbm": sig(r["roofline"]["frac"], 3),
                "cpu_1c": sig(cb.get("value"))}
    return r


VARIANTS = {"mw_dop853": None, "hernquist_leapfrog": run_hernquist_leapfrog, "scf_surrogate": run_scf_surrogate,
            "mock_streams": run_mock_streams, "orbit_reductions": run_orbit_reductions}


def run_gx(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import gala_gb300 as g

    g.load_library()
    stream = torch.cuda.current_stream()

    if args.workload != "all":
        if args.workload == "uneven_batch":
            res = run_uneven_batch(args, torch, stream, args.steps, args.warmup)
        elif args.workload == "mw_dop853":
            res = run_mw_dop853(args, torch, stream, args.dop_reps, 1)
        elif args.workload == "mw_dop853_fp32":
            from gala_gb300 import workloads as W

            t = g.parse_time_specification(dt=0.5, n_steps=args.nsteps)
            w0d = torch.from_numpy(W.mw_ics(args.orbits, seed=W.SEED_BASE + 2)).cuda()
            td = torch.from_numpy(t).cuda()
            flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
            res = run_dop853_fp32(args, torch, stream, W.mw_composite(), w0d, td, len(t), 100, args.orbits, flush)
        else:
            res = VARIANTS[args.workload](args, torch, stream)
        if rank == 0:
            print(json.dumps(res), flush=True)
        return

    # ---- headline: the uneven batch, FP32 compensated against plain FP64
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    head = run_uneven_batch(args, torch, stream, args.steps, args.warmup, world=world, clocks=clocks)
    f32, f64 = head["fp32c"], head.get("fp64", {})
    details = {"uneven_batch": head}
    variants = {}
    skip = {s for s in args.skip.split(",") if s}
    for name, fn in VARIANTS.items():
        if name in skip:
            continue
        if name == "mw_dop853":
            r = run_mw_dop853(args, torch, stream, args.dop_reps, 1, world, rank)
        elif world > 1:
            continue   # the other variants are single-GPU workloads
        else:
            r = fn(args, torch, stream)
        details[name] = r
        variants[name] = compact(name, r)
    if args.detail and rank == 0:
        Path(args.detail).write_text(json.dumps(details, indent=1))
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    pe = head.get("position_error_vs_fp64", {})
    line = {
        "metric": METRIC,
        "value": f32["value"],
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": f32["ms"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded ICs, no dataset)",
        "config": {
            "workload": head["workload"],
            "orbits_per_gpu": head["orbits"], "orbit_steps_per_gpu": head["orbit_steps"],
            "form": "FP32 force, Kahan-compensated FP32 state, FP64 in/out and energy",
            "plain_fp64_value": sig(f64.get("value")),
            "speedup_vs_plain_fp64": sig(head.get("speedup_fp32c_vs_fp64")),
            "dE_over_E_median": sig(f32["dE_over_E_median"], 3),
            "dE_over_E_p99": sig(f32["dE_over_E_p99"], 3),
            "position_error_vs_fp64_median": sig(pe.get("median"), 3),
            "position_error_vs_fp64_p99": sig(pe.get("p99"), 3),
            "position_error_vs_fp64_max": sig(pe.get("max"), 3),
            "orbits_within_1e-4": sig(pe.get("frac_le_1e-4"), 5),
            "launch": f32["config"],
            "l2": "flushed (256 MB write) between timed iterations",
        },
        "e2e": {k: (sig(v) if isinstance(v, float) else v) for k, v in head["e2e"].items()},
        "gpu_launches": 3 * args.steps,
        "roofline": {**{k: sig(v, 4) for k, v in f32["roofline"].items()},
                     "kernel": "batch_fp32_kernel, CUDA events",
                     "peak_source": "FP32 FMA-chain probe, same run",
                     "work": "flops/step: Leapfrog 102, Ruth4 306 (3 gradients)"},
        "clocks": clocks.summary(),
        "wall_s_timed_region": sig(head.get("wall_s_timed_region")),
        "variants": variants,
    }
    if "cpu_baseline" in head:
        line["cpu_baseline"] = {k: sig(v) if isinstance(v, float) else v for k, v in head["cpu_baseline"].items()}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gx(args)


if __name__ == "__main__":
    main()
