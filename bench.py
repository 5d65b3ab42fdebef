"""Benchmark: vesicle-steps/s of the implicit BIEM step on GB300.

Workload (the BIEM arm of the nv=4096, N=128 MLARM-vs-BIEM comparison): 4096
vesicles of 128 points, reduced area 0.65, area pi, k=2..8 radius
perturbations, random rotations, centres uniform in a square sized for 15%
area fraction (min gap 0.05, seed 0); shear flow of rate 2, dt=1e-5, kappa=1,
GMRES tol 1e-10 (restart 20), block-diagonal LU preconditioner, reference
(py_hh) near-field scheme, FP32-compensated all-pairs sum and Alpert matrix.
One step = one TStepBiem.time_step (geometry, Alpert matrix, near lists,
preconditioner, GMRES).  Synthetic seeded data stands in for the reference
drivers' missing initial-condition files.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vesicle-steps/sec at nv=4096 N=128: MLARM vs plain BIEM, ≤1e-2 vel err"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nv", type=int, default=4096)
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--area-fraction", type=float, default=0.15)
    ap.add_argument("--near", default="py_hh")
    ap.add_argument("--precision", default="fp32c")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def workload(nv, N, phi, seed=0):
    from ves2dpy_gb300.suspension import random_suspension
    return random_suspension(nv, N, phi, min_gap=0.05, seed=seed)


STEP = dict(dt=1e-5, kappa=1.0, gmresTol=1e-10, gmresMaxIter=200, farFieldSpeed=2.0, chanWidth=2.5, vortexSize=2.5)


# ---------------------------------------------------------------------------
# CPU reference leg: the oracle's all-pairs sum (the dominant cost of the
# reference step) timed on a bounded sample on every host core, extrapolated
# to the pairs one step evaluates.
def _cpu_worker(args):
    import numpy as np
    Xup, sa, fup, tar, nsrc_vesicles = args
    from oracle import ves2d_oracle as O
    t0 = time.perf_counter()
    O.all_exact_stokes_sl_target(Xup, sa, fup, tar, None)
    return time.perf_counter() - t0, tar.shape[0] // 2 * (Xup.shape[0] // 2) * (Xup.shape[1] - 1)


def cpu_pair_rate(N, seconds, cores=None):
    """Pairs/s of the oracle far field on ``cores`` processes (spawned)."""
    import multiprocessing as mp
    import numpy as np
    from oracle import ves2d_oracle as O
    cores = cores or os.cpu_count() or 1
    tab = O.PotenTables(N)
    X = workload(64, N, 0.15, seed=1)
    rng = np.random.default_rng(0)
    f = rng.normal(size=X.shape)
    Xup = O.interpft_vec(X, tab.Nup)
    fup = O.interpft_vec(f, tab.Nup)
    sa = O.diff_prop(Xup)[0]
    # one task = one target vesicle against nsv source vesicles
    nsv = 16 if N >= 128 else 64
    task = (Xup[:, :nsv + 1], sa[:, :nsv + 1], fup[:, :nsv + 1], X[:, :1], nsv)
    t1, p1 = _cpu_worker(task)  # calibrate in-process
    reps = max(1, int(seconds / max(t1, 1e-3)))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [task] * (reps * cores))
    wall = time.perf_counter() - t0
    pairs = sum(p for _, p in res)
    return pairs / wall, cores, f"{reps * cores} x (1 target vesicle vs {nsv} source vesicles, N={N}, Nup={tab.Nup})"


def pairs_per_eval(nv, N):
    Nup = N * math.ceil(math.sqrt(N))
    return float(nv) * (nv - 1) * N * Nup


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.proc = None
        self.index = index
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit())
        mx = max((float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def run_gb300(a, rank, world):
    import numpy as np
    import torch
    from ves2dpy_gb300 import _native as nat
    from ves2dpy_gb300.layout import to_vm
    from ves2dpy_gb300.tstep_biem import TStepBiem

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    X0 = workload(a.nv, a.N, a.area_fraction, seed=rank)
    N, nv = a.N, a.nv
    options = dict(farField="shear", usePreco=True, repulsion=False)
    prams = dict(STEP, viscCont=[1.0] * nv)
    Xd = torch.tensor(X0, dtype=torch.float64, device=dev)
    tt = TStepBiem(Xd, None, options, prams, near=a.near, farfield_precision=a.precision,
                   sl_precision=a.precision)
    ctx = nat.context(N, dev)
    ws = ctx.workspace(tt.workspace_bytes())
    Xv = to_vm(Xd)
    sv = torch.zeros(nv, N, dtype=torch.float64, device=dev)
    Xo, so = torch.empty_like(Xv), torch.empty_like(sv)

    from ves2dpy_gb300.replicas import barrier

    mv = []
    for _ in range(a.warmup):
        Xo, so, res = tt.step_device(Xv, sv, Xo, so, ws)
        Xv, Xo, sv, so = Xo, Xv, so, sv
    torch.cuda.synchronize()
    ctx.set_timing(True)
    ctx.stats(reset=True)
    l0 = ctx.stats().kernel_launches
    barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(dev.index) as clk:
        e0.record(stream)
        for _ in range(a.steps):
            Xo, so, res = tt.step_device(Xv, sv, Xo, so, ws)
            mv.append(res.matvecs)
            Xv, Xo, sv, so = Xo, Xv, so, sv
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    st = ctx.stats(reset=True)
    ctx.set_timing(False)
    launches = st.kernel_launches - l0
    from ves2dpy_gb300.replicas import aggregate
    t_max, value = aggregate(ms, float(nv * a.steps), dev)
    ms_per_step = t_max / a.steps

    # end to end through the public API with pinned host buffers
    Xh = torch.from_numpy(X0).pin_memory()
    sh = torch.zeros(N, nv, dtype=torch.float64).pin_memory()
    Xback = torch.empty_like(Xh).pin_memory()
    sback = torch.empty_like(sh).pin_memory()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.e2e_steps):
        Xdd = Xh.to(dev, non_blocking=True)
        sdd = sh.to(dev, non_blocking=True)
        Xn, sn, _, _, it, iflag = tt.time_step(Xdd, sdd)
        Xback.copy_(Xn, non_blocking=True)
        sback.copy_(sn, non_blocking=True)
        torch.cuda.synchronize()
        Xh, Xback = Xback, Xh
        sh, sback = sback, sh
    e2e_s = (time.perf_counter() - t0) / a.e2e_steps
    bytes_io = Xh.numel() * 8 + sh.numel() * 8

    out = None
    if rank == 0:
        sfu_peak = nat.probe_sfu_peak(dev)
        ff_ms = st.farfield_ms / max(st.farfield_launches, 1)
        ff_pairs = st.farfield_pairs / max(st.farfield_launches, 1)
        mufu_rate = 2.0 * ff_pairs / (ff_ms * 1e-3) if ff_ms > 0 else 0.0
        clocks = clk.summary()
        out = {
            "metric": METRIC,
            "value": value,
            "unit": "vesicle-steps/s",
            "n_gpus": world,
            "steps": a.steps,
            "warmup": a.warmup,
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64 (solve, spectral, near field) + f32 compensated (all-pairs sum, Alpert kernel)",
            "data": "synthetic (seeded suspension generator; no reference initial conditions exist)",
            "config": {"workload": f"plain BIEM implicit step (TStepBiem.time_step), nv={nv}, N={N}, "
                                   f"Nup={ctx.Nup}, area fraction {a.area_fraction}, shear rate 2, dt=1e-5, "
                                   "GMRES tol 1e-10",
                       "stepper": "biem", "mlarm": "not built (no trained networks)",
                       "near_scheme": a.near, "precision": a.precision,
                       "matvecs_per_step": mv, "l2": "inputs larger than L2 (G 2.1 GB, LU 4.8 GB per step)",
                       "parallelism": "replicas only" if world > 1 else "single GPU"},
            "e2e": {"value": world * nv / e2e_s, "unit": "vesicle-steps/s", "h2d_bytes_per_step": bytes_io,
                    "d2h_bytes_per_step": bytes_io},
            "gpu_launches": int(launches),
            "roofline": {"bound": "sfu", "kernel": "ff_main_kernel<float> (all-pairs Stokeslet sum)",
                         "achieved": mufu_rate / 1e9, "peak": sfu_peak / 1e9, "unit": "Gop/s (MUFU lg2+rcp)",
                         "frac": mufu_rate / sfu_peak if sfu_peak else None, "traffic": None,
                         "traffic_note": "compute-bound; ncu measured 6.7 MB DRAM per launch at nv=256 "
                                         "(sources L2-resident), see profiles/ff_main_kernel_nv256_N128_full.md",
                         "pairs_per_launch": ff_pairs, "ms_per_launch": ff_ms,
                         "gpairs_per_s": ff_pairs / (ff_ms * 1e-3) / 1e9 if ff_ms > 0 else None,
                         "peak_source": "measured by ves_probe_sfu_peak on this GPU",
                         "share_of_step": st.farfield_ms / t_max if t_max else None},
            "clocks": clocks,
        }
    return out


def run_cpu_reference(a, rank):
    """--impl reference: the oracle port of the reference path on host cores."""
    if rank != 0:
        return None
    rate, cores, sample = cpu_pair_rate(a.N, a.cpu_sample_seconds)
    mv = 8  # matvecs per step measured for this workload on the GPU arm (tol 1e-10)
    step_s = mv * pairs_per_eval(a.nv, a.N) / rate
    v = a.nv / step_s
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "vesicle-steps/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"plain BIEM implicit step, nv={a.nv}, N={a.N} (CPU oracle, extrapolated)"},
            "cpu_baseline": {"value": v, "unit": "vesicle-steps/s", "cores": cores, "kind": "port",
                             "sample": sample + f"; extrapolated to {mv} all-pairs evaluations of "
                                                f"{pairs_per_eval(a.nv, a.N):.3e} pairs per step"},
            "e2e": {"value": v, "unit": "vesicle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    a = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if a.impl == "reference":
        out = run_cpu_reference(a, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    out = run_gb300(a, rank, world)
    if rank == 0 and out is not None:
        if not a.no_cpu_baseline:
            rate, cores, sample = cpu_pair_rate(a.N, a.cpu_sample_seconds)
            mv = out["config"]["matvecs_per_step"]
            mean_mv = sum(mv) / len(mv)
            step_s = mean_mv * pairs_per_eval(a.nv, a.N) / rate
            out["cpu_baseline"] = {"value": a.nv / step_s, "unit": "vesicle-steps/s", "cores": cores,
                                   "kind": "port",
                                   "sample": sample + f"; extrapolated to {mean_mv:.1f} all-pairs evaluations "
                                                      f"of {pairs_per_eval(a.nv, a.N):.3e} pairs per step"}
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
