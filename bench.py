"""Benchmark: vesicle-steps/s of the MLARM surrogate step against the plain
BIEM step, nv=4096 vesicles of N=128 points, on one GB300.

Workload (the MLARM-vs-BIEM configuration): 4096 vesicles of reduced area
0.65 and unit length (area 0.65/(4 pi)), k=2..8 radius perturbations, random
rotations, centres uniform in a square sized for 15% area fraction (min gap
0.0064, i.e. 0.05 scaled to unit length; seed 0); shear flow of rate 2,
dt=1e-5, kappa=1.

* MLARM step (the headline ``value``): MLARM_manyfree_py.time_step_many_noinfo
  with the five networks on the tensor cores (BF16 operands, FP32
  accumulation), two FP32-compensated all-pairs sums over Nup=1536 upsampled
  points, FP64 geometry and post-step conditioning.  The networks carry
  seeded synthetic weights of the reference architectures (the trained
  weights are not part of the reference tree).
* Plain BIEM step, same suspension: TStepBiem.time_step (GMRES tol 1e-8, the
  accuracy floor of the FP32-compensated all-pairs operator here,
  block-diagonal LU preconditioner, reference near scheme, FP32-compensated
  all-pairs sum and Alpert matrix).

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
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vesicle-steps/sec at nv=4096 N=128: MLARM vs plain BIEM, ≤1e-2 vel err"
UNIT_AREA = 0.65 / (4 * math.pi)   # reduced area 0.65 at unit length
MIN_GAP = 0.05 / 7.79              # the 0.05 gap of radius-1 vesicles (length 7.79) at unit length


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nv", type=int, default=4096)
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--area-fraction", type=float, default=0.15)
    ap.add_argument("--nets", default="bf16", choices=["bf16", "fp32"])
    ap.add_argument("--precision", default="fp32m", choices=["fp32m", "fp32c", "fp64"],
                    help="all-pairs sums: fp32m (multipole for separated vesicle pairs), fp32c (direct), fp64")
    ap.add_argument("--biem-steps", type=int, default=1)
    ap.add_argument("--biem-warmup", type=int, default=0)
    ap.add_argument("--biem-tol", type=float, default=1e-8)
    ap.add_argument("--no-biem", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=-1,
                    help="steps of the end-to-end leg (default: the same number as the timed steps)")
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-net-timing", action="store_true", help="skip the per-network forward timings")
    ap.add_argument("--no-autotune", action="store_true",
                    help="fixed launch shapes for the network kernels (no timing of the shapes on the first step)")
    ap.add_argument("--only-net", default=None, help="time one network's forward pass at --nv and exit "
                    "(relax, adv, near, selften, advten)")
    ap.add_argument("--synthetic-weights", action="store_true",
                    help="seeded synthetic networks instead of the trained ones in ves2dpy_gb300/trained")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="after the timed steps, continue the MLARM trajectory this many steps and compare with the "
                         "BIEM step every --accuracy-every steps (velocity error, drift)")
    ap.add_argument("--accuracy-every", type=int, default=25)
    ap.add_argument("--conserve", action="store_true",
                    help="MLARM option: advection and relaxation displacements area- and length-preserving to first "
                         "order")
    ap.add_argument("--area-len-tol", type=float, default=0.0,
                    help="tolerance of the MLARM step's area/length correction (0: the reference's 1e-2)")
    ap.add_argument("--judge-tol", type=float, default=0.0,
                    help="> 0: the BIEM step judges each vesicle's surrogate step and stands in where it moved the "
                         "area or length by more than this (relative)")
    ap.add_argument("--biem-precond", default="fp32", choices=["fp32", "fp64"],
                    help="precision of the BIEM step's block-diagonal preconditioner (GMRES solves the FP64 system)")
    return ap.parse_args()


def workload(nv, N, phi, seed=0):
    from ves2dpy_gb300.suspension import random_suspension
    return random_suspension(nv, N, phi, min_gap=MIN_GAP, area=UNIT_AREA, seed=seed)


STEP = dict(dt=1e-5, kappa=1.0, gmresTol=1e-10, gmresMaxIter=200, farFieldSpeed=2.0, chanWidth=2.5, vortexSize=2.5)


def net_flops(spec):
    """Multiply-adds x 2 of one vesicle through a network (the useful work)."""
    L, G, f = spec.L, spec.rep, 0
    for b in spec.blocks:
        d = 2 * b.c2
        f += 2 * (L // 2) * b.c1 * b.cin * 7            # conv pair 1
        f += 2 * (L // 4) * b.c2 * 2 * b.c1 * 7         # conv pair 2
        f += (L // 2) * d * d * 5 + L * d * d * 5        # transposed convs (5 taps per output)
        f += L * b.cmix * d * 3                          # mix
    return 2.0 * f * G


# ---------------------------------------------------------------------------
# CPU legs (oracle port of the reference algorithm on the host cores)
def _cpu_worker(args):
    Xup, sa, fup, tar, nsrc_vesicles = args
    from oracle import ves2d_oracle as O
    t0 = time.perf_counter()
    O.all_exact_stokes_sl_target(Xup, sa, fup, tar, None)
    return time.perf_counter() - t0, tar.shape[0] // 2 * (Xup.shape[0] // 2) * (Xup.shape[1] - 1)


def cpu_pair_rate(N, seconds, cores=None):
    """Pairs/s of the oracle all-pairs sum on ``cores`` spawned processes."""
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
    nsv = 16 if N >= 128 else 64
    task = (Xup[:, :nsv + 1], sa[:, :nsv + 1], fup[:, :nsv + 1], X[:, :1], nsv)
    t1, _ = _cpu_worker(task)
    reps = max(1, int(seconds / max(t1, 1e-3)))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [task] * (reps * cores))
    wall = time.perf_counter() - t0
    pairs = sum(p for _, p in res)
    return pairs / wall, cores, f"{reps * cores} x (1 target vesicle vs {nsv} source vesicles, N={N}, Nup={tab.Nup})"


def cpu_net_seconds(state_dicts, cores):
    """Seconds of the five networks for one vesicle in FP32 (the reference
    networks' precision) with torch on ``cores`` host threads."""
    import numpy as np
    import torch
    from oracle import mlarm_oracle as M
    from ves2dpy_gb300.mlarm_weights import NETS, net_test_input
    torch.set_num_threads(cores)
    M.net_forward(NETS["relax"], state_dicts["relax"], net_test_input("relax"), dtype=np.float32)
    t0 = time.perf_counter()
    for n in NETS:
        M.net_forward(NETS[n], state_dicts[n], net_test_input(n), dtype=np.float32)
    return time.perf_counter() - t0


def pairs_per_eval(nv, N):
    Nup = N * math.ceil(math.sqrt(N))
    return float(nv) * (nv - 1) * N * Nup


def cpu_estimates(a, state_dicts, biem_matvecs):
    """MLARM and BIEM vesicle-steps/s of the CPU oracle port, from a bounded
    sample: the all-pairs rate (spawned processes on all cores) extrapolated
    to the step's all-pairs evaluations, plus the networks of one vesicle
    (FP32 torch) times nv."""
    rate, cores, sample = cpu_pair_rate(a.N, a.cpu_sample_seconds)
    net_s = cpu_net_seconds(state_dicts, cores) if state_dicts is not None else float("nan")
    ppe = pairs_per_eval(a.nv, a.N)
    mlarm_s = 2 * ppe / rate + a.nv * net_s
    out = {"value": a.nv / mlarm_s, "unit": "vesicle-steps/s", "cores": cores, "kind": "port",
           "sample": f"{sample}; all-pairs rate {rate:.3e} pairs/s extrapolated to 2 evaluations of {ppe:.3e} "
                     f"pairs, plus the five networks of one vesicle in FP32 torch ({net_s:.3f} s) times nv"}
    if biem_matvecs:
        mv = sum(biem_matvecs) / len(biem_matvecs)
        out["biem_value"] = a.nv / (mv * ppe / rate)
        out["biem_note"] = f"{mv:.1f} all-pairs evaluations per BIEM step (the GPU arm's GMRES count)"
    return out


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region (raw samples written to
    $VES_CLOCKS_DIR, default the system temporary directory)."""

    def __init__(self, index=0):
        self.proc = None
        self.index = index
        self.path = os.path.join(os.environ.get("VES_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"clocks_{os.getpid()}.csv")

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


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def prepare_initial(X):
    """The reference MLARM driver's preparation of the initial shapes
    (entry_driver_manyfreeSpaceVesicle_N128.py:157-167): the reference area
    and length first, then up to 10 equal-arclength passes.  Returns
    (X, area0, len0)."""
    from ves2dpy_gb300.curve import Curve
    cv = Curve()
    _, area0, len0 = cv.geomProp(X)
    for _ in range(10):
        X, good = cv.redistributeArcLength(X)
        if good:
            break
    return X, area0, len0


def networks(a):
    """(state dicts, normalisation arrays, description): the trained networks
    of ves2dpy_gb300/trained (ves2dpy_gb300.train_surrogate) unless
    --synthetic-weights or none are present."""
    from ves2dpy_gb300 import training as TR
    from ves2dpy_gb300.mlarm_weights import NETS, synthetic_norms, synthetic_state_dict
    if not a.synthetic_weights and TR.have_trained():
        sds, norms = TR.load()
        log = {}
        try:
            log = json.load(open(os.path.join(TR.TRAINED_DIR, "train_log.json")))
        except Exception:
            pass
        val = {k: v.get("validation_rel_error") for k, v in log.get("nets", {}).items()}
        return sds, norms, {"weights": "trained on BIEM-generated data (ves2dpy_gb300/trained)",
                            "validation_rel_error_vs_biem": val, "training_shapes": log.get("shapes")}
    return ({n: synthetic_state_dict(n, 0) for n in NETS}, synthetic_norms(0),
            {"weights": "seeded synthetic (untrained)"})


def run_mlarm(a, dev, X0, state_dicts, norms=None):
    """Timed MLARM steps on the device (inputs resident), then one end-to-end
    step through MLARM_manyfree_py with pinned host buffers."""
    import numpy as np
    import torch
    from ves2dpy_gb300 import _native as nat
    from ves2dpy_gb300.curve import Curve
    from ves2dpy_gb300.mlarm import MLARM_manyfree_py
    from ves2dpy_gb300.mlarm_weights import NETS, synthetic_norms
    from ves2dpy_gb300.replicas import barrier

    N, nv = a.N, a.nv
    nrm = {k: torch.from_numpy(np.asarray(v, dtype=np.float64)) for k, v in (norms or synthetic_norms(0)).items()}

    def vinf(X):  # shear, rate 2 (entry_driver_manyfreeSpaceVesicle_N128.py:53)
        n = X.shape[0] // 2
        return 2.0 * torch.vstack((X[n:], torch.zeros_like(X[:n])))

    m = MLARM_manyfree_py(STEP["dt"], vinf, Curve(), False, 1e2, -1, nrm["adv_in"], nrm["adv_out"],
                          nrm["relax_in"], nrm["relax_out"], nrm["near_in"], nrm["near_out"], nrm["selften_in"],
                          nrm["selften_out"], nrm["advten_in"], nrm["advten_out"], dev, state_dicts=state_dicts,
                          net_precision=a.nets, farfield_precision=a.precision, autotune=not a.no_autotune,
                          judge_tol=a.judge_tol, conserve=a.conserve, area_len_tol=a.area_len_tol)
    Xd = torch.tensor(X0, dtype=torch.float64, device=dev)
    Xd, area0, len0 = prepare_initial(Xd)
    m.area0, m.len0 = area0, len0
    ten = torch.zeros(N, nv, dtype=torch.float64, device=dev)
    X, t = Xd, ten
    for _ in range(a.warmup):
        X, t = m.time_step_many_noinfo(X, t, 3)
    torch.cuda.synchronize()
    # the state the timed steps start from, kept on the host for the e2e leg
    Xw = X.detach().cpu().pin_memory()
    tw = t.detach().cpu().pin_memory()
    ctx = nat.context(N, dev)
    ctx.set_timing(True)
    ctx.stats(reset=True)
    l0 = ctx.stats().kernel_launches
    barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = _events()
    nfb = 0
    with Clocks(dev.index) as clk:
        e0.record(stream)
        for _ in range(a.steps):
            X, t = m.time_step_many_noinfo(X, t, 3)
            nfb += m.last_result.n_fallback
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    st = ctx.stats(reset=True)
    ctx.set_timing(False)
    launches = st.kernel_launches - l0
    near_pairs = m.last_result.n_near_pairs
    _, a1, l1 = Curve().geomProp(X)
    drift = max(float(((a1 - area0).abs() / area0).max()), float(((l1 - len0).abs() / len0).max()))

    # networks alone at this nv (forward passes on the step's own input sizes)
    net_ms = {}
    for n, net in ({} if a.no_net_timing else m.nets).items():
        spec = NETS[n]
        x = torch.randn(nv, spec.rep * spec.cin, spec.L, device=dev, dtype=net.dtype)
        net(x)
        b0, b1 = _events()
        torch.cuda.synchronize()
        b0.record(stream)
        net(x)
        b1.record(stream)
        torch.cuda.synchronize()
        net_ms[n] = b0.elapsed_time(b1)
        del x

    # end to end through the public API: the same timed steps again, from the
    # same state, each step's input copied from pinned host memory to the
    # device and its result (shape and tension) copied back
    Xh, th = Xw.clone().pin_memory(), tw.clone().pin_memory()
    Xback, tback = torch.empty_like(Xh).pin_memory(), torch.empty_like(th).pin_memory()
    e2e_steps = a.steps if a.e2e_steps < 0 else a.e2e_steps
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        Xn, tn = m.time_step_many_noinfo(Xh.to(dev, non_blocking=True), th.to(dev, non_blocking=True), 3)
        Xback.copy_(Xn, non_blocking=True)
        tback.copy_(tn, non_blocking=True)
        torch.cuda.synchronize()
        Xh, Xback = Xback, Xh
        th, tback = tback, th
    e2e_s = (time.perf_counter() - t0) / e2e_steps if e2e_steps > 0 else None
    io = Xh.numel() * 8 + th.numel() * 8
    # one step from the timed steps' starting state: the surrogate velocity
    # the accuracy check compares with the BIEM step's from the same state
    Xs1, _ = m.time_step_many_noinfo(Xw.to(dev), tw.to(dev), 3)
    # the BIEM operators as the judge of each network on that state (512 vesicles)
    from ves2dpy_gb300 import training as TR
    from ves2dpy_gb300.layout import to_vm
    sub = to_vm(Xw.to(dev))[: min(nv, 512)].contiguous()
    judge = TR.surrogate_errors(m.nets, norms or synthetic_norms(0), TR.standardize(sub))
    accuracy = accuracy_leg(a, dev, m, X, t, area0, len0) if a.accuracy_steps > 0 else None
    return dict(ms=ms, stats=st, launches=launches, clocks=clk.summary(), net_ms=net_ms, e2e_s=e2e_s, io=io,
                e2e_steps=e2e_steps, drift=drift, near_pairs=near_pairs, Xw=Xw.numpy().copy(), tw=tw,
                X1=Xs1.cpu(), nets=m.nets, fallbacks=nfb, judge=judge, accuracy=accuracy)


def accuracy_leg(a, dev, m, X, t, area0, len0):
    """The MLARM trajectory continued from the timed steps' end for
    --accuracy-steps steps; every --accuracy-every steps, one MLARM step and
    one BIEM step from the same state give the velocity error, and the drift
    of area and length since the start is recorded.  A failure ends the leg
    and is reported with its step."""
    import torch
    from ves2dpy_gb300.curve import Curve
    from ves2dpy_gb300.tstep_biem import TStepBiem
    nv = X.shape[1]
    prams = dict(STEP, viscCont=[1.0] * nv, gmresTol=a.biem_tol)
    rows = []
    try:
        for k in range(a.accuracy_steps + 1):
            if k % a.accuracy_every == 0:
                tt = TStepBiem(X, None, dict(farField="shear", usePreco=True), prams, near="py_hh",
                               farfield_precision=a.precision, sl_precision="fp32c", precond_precision=a.biem_precond)
                Xb, *_ = tt.time_step(X, t)
                Xm, _ = m.time_step_many_noinfo(X, t, 3)
                _, ar, ln = Curve().geomProp(X)
                drift = max(float(((ar - area0).abs() / area0).max()), float(((ln - len0).abs() / len0).max()))
                rows.append({"step": k, "velocity_error": centroid_velocity_error(X, Xm, Xb, STEP["dt"], dev),
                             "drift": drift})
            if k < a.accuracy_steps:
                X, t = m.time_step_many_noinfo(X, t, 3)
    except Exception as e:  # the trajectory ended (e.g. a non-finite shape): report where
        rows.append({"failed_at_step": k, "error": str(e)[:200]})
    return rows


def run_biem(a, dev, X0):
    import torch
    from ves2dpy_gb300 import _native as nat
    from ves2dpy_gb300.layout import from_vm, to_vm
    from ves2dpy_gb300.tstep_biem import TStepBiem
    from ves2dpy_gb300.replicas import barrier

    N, nv = a.N, a.nv
    options = dict(farField="shear", usePreco=True, repulsion=False)
    prams = dict(STEP, viscCont=[1.0] * nv, gmresTol=a.biem_tol)
    Xd = torch.tensor(X0, dtype=torch.float64, device=dev)
    tt = TStepBiem(Xd, None, options, prams, near="py_hh", farfield_precision=a.precision,
                   sl_precision="fp64" if a.precision == "fp64" else "fp32c", precond_precision=a.biem_precond)
    ctx = nat.context(N, dev)
    ws = ctx.workspace(tt.workspace_bytes())
    Xv = to_vm(Xd)
    sv = torch.zeros(nv, N, dtype=torch.float64, device=dev)
    Xo, so = torch.empty_like(Xv), torch.empty_like(sv)
    X1 = None
    for i in range(a.biem_warmup):
        Xo, so, res = tt.step_device(Xv, sv, Xo, so, ws)
        if i == 0:
            X1 = from_vm(Xo).cpu()
        Xv, Xo, sv, so = Xo, Xv, so, sv
    mv, info = [], []
    torch.cuda.synchronize()
    barrier()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = _events()
    e0.record(stream)
    for i in range(a.biem_steps):
        Xo, so, res = tt.step_device(Xv, sv, Xo, so, ws)
        mv.append(res.matvecs)
        info.append((res.info, res.resid))
        Xv, Xo, sv, so = Xo, Xv, so, sv
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    if X1 is None and a.biem_steps == 1:
        X1 = from_vm(Xv).cpu()  # the first step from X0
    return dict(ms=e0.elapsed_time(e1), matvecs=mv, info=info, X1=X1)


def centroid_velocity_error(X0, Xm, Xb, dt, dev):
    """Relative error (2-norm over all vesicles) of the MLARM step's vesicle
    velocities against the BIEM step's from the same state.  A vesicle's
    velocity is that of its physical (area) centre, getPhysicalCenter
    (curve_batch_compile.py:84-100): unlike the mean of the points, it does
    not depend on the parametrisation, which the MLARM step redistributes
    every step and the BIEM step carries with the flow."""
    import torch
    from ves2dpy_gb300.curve import Curve
    cv = Curve()

    def c(X):
        return cv.getPhysicalCenter(torch.as_tensor(X, dtype=torch.float64, device=dev)).double()

    c0 = c(X0)
    vm = (c(Xm) - c0) / dt
    vb = (c(Xb) - c0) / dt
    return float(torch.linalg.norm(vm - vb) / torch.linalg.norm(vb))


def run_gb300(a, rank, world):
    import numpy as np
    import torch
    from ves2dpy_gb300 import _native as nat
    from ves2dpy_gb300.mlarm_weights import NETS, synthetic_state_dict
    from ves2dpy_gb300.replicas import aggregate

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    X0 = workload(a.nv, a.N, a.area_fraction, seed=rank)
    sds, norms, net_info = networks(a)
    r = run_mlarm(a, dev, X0, sds, norms)
    t_max, value = aggregate(r["ms"], float(a.nv * a.steps), dev)
    ms_per_step = t_max / a.steps
    b = None if a.no_biem else run_biem(a, dev, r["Xw"])
    if b is not None:
        tb, vb = aggregate(b["ms"], float(a.nv * a.biem_steps), dev)
    if rank != 0:
        return None, sds, None
    st = r["stats"]
    sfu_peak = nat.probe_sfu_peak(dev)
    ff_ms = st.farfield_ms / max(st.farfield_launches, 1)
    ff_pairs = st.farfield_pairs / max(st.farfield_launches, 1)
    mufu_rate = 2.0 * ff_pairs / (ff_ms * 1e-3) if ff_ms > 0 else 0.0
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    # the network kernels are timed inside a step of about a second: the
    # sustained BF16 figure is their denominator
    bf16_peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1700.0))
    if "bf16_tflops_sustained" in peaks:
        bf16_src = ("MEASURED_PEAKS.json bf16_tflops_sustained (cuBLAS BF16 GEMM looped for seconds under the power "
                    "cap), of measured")
    elif "bf16_tflops" in peaks:
        bf16_src = "MEASURED_PEAKS.json bf16_tflops (burst; no sustained figure), of measured"
    else:
        bf16_src = "no MEASURED_PEAKS.json: 1.7 PFLOP/s, the sustained BF16 figure of an earlier GB300 measurement, of fallback"
    flops = {n: net_flops(NETS[n]) * a.nv for n in NETS}
    net_total_ms = sum(r["net_ms"].values())
    net_tflops = sum(flops.values()) / (net_total_ms * 1e-3) / 1e12 if net_total_ms > 0 else None
    # networks, timed live inside the timed MLARM steps (CUDA events around each forward pass)
    nl_tflops = (st.networks_flops / (st.networks_ms * 1e-3) / 1e12) if st.networks_ms > 0 else None
    roof_net = {"bound": "tensor",
                "kernel": "tcnet::down_kernel / up1_kernel / up2_kernel (tcgen05.mma kind::f16, BF16)",
                "achieved": nl_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": nl_tflops / bf16_peak if nl_tflops else None, "traffic": None,
                "traffic_note": "ncu (profiles/tcnet_blocks_nv64_full.md): the down + up1 + up2 launches of one "
                                "advection-network block at nv=64 move 22 + 108 + 250 MB of DRAM (the FP32 block "
                                "input read by down and up2, the output written by up2, the BF16 intermediates "
                                "written and read once; no re-reads), at most 26% of the DRAM peak",
                "flops_per_step": st.networks_flops / a.steps, "ms_per_step": st.networks_ms / a.steps,
                "passes_per_step": st.networks_launches / a.steps,
                "peak_source": bf16_src,
                "share_of_step": st.networks_ms / r["ms"] if r["ms"] else None}
    # all-pairs sums
    sm_mhz = (r["clocks"] or {}).get("sm_max_mhz") or 2070.0
    if a.precision == "fp32m":
        # FP32 work actually done: 16 FMA per series term (four complex Horner
        # steps) and 12 FP32 operations per direct-rule pair
        ff_flops = 2.0 * (16.0 * st.farfield_mp_terms + 12.0 * st.farfield_direct_pairs) / max(st.farfield_launches, 1)
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6
        ach = ff_flops / (ff_ms * 1e-3) if ff_ms > 0 else 0.0
        roof_ff = {"bound": "fp32", "kernel": "mp_eval_kernel (multipole series + direct rule for close pairs)",
                   "achieved": ach / 1e12, "peak": fp32_peak / 1e12, "unit": "TFLOP/s",
                   "frac": ach / fp32_peak, "traffic": None,
                   "traffic_note": "compute-bound: sources, moments and targets stay in L2",
                   "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 x max SM clock (no measured figure)",
                   "ms_per_launch": ff_ms, "series_terms_per_launch": st.farfield_mp_terms / max(st.farfield_launches, 1),
                   "direct_pairs_per_launch": st.farfield_direct_pairs / max(st.farfield_launches, 1),
                   "reference_pairs_per_launch": ff_pairs,
                   "reference_pairs_per_s": ff_pairs / (ff_ms * 1e-3) if ff_ms > 0 else None,
                   "share_of_step": st.farfield_ms / r["ms"] if r["ms"] else None}
    else:
        roof_ff = {"bound": "sfu", "kernel": "ff_main_kernel (all-pairs Stokeslet sum, direct)",
                   "achieved": mufu_rate / 1e9, "peak": sfu_peak / 1e9, "unit": "Gop/s (MUFU lg2+rcp)",
                   "frac": mufu_rate / sfu_peak if sfu_peak else None, "traffic": None,
                   "traffic_note": "compute-bound; ncu measured 6.7 MB DRAM per launch at nv=256 "
                                   "(sources L2-resident), see profiles/ff_main_kernel_nv256_N128_full.md",
                   "pairs_per_launch": ff_pairs, "ms_per_launch": ff_ms,
                   "gpairs_per_s": ff_pairs / (ff_ms * 1e-3) / 1e9 if ff_ms > 0 else None,
                   "peak_source": "measured by ves_probe_sfu_peak on this GPU",
                   "share_of_step": st.farfield_ms / r["ms"] if r["ms"] else None}
    # the dominant kernel of the step carries the main roofline
    roof_main = roof_ff if (roof_ff.get("share_of_step") or 0) > (roof_net.get("share_of_step") or 0) else roof_net
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
        "dtype": ("bf16 networks (fp32 accumulation) + f32 all-pairs sums (" +
                  ("multipole series for separated vesicle pairs, compensated direct sums for close pairs"
                   if a.precision == "fp32m" else "compensated direct sums" if a.precision == "fp32c" else "f64") +
                  ") + f64 geometry"),
        "data": "synthetic (seeded suspension generator; networks of the reference architectures "
                + ("trained here on BIEM-generated shapes and targets" if "trained" in net_info["weights"]
                   else "with seeded synthetic weights") +
                "; the reference's trained weights and initial conditions are absent)",
        "config": {
            "workload": f"MLARM step (time_step_many_noinfo, nlayers=3) vs plain BIEM step (TStepBiem.time_step), "
                        f"nv={a.nv}, N={a.N}, Nup=1536, unit-length vesicles of reduced area 0.65, area fraction "
                        f"{a.area_fraction}, shear rate 2, dt=1e-5",
            "networks": a.nets, "network_weights": net_info, "farfield_precision": a.precision,
            "network_autotune": not a.no_autotune,
            "l2": "inputs larger than L2 (network activations 11 GB, upsampled sources 50 MB x 2 + near lists, "
                  "per step)",
            "parallelism": "replicas only" if world > 1 else "single GPU",
            "mlarm": {"ms_per_step": ms_per_step, "near_pairs_excluded": r["near_pairs"],
                      "judge_tol": a.judge_tol, "biem_fallbacks_per_step": r["fallbacks"] / max(a.steps, 1),
                      "network_errors_vs_biem_operators": r["judge"],
                      "conserve": a.conserve, "area_len_tol": a.area_len_tol or 1e-2,
                      "accuracy_along_trajectory": r["accuracy"],
                      "network_errors_note": "relative 2-norm error of each network (as the step runs it) against "
                                             "the BIEM operator it stands for, on 512 vesicles of the timed steps' "
                                             "starting state (ves_mlarm_targets; merged networks on |k| <= 16)",
                      "area_length_drift": r["drift"],
                      "drift_note": "max over vesicles of the relative area and length change after the warm-up "
                                    "and timed steps against the initial shapes; the step's correction "
                                    "(correctAreaAndLengthAugLag) acts only beyond 1e-2 (its tolerance), so the "
                                    "drift below that is the networks' own",
                      "network_ms": r["net_ms"],
                      "network_tflops": net_tflops,
                      "farfield_ms_per_eval": ff_ms, "farfield_evals_per_step": st.farfield_launches / a.steps},
        },
        "e2e": {"value": world * a.nv / r["e2e_s"], "unit": "vesicle-steps/s", "h2d_bytes_per_step": r["io"],
                "d2h_bytes_per_step": r["io"]} if r["e2e_s"] else None,
        "gpu_launches": int(r["launches"]),
        "roofline": roof_main,
        "roofline_networks": roof_net,
        "roofline_farfield": roof_ff,
        "clocks": r["clocks"],
    }
    if b is not None:
        out["config"]["biem"] = {"value": vb, "unit": "vesicle-steps/s", "ms_per_step": tb / a.biem_steps,
                                 "preconditioner": a.biem_precond,
                                 "steps": a.biem_steps, "warmup": a.biem_warmup, "matvecs_per_step": b["matvecs"],
                                 "gmres_info_resid": b["info"], "gmres_tol": a.biem_tol,
                                 "note": "the context, kernels and workspace are warm from the MLARM run; same "
                                         "all-pairs precision as the MLARM arm; GMRES tol 1e-8 because the FP32 "
                                         "all-pairs operators are accurate to ~1e-8 on unit-length vesicles (with "
                                         "the direct FP32 sums GMRES stalls near 5e-9 at tol 1e-10 and stops after "
                                         "106 matvecs; the FP64 operator converges in 38-50 at nv=256)"}
        out["config"]["mlarm_over_biem"] = value / vb
        try:
            if r["X1"] is None:
                raise ValueError("no end-to-end step")
            out["config"]["centroid_velocity_error_vs_biem"] = centroid_velocity_error(
                r["Xw"], r["X1"], b["X1"], STEP["dt"], dev)
            out["config"]["velocity_error_note"] = (
                "relative 2-norm over vesicles of the physical-centre velocity of one MLARM step against one BIEM "
                "step from the same state (the timed steps' starting state)" +
                ("" if "trained" in net_info["weights"] else "; synthetic untrained weights: not a physical prediction"))
        except Exception:
            pass
    return out, sds, (b["matvecs"] if b is not None else None)


def run_cpu_reference(a, rank):
    """--impl reference: the oracle port of the reference path on the host cores.

    Every step (warm-up and timed) is one bounded sample of the MLARM step's
    all-pairs work (the same target-vesicle chunk on every core of a spawned
    pool, sized so that the whole run takes a few minutes); the full step's
    time is extrapolated from each sample's measured pair rate, plus the five
    networks of one vesicle (FP32 torch, measured once) times nv.  The line
    says so: ``extrapolated`` is true, ``steps`` counts the sample steps that
    ran, and ``sample_s_per_step`` / ``timed_region_s`` are measured times."""
    if rank != 0:
        return None
    import multiprocessing as mp
    import numpy as np
    from oracle import ves2d_oracle as O
    from ves2dpy_gb300.mlarm_weights import NETS, synthetic_state_dict
    sds = {n: synthetic_state_dict(n, 0) for n in NETS}
    cores = os.cpu_count() or 1
    net_s = cpu_net_seconds(sds, cores)
    tab = O.PotenTables(a.N)
    X = workload(64, a.N, 0.15, seed=1)
    f = np.random.default_rng(0).normal(size=X.shape)
    Xup, fup = O.interpft_vec(X, tab.Nup), O.interpft_vec(f, tab.Nup)
    sa = O.diff_prop(Xup)[0]
    nsv = 16 if a.N >= 128 else 64
    task = (Xup[:, :nsv + 1], sa[:, :nsv + 1], fup[:, :nsv + 1], X[:, :1], nsv)
    t1, _ = _cpu_worker(task)
    per_step = min(6.0, max(1.0, 150.0 / max(a.steps + a.warmup, 1)))
    reps = max(1, int(per_step / max(t1, 1e-3)))
    ppe = pairs_per_eval(a.nv, a.N)
    step_ms, sample_s = [], []
    with mp.get_context("spawn").Pool(cores) as pool:
        pool.map(_cpu_worker, [task] * cores)  # start the workers
        for i in range(a.warmup + a.steps):
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, [task] * (reps * cores))
            wall = time.perf_counter() - t0
            rate = sum(p for _, p in res) / wall
            if i >= a.warmup:
                sample_s.append(wall)
                step_ms.append((2 * ppe / rate + a.nv * net_s) * 1e3)
    ms = float(np.mean(step_ms))
    v = a.nv / (ms * 1e-3)
    sample = (f"each step: {reps * cores} x (1 target vesicle vs {nsv} source vesicles, N={a.N}, Nup={tab.Nup}) "
              f"on {cores} processes ({float(np.mean(sample_s)):.2f} s measured), its pair rate extrapolated to the "
              f"step's 2 all-pairs evaluations of {ppe:.3e} pairs, plus the five networks of one vesicle in FP32 "
              f"torch ({net_s:.3f} s) times nv")
    cb = {"value": v, "unit": "vesicle-steps/s", "cores": cores, "kind": "port", "sample": sample}
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "vesicle-steps/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "extrapolated": True,
            "sample_s_per_step": float(np.mean(sample_s)), "timed_region_s": float(np.sum(sample_s)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 geometry, f32 networks",
            "data": "synthetic",
            "config": {"workload": f"MLARM step, nv={a.nv}, N={a.N}: CPU oracle port of the reference algorithm; "
                                   "ms_per_step is the full step extrapolated from each step's bounded sample"},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "vesicle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_only_net(a):
    """One network's forward pass (BF16 unless --nets fp32) at --nv, twice;
    prints the second pass's CUDA-event time (a profiling target)."""
    import torch
    from ves2dpy_gb300.mlarm import Network
    from ves2dpy_gb300.mlarm_weights import NETS, synthetic_state_dict
    dev = torch.device("cuda", 0)
    spec = NETS[a.only_net]
    net = Network(a.only_net, synthetic_state_dict(a.only_net, 0), a.nets, dev, autotune=not a.no_autotune)
    x = torch.randn(a.nv, spec.rep * spec.cin, spec.L, device=dev, dtype=net.dtype)
    net(x)
    e0, e1 = _events()
    torch.cuda.synchronize()
    e0.record()
    net(x)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    print(json.dumps({"network": a.only_net, "nv": a.nv, "precision": a.nets, "ms": ms,
                      "tflops": net_flops(spec) * a.nv / (ms * 1e-3) / 1e12}), flush=True)


def main():
    a = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if a.only_net:
        run_only_net(a)
        return
    if a.impl == "reference":
        out = run_cpu_reference(a, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    out, sds, mv = run_gb300(a, rank, world)
    if rank == 0 and out is not None:
        if not a.no_cpu_baseline:
            out["cpu_baseline"] = cpu_estimates(a, sds, mv)
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
