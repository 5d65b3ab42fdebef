"""Calibration of the CPU oracle port against the reference's own all-pairs
sum, for the CPU baseline of bench.py.

The baseline times ``oracle.ves2d_oracle.all_exact_stokes_sl_target`` (a NumPy
restatement) on one target vesicle against 16 upsampled source vesicles
(N = 128, Nup = 1536) per task.  This script times the reference's
``allExactStokesSLTarget_compare1`` (mytorch/biem_support.py:7-121, imported
through ref_shim, in torch) on the same sample, through its own ``offset``
argument for the one target column, with 1 and with all torch threads, and
prints the pair rates of both.  Run here (the reference is importable only in
this container): python tests/golden/calibrate_port.py
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def main():
    import ref_shim
    from oracle import ves2d_oracle as O
    from ves2dpy_gb300.suspension import random_suspension
    R = ref_shim.load(promote=True)
    torch = R.torch
    N, nsv = 128, 16
    tab = O.PotenTables(N)
    X = random_suspension(64, N, 0.15, min_gap=0.05 / 7.79, area=0.65 / (4 * np.pi), seed=1)
    f = np.random.default_rng(0).normal(size=X.shape)
    Xup, fup = O.interpft_vec(X, tab.Nup), O.interpft_vec(f, tab.Nup)
    sa = O.diff_prop(Xup)[0]
    src = slice(0, nsv + 1)
    pairs = N * tab.Nup * nsv
    out = {"sample": f"1 target vesicle (N={N}) vs {nsv} source vesicles (Nup={tab.Nup})", "pairs": pairs}

    def rate(fn, reps):
        fn()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return pairs * reps / (time.perf_counter() - t0)

    out["oracle_port_1proc_pairs_per_s"] = rate(
        lambda: O.all_exact_stokes_sl_target(Xup[:, src], sa[:, src], fup[:, src], X[:, :1], None), 5)
    Xt, st, ft = (torch.tensor(a[:, src]) for a in (Xup, sa, fup))
    tar = torch.tensor(X[:, :1])
    for threads in (1, os.cpu_count()):
        torch.set_num_threads(threads)
        out[f"reference_{threads}threads_pairs_per_s"] = rate(
            lambda: R.biem_support.allExactStokesSLTarget_compare1(Xt, st, ft, tar, 1.0, 0), 5)
    out["reference_over_port_1core"] = out["reference_1threads_pairs_per_s"] / out["oracle_port_1proc_pairs_per_s"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
