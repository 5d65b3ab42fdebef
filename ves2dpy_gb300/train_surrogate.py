"""Train the MLARM networks on BIEM-generated data and write them to a model
directory that ``training.load`` (and ``MLARM_manyfree_py.from_trained``)
reads.

    python -m ves2dpy_gb300.train_surrogate --out DIR [--shapes 60000]
           [--seconds relax=900,selften=600,adv=420,advten=300] [--seed 0]

Every stage runs on the current CUDA device: shape generation and evolution
(``ves_isolated_step``), standardisation, the BIEM targets
(``ves_mlarm_targets``) and the training kernels (``ves_trainer``).  5% of
the shapes are held out; the log records each network's relative error on
them against the BIEM targets.
"""
from __future__ import annotations

import argparse
import json
import time

import torch

from . import training as T


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--shapes", type=int, default=60000)
    ap.add_argument("--seconds", default="relax=900,selften=600,adv=420,advten=300")
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=5e-4)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    dev = torch.device("cuda", torch.cuda.current_device())
    budget = {k: float(v) for k, v in (kv.split("=") for kv in a.seconds.split(","))}
    t0 = time.perf_counter()

    def log(msg):
        print(f"[{time.perf_counter() - t0:7.1f} s] {msg}", flush=True)

    Xs = T.shape_dataset(a.shapes, a.seed, dev)
    log(f"{Xs.shape[0]} standardised shapes")
    data = T.Dataset(Xs)
    log(f"BIEM targets done; {data.n} shapes kept, {data.dropped} dropped as outliers")
    # indices into the kept shapes (the dataset drops outliers)
    perm = torch.randperm(data.n, device=dev, generator=torch.Generator(dev).manual_seed(a.seed))
    nval = max(256, data.n // 20)
    val, train = perm[:nval], perm[nval:]
    nets, meta = {}, {"shapes": data.n, "dropped": data.dropped, "validation_shapes": nval,
                      "modes": list(T.TRAIN_MODES), "nets": {}}
    for name, sec in budget.items():
        tr, info = T.train_network(name, data, train, sec, batch=a.batch, lr=a.lr, seed=a.seed, log=log)
        err = T.evaluate(name, tr, data, val)
        log(f"{name}: {info['steps']} steps, validation relative error {err:.3e}")
        nets[name] = tr.state_dict()
        meta["nets"][name] = {"steps": info["steps"], "s_per_step": info["s_per_step"], "batch": a.batch,
                              "seconds": sec, "validation_rel_error": err, "losses": info["losses"]}
        del tr
    T.save(a.out, nets, data.norms(), meta)
    log(f"written to {a.out}")
    print(json.dumps({k: v["validation_rel_error"] for k, v in meta["nets"].items()}))


if __name__ == "__main__":
    main()
