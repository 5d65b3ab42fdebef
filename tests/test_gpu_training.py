"""GPU parity of the training path of the MLARM networks.

* ves_mlarm_targets against the oracle's FP64 restatement
  (oracle/mlarm_oracle.py exact_targets), ves_isolated_step against the
  oracle BIEM step of one vesicle (tstep_biem.py:181-428, nv = 1);
* the trainer's forward pass (FP64) against the oracle's
  torch.nn.functional forward of each network's one-group architecture;
* one backward pass of every layer type (stride-2 and dilated circular
  convolutions, transposed convolutions, the mixing convolution, batch norm,
  ReLU, residual and pass-through channels) against torch.autograd in FP64;
* a short training run that lowers the loss.

Tolerances: FP64 paths 1e-10 (gradients, forward) and 1e-8 for the targets,
which go through two dense solves per vesicle.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _shapes(n, seed):
    from ves2dpy_gb300.training import random_shapes
    return random_shapes(n, seed, amp=(0.0, 0.03))


def test_targets_match_oracle():
    from oracle import mlarm_oracle as M
    from ves2dpy_gb300 import training as T
    X = _shapes(3, 11)
    Xs = T.standardize(torch.tensor(X, dtype=torch.float64, device=DEV))
    Xs_o, _ = M.standardization_step(X.T)
    assert rel(Xs.T, Xs_o) < 1e-10
    got = T.targets(Xs, dt=1e-5, sl_precision="fp64")
    want = M.exact_targets(Xs.cpu().numpy().T, dt=1e-5)
    assert rel(got["relax"].T, want["relax"]) < 1e-8
    assert rel(got["selften"].T, want["selften"]) < 1e-8
    assert rel(got["advten"], want["advten"]) < 1e-8
    assert rel(got["adv"], want["adv"]) < 1e-8


@pytest.mark.parametrize("speed", [0.0, 2.0])
def test_isolated_step_matches_biem_step_of_one_vesicle(speed):
    from oracle import ves2d_oracle as O
    from ves2dpy_gb300 import training as T
    X = _shapes(2, 12)
    Xt = torch.tensor(X, dtype=torch.float64, device=DEV)
    vinf = None
    if speed:
        vinf = torch.cat([speed * Xt[:, 128:], torch.zeros_like(Xt[:, :128])], 1)
    got = T.isolated_step(Xt, vinf, 1e-4, sl_precision="fp64")
    for k in range(2):
        res = O.time_step(X[k][:, None], np.zeros((128, 1)), O.StepParams(dt=1e-4, speed=speed, gmres_tol=1e-13))
        assert rel(got[k], res.X[:, 0]) < 1e-10


def _torch_net(spec, sd):
    return {k: torch.tensor(np.asarray(v, dtype=np.float64),
                            requires_grad=not (k.endswith("running_mean") or k.endswith("running_var")))
            for k, v in sd.items()}


@pytest.mark.parametrize("name", ["relax", "adv", "selften", "advten", "near"])
def test_trainer_forward_and_gradients_match_autograd(name):
    from oracle import mlarm_oracle as M
    from ves2dpy_gb300 import training as T
    spec = T.group_spec(name)
    sd = T.init_state_dict(spec, seed=5)
    rng = np.random.default_rng(6)
    # exercise the batch-norm statistics and scales too
    for k in sd:
        if k.endswith("running_mean"):
            sd[k] = rng.normal(0, 0.1, sd[k].shape).astype(np.float32)
        elif k.endswith("running_var"):
            sd[k] = rng.uniform(0.5, 1.5, sd[k].shape).astype(np.float32)
        elif ".bn" in k:
            sd[k] = (sd[k] + rng.normal(0, 0.1, sd[k].shape)).astype(np.float32)
    B = 3
    x = rng.normal(size=(B, spec.cin, spec.L))
    t = rng.normal(size=(B, spec.cout, spec.L))
    tr = T.Trainer(spec, sd, "fp64", B, DEV)
    y = tr.forward(torch.from_numpy(x))
    W = _torch_net(spec, sd)
    yr = M.net_forward_t(spec, W, torch.from_numpy(x))
    assert rel(y, yr) < 1e-12
    loss = tr.backward(torch.from_numpy(t))
    lr = ((yr - torch.from_numpy(t)) ** 2).mean()
    lr.backward()
    assert abs(loss - lr.item()) <= 1e-12 * abs(lr.item())
    g = tr.grads_f64()
    off = 0
    worst = 0.0
    for b in spec.blocks:
        for key in T.ORDER:
            name_k = f"{b.prefix}.{key}"
            n = W[name_k].numel()
            if not (key.endswith("running_mean") or key.endswith("running_var")):
                ref = W[name_k].grad.numpy().reshape(-1)
                err = np.abs(g[off:off + n] - ref).max() / max(np.abs(ref).max(), 1e-300)
                worst = max(worst, err)
                assert err < 1e-10, (name_k, err)
            off += n
    assert off == g.size


@pytest.mark.parametrize("name", ["relax", "adv"])
def test_fp32_trainer_at_a_large_batch_matches_fp64(name):
    """Batches large enough that each CTA walks several samples: the FP32
    kernels' gradients against the FP64 trainer's: FP32 rounding of sums
    over 300 samples x up to 256 positions, with cancellation in the first
    layers of the deep networks (5e-3 of each array's 2-norm)."""
    from ves2dpy_gb300 import training as T
    spec = T.group_spec(name)
    sd = T.init_state_dict(spec, seed=9)
    rng = np.random.default_rng(10)
    B = 300
    x = torch.from_numpy(rng.normal(size=(B, spec.cin, spec.L)))
    t = torch.from_numpy(rng.normal(size=(B, spec.cout, spec.L)))
    w = torch.from_numpy(rng.uniform(0.5, 2.0, size=B))
    g = {}
    for prec in ("fp64", "fp32"):
        tr = T.Trainer(spec, sd, prec, B, DEV)
        tr.forward(x)
        tr.backward(t, sample_weights=w)
        g[prec] = tr.grads()
    for k in g["fp64"]:
        if k.endswith("running_mean") or k.endswith("running_var"):
            continue
        a, b = g["fp32"][k], g["fp64"][k]
        assert np.linalg.norm(a - b) <= 5e-3 * max(np.linalg.norm(b), 1e-30), k


def test_training_lowers_the_loss():
    from ves2dpy_gb300 import training as T
    Xs = T.standardize(torch.tensor(_shapes(512, 13), dtype=torch.float64, device=DEV))
    data = T.Dataset(Xs, chunk=512)
    idx = torch.arange(data.n, device=DEV)   # the shapes the dataset kept
    tr, info = T.train_network("relax", data, idx, seconds=15.0, batch=128)
    first = T.evaluate("relax", T.Trainer(T.group_spec("relax"), T.init_state_dict(T.group_spec("relax"), 0),
                                          "fp32", 256, DEV), data, idx[:256])
    last = T.evaluate("relax", tr, data, idx[:256])
    assert info["steps"] >= 40
    assert last < 0.5 * first, (first, last, info["losses"])


def test_surrogate_errors_of_the_trained_networks():
    """The BIEM operators judging the trained networks as the step runs them
    (merged, BF16 tensor cores, the step's normalisation): each relative
    error is finite and below 1 on the benchmark generator's shapes."""
    import math
    from ves2dpy_gb300 import training as T
    from ves2dpy_gb300.mlarm import Network
    from ves2dpy_gb300.suspension import random_suspension
    if not T.have_trained():
        pytest.skip("no trained networks in the package")
    sds, norms = T.load()
    nets = {n: Network(n, sds[n], "bf16", DEV) for n in ("relax", "selften", "adv", "advten")}
    X = random_suspension(64, 128, 0.15, min_gap=0.05 / 7.79, area=0.65 / (4 * math.pi), seed=3)
    Xs = T.standardize(torch.tensor(X.T.copy(), dtype=torch.float64, device=DEV))
    err = T.surrogate_errors(nets, norms, Xs)
    for name, e in err.items():
        assert np.isfinite(e) and e < 1.0, (name, e)
