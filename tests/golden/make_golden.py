"""Record golden fixtures from the Ves2Dpy reference (``mytorch/``).

Run in the development container (the reference tree must be present):

    python tests/golden/make_golden.py

Each fixture is produced in a fresh subprocess because the FP64 promotion of
``ref_shim.load(promote=True)`` rebinds torch dtypes process-wide.  Inputs
come from the package's seeded generators, so the fixture files are
reproducible.  The files are small ``.npz`` archives committed next to this
script; tests read them without needing the reference.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)


def _np(t):
    return t.detach().cpu().numpy()


def small_cluster(nv=6, N=16, seed=3, gap=0.02):
    """Closely packed small suspension so that near pairs (< 1/N) exist."""
    from ves2dpy_gb300.suspension import vesicle_shape
    rng = np.random.default_rng(seed)
    X = np.zeros((2 * N, nv))
    # two rows of vesicles with small gaps, scaled to length ~1 so 1/N matters
    for k in range(nv):
        x, y = vesicle_shape(N, rng, 0.8, area=0.06)
        X[:N, k] = x + (k % 3) * 0.32
        X[N:, k] = y + (k // 3) * 0.30
    return X


def patch_exact_stokes_sl(R):
    """Evaluate exactStokesSL_ per target column (the reference raises a shape
    error at mytorch/biem_support.py:382 for multi-column targets)."""
    torch = R.torch

    def fixed(vesicle, f, Xtar=None, K1=None):
        Ntar, ncol = Xtar.shape[0] // 2, Xtar.shape[1]
        out = torch.zeros((2 * Ntar, ncol), dtype=torch.float64)
        den = f * torch.tile(vesicle.sa, (2, 1)) * 2 * torch.pi / vesicle.N
        xs = vesicle.X[:vesicle.N, K1].reshape(-1)
        ys = vesicle.X[vesicle.N:, K1].reshape(-1)
        dxs = den[:vesicle.N, K1].reshape(-1)
        dys = den[vesicle.N:, K1].reshape(-1)
        for k in range(ncol):
            dx = Xtar[:Ntar, k][None, :] - xs[:, None]
            dy = Xtar[Ntar:, k][None, :] - ys[:, None]
            r2 = dx ** 2 + dy ** 2
            c = (dx * dxs[:, None] + dy * dys[:, None]) / r2
            lg = 0.5 * torch.log(r2)
            out[:Ntar, k] = torch.sum(c * dx - lg * dxs[:, None], dim=0)
            out[Ntar:, k] = torch.sum(c * dy - lg * dys[:, None], dim=0)
        return out / (4 * torch.pi)

    R.poten.exactStokesSL_ = fixed


def make_prams(R, N, nv, dt, speed, tol=1e-10, kind='shear'):
    torch = R.torch
    prams = dict(N=N, nv=nv, dt=dt, T=10 * dt, kappa=1.0, viscCont=torch.ones(nv), gmresTol=tol,
                 gmresMaxIter=200, areaLenTol=1e-2, repStrength=900, minDist=0.4, farFieldSpeed=speed,
                 chanWidth=2.5, vortexSize=2.5)
    options = dict(farField=kind, repulsion=False, correctShape=False, reparameterization=False,
                   usePreco=True, matFreeWalls=False, confined=False)
    return prams, options


def job_far(promote):
    import ref_shim
    R = ref_shim.load(promote=promote)
    torch = R.torch
    X = small_cluster()
    N, nv = X.shape[0] // 2, X.shape[1]
    rng = np.random.default_rng(11)
    f = rng.normal(size=(2 * N, nv))
    Xt = torch.tensor(X)
    ft = torch.tensor(f)
    op = R.poten.Poten(N)
    Xup = R.filter.interpft_vec(Xt, op.Nup)
    fup = R.filter.interpft_vec(ft, op.Nup)
    vesUp = R.capsules.capsules(Xup, None, None, 1.0, 1.0)
    near = R.biem_support.naiveNearZoneInfo(Xt, Xup)
    far1, ids1 = R.biem_support.allExactStokesSLTarget_compare1(Xup, vesUp.sa, fup, Xt)
    far2 = R.biem_support.allExactStokesSLTarget_compare2(Xup, vesUp.sa, fup, Xt, *near[4])
    far_noexcl = R.biem_support.allExactStokesSLTarget_compare2(
        Xup, vesUp.sa, fup, Xt, torch.zeros(0, dtype=torch.long), torch.zeros(0, dtype=torch.long),
        torch.zeros(0, dtype=torch.long))
    # Poten.exactStokesSL: one target column, sources = all vesicles but 0
    ves = R.capsules.capsules(Xt, None, None, 1.0, torch.ones(nv))
    sl = R.poten.Poten.exactStokesSL(op, ves, ft, Xt[:, :1], list(range(1, nv)))
    return dict(X=X, f=f, Xup=_np(Xup), fup=_np(fup), sa_up=_np(vesUp.sa),
                closest_dist=_np(near[0]), idx_closest=_np(near[1]),
                id1=_np(near[2][0]), id2=_np(near[2][1]), id1_hh=_np(near[3][0]), id2_hh=_np(near[3][1]),
                ids0=_np(near[4][0]), ids1=_np(near[4][1]), ids2=_np(near[4][2]),
                far1=_np(far1), c1_ids0=_np(ids1[0]), c1_ids1=_np(ids1[1]), c1_ids2=_np(ids1[2]),
                far2=_np(far2), far_noexcl=_np(far_noexcl), exact_sl_col0=_np(sl))


def job_capsules(promote):
    import ref_shim
    from ves2dpy_gb300.suspension import vesicle_shape
    R = ref_shim.load(promote=promote)
    torch = R.torch
    out = {}
    for N in (16, 32):
        rng = np.random.default_rng(100 + N)
        nv = 4
        X = np.zeros((2 * N, nv))
        for k in range(nv):
            x, y = vesicle_shape(N, rng, 0.65 + 0.08 * k)
            X[:N, k] = x + 3 * k
            X[N:, k] = y - k
        sig = rng.normal(size=(N, nv))
        f = rng.normal(size=(2 * N, nv))
        dtype = torch.float64 if promote else torch.float32
        Xt = torch.tensor(X, dtype=dtype)
        ves = R.capsules.capsules(Xt, None, None, 1.0, torch.ones(nv))
        Ben, Ten, Div = ves.computeDerivs()
        oc = R.curve.Curve()
        ra, area, length = oc.geomProp(Xt)
        op = R.poten.Poten(N)
        G = op.stokesSLmatrix(ves)
        out.update({
            f'X{N}': X, f'sig{N}': sig, f'f{N}': f,
            f'sa{N}': _np(ves.sa), f'xt{N}': _np(ves.xt), f'cur{N}': _np(ves.cur),
            f'trac{N}': _np(ves.tracJump(Xt, torch.tensor(sig, dtype=dtype))),
            f'sdiv{N}': _np(ves.surfaceDiv(torch.tensor(f, dtype=dtype))),
            f'Ben{N}': _np(Ben), f'Ten{N}': _np(Ten), f'Div{N}': _np(Div),
            f'ra{N}': _np(ra), f'area{N}': _np(area), f'len{N}': _np(length),
            f'up{N}': _np(R.filter.interpft_vec(Xt, op.Nup)),
            f'G{N}': _np(G), f'qw{N}': _np(op.qw[:, 0]), f'qp{N}': _np(op.qp),
            f'Rlp{N}': _np(op.Restrict_LP), f'Plp{N}': _np(op.Prolong_LP),
        })
    return out


def job_step(promote, which):
    import ref_shim
    from ves2dpy_gb300.suspension import config1_suspension
    R = ref_shim.load(promote=promote)
    torch = R.torch
    if which == 'c1':
        X = config1_suspension(32, 0)
        dt, speed, nsteps = 1e-4, 2.0, 10 if promote else 1   # the configuration's 10 steps
    else:
        patch_exact_stokes_sl(R)
        X = small_cluster(nv=4, N=16, seed=1)
        dt, speed, nsteps = 1e-4, 2.0, 1
    N, nv = X.shape[0] // 2, X.shape[1]
    dtype = torch.float64 if promote else torch.float32
    Xt = torch.tensor(X, dtype=dtype)
    prams, options = make_prams(R, N, nv, dt, speed)
    tt = R.tstep_biem.TStepBiem(Xt, None, options, prams)
    sig = torch.zeros(N, nv, dtype=dtype)
    out = dict(X0=X, dt=dt, speed=speed)
    if which == 'near':
        near = R.biem_support.naiveNearZoneInfo(Xt, R.filter.interpft_vec(Xt, tt.op.Nup))
        out['n_near'] = len(near[4][0])
        out['n_hh'] = len(near[3][0])
        rng = np.random.default_rng(7)
        f = torch.tensor(rng.normal(size=(2 * N, nv)))
        ves = R.capsules.capsules(Xt, None, None, 1.0, torch.ones(nv))
        G = tt.op.stokesSLmatrix(ves)
        SLP = lambda F: tt.op.exactStokesSLdiag(ves, G, F)  # noqa: E731
        LP, nearF = tt.op.nearSingInt_hh(ves, f, SLP, near, R.biem_support.wrapper_allExactStokesSLTarget_compare2,
                                        ves, True)
        out.update(f_near=_np(f), LP_near=_np(LP), nearField=_np(nearF))
    for s in range(nsteps):
        Xn, sig, _, _, it, iflag = tt.time_step(Xt, sig, None, None)
        out[f'X{s + 1}'] = _np(Xn).astype(np.float64)
        out[f'sig{s + 1}'] = _np(sig).astype(np.float64)
        out[f'iter{s + 1}'] = int(it)
        out[f'iflag{s + 1}'] = bool(iflag)
        Xt = Xn
    return out


def job_post(promote):
    """Post-step conditioning (curve_batch_compile.py:590-972) on perturbed shapes."""
    import ref_shim
    from ves2dpy_gb300.suspension import vesicle_shape
    R = ref_shim.load(promote=promote)
    torch = R.torch
    dtype = torch.float64 if promote else torch.float32
    oc = R.curve.Curve()
    out = {}
    for tag, N, area in (("unit", 32, 0.06), ("big", 32, float(np.pi))):
        rng = np.random.default_rng(21 if tag == "unit" else 22)
        nv = 4
        X = np.zeros((2 * N, nv))
        for k in range(nv):
            # non-equispaced parametrisation: theta -> theta + 0.15 sin(theta)
            x, y = vesicle_shape(N, rng, 0.65 + 0.05 * k, area=area)
            th = np.arange(N) * 2 * np.pi / N
            z = np.fft.fft(x + 1j * y) / N
            m = np.concatenate([np.arange(0, N // 2), np.arange(-N // 2, 0)])
            tw = th + 0.15 * np.sin(th + k)
            zz = (z[None, :] * np.exp(1j * np.outer(tw, m))).sum(1)
            X[:N, k] = zz.real + 2.0 * k
            X[N:, k] = zz.imag - 1.0 * k
        modes = torch.concatenate((torch.arange(0, N // 2), torch.arange(-N // 2, 0)))
        Xt = torch.tensor(X, dtype=dtype)
        X1, good = oc.redistributeArcLength(Xt.clone(), modes)
        X5 = Xt.clone()
        for _ in range(5):
            X5, _ = oc.redistributeArcLength(X5, modes)
        Xal = oc.alignCenterAngle(Xt, X5)
        ctr = oc.getPhysicalCenter(Xt)
        ia = oc.getIncAngle(Xt)
        _, a0, l0 = oc.geomProp(Xt)
        # a shape whose area and length are off by a few percent
        Xpert = Xt.clone()
        Xpert[:, 1] = Xpert[:, 1] * 1.03
        Xpert[:N, 2] = Xpert[:N, 2] * 1.02
        Xc = oc.correctAreaAndLengthAugLag(Xpert.clone(), a0, l0)
        out.update({f"X_{tag}": X, f"redist1_{tag}": _np(X1), f"redist5_{tag}": _np(X5), f"align_{tag}": _np(Xal),
                    f"center_{tag}": _np(ctr), f"incangle_{tag}": _np(ia), f"pert_{tag}": _np(Xpert),
                    f"corrected_{tag}": _np(Xc), f"a0_{tag}": _np(a0), f"l0_{tag}": _np(l0)})
    return out


def mlarm_suspension(nv=4, N=128, seed=17):
    """Four unit-length vesicles (reduced area 0.65), one pair closer than 1/N."""
    import math
    from ves2dpy_gb300.suspension import random_suspension
    return random_suspension(nv, N, 0.35, min_gap=0.003, area=0.65 / (4 * math.pi), seed=seed)


def _mlarm_instance(R, precision, root, dt=1e-5, speed=2.0):
    """The reference MLARM with seeded synthetic networks saved as TorchScript
    files where its constructor looks for them (``../trained/torch_script_models``
    relative to the working directory)."""
    torch = R.torch
    from ves2dpy_gb300.mlarm_weights import NETS, NET_ARGS, MODEL_FILES, synthetic_state_dict, synthetic_norms
    mdir = os.path.join(root, "trained", "torch_script_models")
    os.makedirs(mdir, exist_ok=True)
    os.makedirs(os.path.join(root, "run"), exist_ok=True)
    for name in NETS:
        m = getattr(R.nets, name)(*NET_ARGS[name])
        sd = synthetic_state_dict(name, 0)
        m.load_state_dict({k: torch.from_numpy(v) for k, v in sd.items()}, strict=False)
        m.eval()
        torch.jit.script(m).save(os.path.join(mdir, MODEL_FILES[name]))
    nrm = synthetic_norms(0)

    def T(a):
        return torch.from_numpy(np.asarray(a, dtype=np.float64))

    def vinf(X):  # shear, entry_driver_manyfreeSpaceVesicle_N128.py:53
        N = X.shape[0] // 2
        return speed * torch.vstack((X[N:], torch.zeros_like(X[:N])))

    cwd = os.getcwd()
    os.chdir(os.path.join(root, "run"))
    try:
        oc = R.curve.Curve()
        m = R.wrapper.MLARM_manyfree_py(
            dt, vinf, oc, False, 1e2, -1,
            T(nrm["adv_in"]), T(nrm["adv_out"]), T(nrm["relax_in"]), T(nrm["relax_out"]),
            T(nrm["near_in"]), T(nrm["near_out"]), T(nrm["selften_in"]), T(nrm["selften_out"]),
            T(nrm["advten_in"]), T(nrm["advten_out"]), device=torch.device("cpu"), logger=None)
    finally:
        os.chdir(cwd)
    if precision == "fp64":
        for net in (m.relaxNetwork, m.mergedAdvNetwork, m.nearNetwork, m.tenSelfNetwork, m.tenAdvNetwork):
            net.model.double()
    return m, oc


def job_mlarm(precision):
    """Two MLARM steps (time_step_many_noinfo, N128:986-1206) with stage outputs of the first."""
    import tempfile
    import ref_shim
    R = ref_shim.load_mlarm(precision)
    torch = R.torch
    root = tempfile.mkdtemp(prefix="mlarm_golden_")
    m, oc = _mlarm_instance(R, precision, root)
    X0 = mlarm_suspension()
    N, nv = X0.shape[0] // 2, X0.shape[1]
    X = torch.from_numpy(X0.copy())
    # entry_driver_manyfreeSpaceVesicle_N128.py:157-167: reference area and
    # length first, then up to 10 redistribution passes
    area0, len0 = oc.geomProp(X)[1:]
    m.area0, m.len0 = area0, len0
    modes = torch.concatenate((torch.arange(0, N // 2), torch.arange(-N // 2, 0)))
    for _ in range(10):
        X, flag = oc.redistributeArcLength(X, modes)
        if flag:
            break
    Xinit = X.clone()
    rec = {}

    def wrap(cls, name):
        f = getattr(cls, name)

        def g(self, *a, **k):
            r = f(self, *a, **k)
            # copies: redistributeArcLength later updates some results in place
            rec.setdefault(name, []).append(_clone(r))
            return r
        setattr(cls, name, g)

    def _clone(r):
        if isinstance(r, torch.Tensor):
            return r.clone()
        if isinstance(r, (tuple, list)):
            return type(r)(_clone(x) for x in r)
        return r

    for nm in ("standardizationStep", "translateVinfwTorch", "relaxWTorchNet", "invTenMatOnVback",
               "invTenMatOnSelfBend", "computeStokesInteractions_noinfo"):
        wrap(type(m), nm)
    for nm in ("alignCenterAngle", "correctAreaAndLengthAugLag"):
        wrap(type(oc), nm)
    ten = torch.zeros((N, nv), dtype=torch.float64)  # entry :121
    out = {"X0": X0, "Xinit": _np(Xinit), "area0": _np(area0), "len0": _np(len0)}
    nsteps = 10 if precision == "fp64" else 2
    out["nsteps"] = nsteps
    for step in range(nsteps):
        with torch.no_grad():
            X, ten = m.time_step_many_noinfo(X, ten, 3)
        out[f"X{step + 1}"] = _np(X)
        out[f"ten{step + 1}"] = _np(ten)
        if step == 0:
            Xs, sv = rec["standardizationStep"][0]
            out["stand_X"] = _np(Xs)
            for k, v in zip(("scaling", "rotate", "rotCenter", "trans", "sortIdx"), sv):
                out["stand_" + k] = _np(v)
            Xs2, sv2 = rec["standardizationStep"][1]
            out["relax_stand_X"] = _np(Xs2)
            f1, _, ids = rec["computeStokesInteractions_noinfo"][0]
            out["far1"] = _np(f1)
            for i in range(3):
                out[f"near_ids{i}"] = _np(ids[i])
            out["far2"] = _np(rec["computeStokesInteractions_noinfo"][1][0])
            out["vback_solve"] = _np(rec["invTenMatOnVback"][0])
            out["selfbend_solve"] = _np(rec["invTenMatOnSelfBend"][0])
            out["Xadv"] = _np(rec["translateVinfwTorch"][0])
            out["Xrelax"] = _np(rec["relaxWTorchNet"][0])
            out["Xalign"] = _np(rec["alignCenterAngle"][0])
            out["Xcorr"] = _np(rec["correctAreaAndLengthAugLag"][0])
    return out


def job_nets(precision):
    """Each network's output (FP64 reference modules) on seeded inputs, one vesicle.

    The merged networks are independent per channel group, so only groups
    0-3 and the last two are stored."""
    import ref_shim
    from ves2dpy_gb300.mlarm_weights import NETS, NET_ARGS, synthetic_state_dict, net_test_input
    R = ref_shim.load_mlarm(precision)
    torch = R.torch
    out = {}
    for name, spec in NETS.items():
        m = getattr(R.nets, name)(*NET_ARGS[name])
        m.load_state_dict({k: torch.from_numpy(v) for k, v in synthetic_state_dict(name, 0).items()}, strict=False)
        m.eval()
        m.double()
        x = torch.from_numpy(net_test_input(name))
        with torch.no_grad():
            y = m(x).numpy()
        co = spec.cout
        groups = [0, 1, 2, 3, spec.rep - 2, spec.rep - 1] if spec.rep > 6 else list(range(spec.rep))
        out[name + "_groups"] = np.asarray(groups)
        out[name] = np.stack([y[:, g * co:(g + 1) * co] for g in groups], axis=1)  # (nv, groups, cout, L)
    return out


def job_io(promote):
    """Geometry and trajectory tooling: ``Curve.ellipse`` (curve_batch_compile.py:494-527)
    and ``load_ves2d_file`` (newtorch/tools/load_ves2d_file.py:4-72) reading a file
    written with the drivers' statements (driver_confined.py:204-206, 294-296)."""
    import importlib.util
    import tempfile
    import ref_shim
    R = ref_shim.load(promote=promote)
    torch = R.torch
    oc = R.curve.Curve()
    out = {}
    for N, ra in ((32, 0.65), (64, 0.9), (128, 0.5), (16, 0.75)):
        out[f"ellipse_{N}_{int(round(ra * 100))}"] = _np(oc.ellipse(N, torch.tensor([ra])))
    rng = np.random.default_rng(5)
    N, nv = 16, 3
    X0 = rng.normal(size=(2 * N, nv))
    frames = [(1e-5 * (k + 1), rng.normal(size=(2 * N, nv))) for k in range(4)]
    path = os.path.join(tempfile.mkdtemp(), "traj.bin")
    with open(path, 'wb') as fid:
        np.array([N, nv]).flatten().astype('float64').tofile(fid)
        X0.T.flatten().astype('float64').tofile(fid)
    for time_, X in frames:
        output = np.concatenate(([time_], X.T.flatten())).astype('float64')
        with open(path, 'ab') as fid:
            output.tofile(fid)
    spec = importlib.util.spec_from_file_location(
        "load_ves2d_file", os.path.join(ref_shim.REF_ROOT, "newtorch", "tools", "load_ves2d_file.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    vesx, vesy, time_, Nr, nvr, xinit, yinit = mod.load_ves2d_file(path)
    out.update({"traj_bytes": np.fromfile(path, dtype=np.uint8), "traj_X0": X0,
                "traj_frames": np.stack([X for _, X in frames]), "traj_times": np.array([t for t, _ in frames]),
                "load_vesx": vesx, "load_vesy": vesy, "load_time": time_, "load_N": Nr, "load_nv": nvr,
                "load_xinit": xinit, "load_yinit": yinit})
    return out


def job_repulsion(promote):
    """capsules.repulsionForce (capsules.py:209-252) on a packed cluster."""
    import ref_shim
    R = ref_shim.load(promote=promote)
    torch = R.torch
    out = {}
    for tag, (nv, N, gap, W, eta) in {"tight": (6, 16, 0.02, 1e5, 1.0 / 16), "wide": (5, 32, 0.05, 900.0, 0.4)}.items():
        X = small_cluster(nv=nv, N=N, seed=7, gap=gap)
        ves = R.capsules.capsules(torch.tensor(X), None, None, 1.0, 1.0)
        rep = ves.repulsionForce(torch.tensor(X), W, eta)
        out.update({f"X_{tag}": X, f"rep_{tag}": _np(rep), f"W_{tag}": W, f"eta_{tag}": eta})
    return out


def job_rbf(promote):
    """nearSingInt_rbf (poten.py:643-785) with nearFieldCorrectionUP_SOLVE
    (:788-894) and exactStokesSL_onlyself (biem_support.py:468-516), called as
    the newtorch BIEM matvec does (tstep_biem.py:431): self term G f, far field
    with the near-zone exclusions, near pairs corrected by the RBF fit."""
    import ref_shim
    R = ref_shim.load(promote=promote)
    torch = R.torch
    out = {}
    cases = {"n32": (small_cluster_sized(4, 32, seed=11, scale=1.0, gap=0.01), 32),
             "n128": (mlarm_suspension(), 128)}
    for tag, (X, N) in cases.items():
        Xt = torch.tensor(X)
        nv = X.shape[1]
        ves = R.capsules.capsules(Xt, None, None, 1.0, torch.ones(nv))
        op = R.poten.Poten(N)
        G = op.stokesSLmatrix(ves)
        Xup = R.filter.interpft_vec(Xt, op.Nup)
        near = R.biem_support.naiveNearZoneInfo(Xt, Xup)
        rng = np.random.default_rng(12)
        f = torch.tensor(rng.normal(size=(2 * N, nv)))
        SLP = lambda F: op.exactStokesSLdiag(ves, G, F)  # noqa: E731
        far = R.biem_support.wrapper_allExactStokesSLTarget_compare2(
            Xup, R.capsules.capsules(Xup, None, None, 1.0, torch.ones(nv)).sa, R.filter.interpft_vec(f, op.Nup),
            Xt, near[-1])
        LP = op.nearSingInt_rbf(ves, f, SLP, near, R.biem_support.wrapper_allExactStokesSLTarget_compare2, ves, True)
        out.update({f"X_{tag}": X, f"f_{tag}": _np(f), f"G_{tag}": _np(G), f"vself_{tag}": _np(SLP(f)),
                    f"far_{tag}": _np(far), f"LP_{tag}": _np(LP), f"id1_{tag}": _np(near[2][0]),
                    f"id2_{tag}": _np(near[2][1])})
    return out


def small_cluster_sized(nv, N, seed, scale, gap):
    """A row of nv vesicles of area pi*scale^2, each placed so that its leftmost
    point faces the previous vesicle's rightmost point at distance ``gap``."""
    from ves2dpy_gb300.suspension import vesicle_shape
    rng = np.random.default_rng(seed)
    X = np.zeros((2 * N, nv))
    prev = None
    for k in range(nv):
        x, y = vesicle_shape(N, rng, 0.8, area=np.pi * scale ** 2)
        x, y = x - x.mean(), y - y.mean()
        if prev is not None:
            px, py = prev
            i, j = int(np.argmax(px)), int(np.argmin(x))
            x = x + (px[i] - x[j]) + gap
            y = y + (py[i] - y[j])
        X[:N, k], X[N:, k] = x, y
        prev = (x, y)
    return X


def job_step_rbf(promote):
    """One BIEM step of the mytorch stepper with its matvec near field by
    nearSingInt_rbf -- the alternative written (commented) at
    mytorch/tstep_biem.py:494 and used by the newtorch stepper
    (newtorch/tstep_biem.py:431) -- on the packed near cluster.  (The newtorch
    stepper also drops the 1e-7 regularisation of mytorch's stokesSLmatrix,
    newtorch/poten.py:71, so its steps differ from these in G as well.)"""
    import ref_shim
    R = ref_shim.load(promote=promote)
    torch = R.torch
    op_cls = R.poten.Poten

    def hh_as_rbf(self, vesicleSou, f, selfMat, NearV2V, kernelDirect, vesicleTar, tEqualS):
        LP = self.nearSingInt_rbf(vesicleSou, f, selfMat, NearV2V, kernelDirect, vesicleTar, tEqualS)
        return LP, torch.zeros_like(LP)

    op_cls.nearSingInt_hh = hh_as_rbf
    X = small_cluster(nv=4, N=16, seed=1)
    N, nv = X.shape[0] // 2, X.shape[1]
    Xt = torch.tensor(X)
    prams, options = make_prams(R, N, nv, 1e-4, 2.0)
    tt = R.tstep_biem.TStepBiem(Xt, None, options, prams)
    Xn, sig, _, _, it, iflag = tt.time_step(Xt, torch.zeros(N, nv), None, None)
    return dict(X0=X, dt=1e-4, speed=2.0, X1=_np(Xn).astype(np.float64), sig1=_np(sig).astype(np.float64),
                iter1=int(it), iflag1=bool(iflag))


def job_step_rep(promote):
    """One BIEM step with repulsion (tstep_biem.py:250-264: repulsionForce,
    then G rep + nearSingInt_rbf(rep) on the right-hand side) on the packed
    near cluster, mytorch stepper (matvec near field nearSingInt_hh)."""
    import ref_shim
    R = ref_shim.load(promote=promote)
    patch_exact_stokes_sl(R)
    torch = R.torch
    X = small_cluster(nv=4, N=16, seed=1)
    N, nv = X.shape[0] // 2, X.shape[1]
    Xt = torch.tensor(X)
    prams, options = make_prams(R, N, nv, 1e-4, 2.0)
    options['repulsion'] = True
    prams['repStrength'] = 2e3
    prams['minDist'] = 0.06
    tt = R.tstep_biem.TStepBiem(Xt, None, options, prams)
    ves = R.capsules.capsules(Xt, None, None, 1.0, torch.ones(nv))
    rep = ves.repulsionForce(Xt, prams['repStrength'], prams['minDist'])
    Xn, sig, _, _, it, iflag = tt.time_step(Xt, torch.zeros(N, nv), None, None)
    return dict(X0=X, dt=1e-4, speed=2.0, W=prams['repStrength'], eta=prams['minDist'], rep=_np(rep),
                X1=_np(Xn).astype(np.float64), sig1=_np(sig).astype(np.float64), iter1=int(it), iflag1=bool(iflag))


def separated_row(nv, N, seed, spacing=2.5):
    """nv vesicles of the default shape generator on a row, ``spacing`` apart
    (no near pairs at the 1/N threshold)."""
    from ves2dpy_gb300.suspension import vesicle_shape
    rng = np.random.default_rng(seed)
    X = np.zeros((2 * N, nv))
    for k in range(nv):
        x, y = vesicle_shape(N, rng, 0.7)
        X[:N, k] = x - x.mean() + spacing * k
        X[N:, k] = y - y.mean() + 0.3 * (k % 2)
    return X


def job_dl(promote):
    """Double layer of vesicles with a viscosity contrast: stokesDLmatrix,
    exactStokesDLdiag and exactStokesDL (mytorch/poten.py:102-175, 227-238,
    399-441), the far-field loop of nearSingInt with kernelDirect =
    exactStokesDL, and one BIEM step with contrasts.

    The reference's viscosity-contrast step does not run as written: it calls
    ``op.nearSingInt`` (tstep_biem.py:236, 501), which mytorch/poten.py does
    not define, and its block preconditioner adds the 2N x N block G*Ten to a
    2N x 2N one (tstep_biem.py:331-334, a shape error).  The step fixture
    therefore runs with usePreco=False (scipy's removed ``tol`` keyword of
    tstep_biem.py:383 passed as ``rtol``) on vesicles without near pairs, with
    ``nearSingInt`` supplied as the far-field loop of matlab/poten_py.m:571-579
    written with the reference's own interpft_vec, capsules and exactStokesDL
    (with no near pairs that loop is the whole of nearSingInt)."""
    import ref_shim
    R = ref_shim.load(promote=promote)
    torch = R.torch
    out = {}

    def far_loop(op):
        def nearSingInt(vesicleSou, f, selfMat, NearStruct, kernelDirect, vesicleTar, tEqualS):
            assert tEqualS and vesicleTar is vesicleSou
            if NearStruct is not None:
                assert len(NearStruct[4][0]) == 0 and len(NearStruct[3][0]) == 0, "near pairs present"
            Xup = R.filter.interpft_vec(vesicleSou.X, op.Nup)
            fup = R.filter.interpft_vec(f, op.Nup)
            vup = R.capsules.capsules(Xup, None, None, vesicleSou.kappa, vesicleSou.viscCont)
            nvs = vesicleSou.X.shape[1]
            cols = [kernelDirect(vup, fup, vesicleTar.X[:, k:k + 1], [j for j in range(nvs) if j != k])
                    for k in range(nvs)]
            return torch.cat(cols, dim=1)
        return nearSingInt

    for tag, N, nv, seed, visc in (("n32", 32, 3, 41, [3.0, 1.0, 0.5]), ("n128", 128, 2, 42, [0.25, 4.0])):
        X = separated_row(nv, N, seed)
        Xt = torch.tensor(X)
        vt = torch.tensor(visc)
        ves = R.capsules.capsules(Xt, None, None, 1.0, vt)
        op = R.poten.Poten(N)
        D = op.stokesDLmatrix(ves)
        rng = np.random.default_rng(seed + 100)
        f = torch.tensor(rng.normal(size=(2 * N, nv)))
        Xtar = Xt + torch.tensor([0.0] * N + [4.0] * N)[:, None]
        dl = op.exactStokesDL(ves, f, Xtar, list(range(nv)))
        near = R.biem_support.naiveNearZoneInfo(Xt, R.filter.interpft_vec(Xt, op.Nup))
        assert len(near[4][0]) == 0
        far = far_loop(op)(ves, f, None, near, op.exactStokesDL, ves, True)
        out.update({f"X_{tag}": X, f"visc_{tag}": np.array(visc), f"f_{tag}": _np(f), f"D_{tag}": _np(D),
                    f"DLdiag_{tag}": _np(op.exactStokesDLdiag(ves, D, f)), f"Xtar_{tag}": _np(Xtar),
                    f"DL_{tag}": _np(dl), f"far_{tag}": _np(far)})

    # one step, nv=3, N=32, contrasts 3, 1, 0.5
    _gmres = R.tstep_biem.gmres

    def gmres_rtol(A, b, tol=None, **kw):
        return _gmres(A, b, rtol=tol, **kw)

    R.tstep_biem.gmres = gmres_rtol
    X = out["X_n32"]
    N, nv = X.shape[0] // 2, X.shape[1]
    Xt = torch.tensor(X)
    prams, options = make_prams(R, N, nv, 1e-4, 2.0)
    prams['viscCont'] = torch.tensor([3.0, 1.0, 0.5])
    options['usePreco'] = False
    tt = R.tstep_biem.TStepBiem(Xt, None, options, prams)
    tt.op.nearSingInt = far_loop(tt.op)
    Xn, sig, _, _, it, iflag = tt.time_step(Xt, torch.zeros(N, nv), None, None)
    out.update(step_X0=X, step_visc=np.array([3.0, 1.0, 0.5]), step_dt=1e-4, step_speed=2.0,
               step_X1=_np(Xn).astype(np.float64), step_sig1=_np(sig).astype(np.float64), step_iter1=int(it),
               step_iflag1=bool(iflag))
    return out


def job_bgflow(promote):
    """bg_flow (mytorch/tstep_biem.py:849-952) for every unconfined kind, with
    non-default speed, channel width and vortex size, on a lattice suspension."""
    import ref_shim
    from ves2dpy_gb300.suspension import lattice_suspension
    R = ref_shim.load(promote=promote)
    torch = R.torch
    X = lattice_suspension(3, 32, spacing=3.0, jitter=0.2, min_gap=0.3, seed=4)
    N, nv = X.shape[0] // 2, X.shape[1]
    Xt = torch.tensor(X, dtype=torch.float64)
    prams, options = make_prams(R, N, nv, 1e-4, 1.0)
    tt = R.tstep_biem.TStepBiem(Xt, None, options, prams)
    out = {"X": X, "kinds": np.array(["relaxation", "extensional", "parabolic", "taylorGreen", "vortex", "shear"])}
    for kind in out["kinds"]:
        v = tt.bg_flow(Xt, None, str(kind), Speed=1.7, chanWidth=2.3, vortexSize=1.9)
        out[f"v_{kind}"] = _np(v)
    return out


JOBS = {
    'bgflow_fp64': (job_bgflow, True, ()),
    'dl_fp64': (job_dl, True, ()),
    'io_fp64': (job_io, True, ()),
    'step_rep_fp64': (job_step_rep, True, ()),
    'step_near_rbf_fp64': (job_step_rbf, True, ()),
    'rbf_fp64': (job_rbf, True, ()),
    'repulsion_fp64': (job_repulsion, True, ()),
    'mlarm_fp64': (job_mlarm, 'fp64', ()),
    'mlarm_mixed': (job_mlarm, 'mixed', ()),
    'nets_fp64': (job_nets, 'fp64', ()),
    'post_fp64': (job_post, True, ()),
    'post_mixed': (job_post, False, ()),
    'far_fp64': (job_far, True, ()),
    'capsules_fp64': (job_capsules, True, ()),
    'capsules_mixed': (job_capsules, False, ()),
    'step_c1_fp64': (job_step, True, ('c1',)),
    'step_c1_mixed': (job_step, False, ('c1',)),
    'step_near_fp64': (job_step, True, ('near',)),
}


def main():
    if len(sys.argv) > 2 and sys.argv[1] == '--job':
        name = sys.argv[2]
        fn, promote, extra = JOBS[name]
        out = fn(promote, *extra)
        np.savez_compressed(os.path.join(HERE, f'{name}.npz'), **out)
        print('wrote', name)
        return
    names = sys.argv[1:] or list(JOBS)
    for name in names:
        subprocess.run([sys.executable, os.path.abspath(__file__), '--job', name], check=True)


if __name__ == '__main__':
    main()
