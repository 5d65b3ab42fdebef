"""CPU FP64 oracle for the MLARM surrogate step (N = 128).

TEST INFRASTRUCTURE ONLY.  This module is the checker that the CUDA MLARM
path is compared against.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU legs of ``bench.py`` may import it; the ``ves2dpy_gb300`` package
never does.

It restates ``MLARM_manyfree_py.time_step_many_noinfo``
(``newtorch/wrapper_MLARM_batch_compile_N128.py:986-1206``) in NumPy double
precision, with the five networks evaluated by ``torch.nn.functional`` in
float64 from a state dict in the reference's naming.  Parity of this
restatement is pinned by ``tests/test_oracle_golden.py`` against fixtures
recorded from the reference itself (``tests/golden/make_golden.py``).

Work whose result the reference step never reads is not restated: the
Gaussian RBF matrix and its Cholesky factor (``:1063-1070``; consumed only
when ``use_near_correct`` is true, ``:2660``), the layer tracer coordinates
(``:1741-1797``, consumed by that matrix only) and the near network, whose
velocities enter the step only multiplied by the repulsion force
(``:2500``), which is zero without repulsion.
"""
from __future__ import annotations

import math

import numpy as np

from oracle import ves2d_oracle as O

RELAX_DT_SCALE = 1e-5  # get_network_torch.py:77: DX / 1E-5 * dt


# --------------------------------------------------------------------------
# networks (model_zoo/*.py) through torch.nn.functional in float64
# --------------------------------------------------------------------------

def net_forward(spec, sd, x, dtype=np.float64):
    """Forward of a network described by ``spec`` (mlarm_weights.NetSpec) with
    state dict ``sd`` on input x (nv, rep*cin, L); numpy in/out in ``dtype``
    (float64 for parity, float32 to time the reference networks' precision)."""
    import torch
    t = torch.from_numpy(np.asarray(x, dtype=dtype))
    W = {k: torch.from_numpy(np.asarray(v, dtype=dtype)) for k, v in sd.items()}
    return net_forward_t(spec, W, t).numpy()


def net_forward_t(spec, W, t):
    """net_forward on torch tensors (state dict W, input t): differentiable,
    the reference for the training kernels' gradients."""
    import torch
    import torch.nn.functional as F

    G = spec.rep
    nv = t.shape[0]

    def conv(inp, name, pad, dil):
        return F.conv1d(F.pad(inp, (pad, pad), mode="circular"), W[name + ".weight"], W[name + ".bias"],
                        stride=2, dilation=dil, groups=G)

    def bn(inp, name):
        return F.batch_norm(inp, W[name + ".running_mean"], W[name + ".running_var"], W[name + ".weight"],
                            W[name + ".bias"], training=False, eps=1e-5)

    def pair(a, b):
        ch = a.shape[1] // G
        return torch.cat((a.reshape(nv, G, ch, -1), b.reshape(nv, G, ch, -1)), dim=2).reshape(nv, 2 * ch * G, -1)

    for blk in spec.blocks:
        p = blk.prefix
        a = pair(F.relu(conv(t, p + ".conv1_1", 3, 1)), F.relu(conv(t, p + ".conv1_2", 6, 2)))
        a = bn(a, p + ".bn1")
        b = pair(F.relu(conv(a, p + ".conv2_1", 3, 1)), F.relu(conv(a, p + ".conv2_2", 6, 2)))
        b = bn(b, p + ".bn2")
        c = bn(F.relu(F.conv_transpose1d(b, W[p + ".deconv1.weight"], W[p + ".deconv1.bias"], stride=2, padding=4,
                                         groups=G)), p + ".bn3")
        d = bn(F.relu(F.conv_transpose1d(c, W[p + ".deconv2.weight"], W[p + ".deconv2.bias"], stride=2, padding=4,
                                         groups=G)), p + ".bn4")
        m = F.conv1d(d, W[p + ".mix.weight"], W[p + ".mix.bias"], padding=1, groups=G)
        L = m.shape[-1]
        xs = t.reshape(nv, G, blk.cin, L)
        mm = m.reshape(nv, G, blk.cmix, L)
        if blk.residual:
            mm = mm + xs[:, :, :blk.cmix]
        if blk.npass:
            mm = torch.cat((mm, xs[:, :, blk.cin - blk.npass:]), dim=2)
        t = mm.reshape(nv, G * blk.cout, L)
    return t


# --------------------------------------------------------------------------
# symmetric 2x2 eigen-decomposition with LAPACK's conventions
# --------------------------------------------------------------------------

def _sign(a, b):
    return abs(a) if b >= 0 else -abs(a)


def eig2_lapack(a, b, c, d):
    """Eigenvalues and unit eigenvectors of [[a, b], [c, d]] with real spectrum
    as LAPACK dgeev returns them for a 2x2 input (torch.linalg.eig on CPU):
    the Schur standardisation of dlanv2 (Bai & Demmel's published scheme)
    followed by back-substitution of the upper-triangular factor.

    Returns (w0, w1), V with V[:, i] the vector of w_i.
    """
    if c == 0.0:
        cs, sn = 1.0, 0.0
        aa, bb, dd = a, b, d
    elif b == 0.0:
        cs, sn = 0.0, 1.0
        aa, bb, dd = d, -c, a
    else:
        p = 0.5 * (a - d)
        bcmax = max(abs(b), abs(c))
        bcmis = min(abs(b), abs(c)) * _sign(1.0, b) * _sign(1.0, c)
        scale = max(abs(p), bcmax)
        z = (p / scale) * p + (bcmax / scale) * bcmis
        z = p + _sign(math.sqrt(scale) * math.sqrt(z), p)
        aa = d + z
        dd = d - (bcmax / z) * bcmis
        tau = math.hypot(c, z)
        cs = z / tau
        sn = c / tau
        bb = b - c
    v1 = np.array([cs, sn])
    if aa == dd:
        x1 = 0.0
    else:
        x1 = -bb / (aa - dd)
    v2 = x1 * np.array([cs, sn]) + np.array([-sn, cs])
    v2 = v2 / np.linalg.norm(v2)
    return (aa, dd), np.stack([v1, v2], axis=1)


def princ_axes(X, center):
    """getPrincAxesGivenCentroid (newtorch/curve_batch_compile.py:279-376):
    eigenvector of the smallest |eigenvalue| of the moment tensor J, with the
    sign LAPACK leaves it (no normalisation of the sign)."""
    N, nv = X.shape[0] // 2, X.shape[1]
    xc, yc = X[:N] - center[0], X[N:] - center[1]
    Dx, Dy = O.get_dxy(np.vstack([xc, yc]))
    jac = np.sqrt(Dx ** 2 + Dy ** 2)
    nx, ny = Dy / jac, -Dx / jac
    rdn = xc * nx + yc * ny
    rho2 = xc ** 2 + yc ** 2
    J11 = np.sum(rdn * (rho2 - xc ** 2) * jac, axis=0)
    J12 = np.sum(rdn * (-xc * yc) * jac, axis=0)
    J21 = np.sum(rdn * (-yc * xc) * jac, axis=0)
    J22 = np.sum(rdn * (rho2 - yc ** 2) * jac, axis=0)
    V = np.zeros((2, nv))
    for k in range(nv):
        w, vec = eig2_lapack(J11[k], J12[k], J21[k], J22[k])
        i = 0 if abs(w[0]) <= abs(w[1]) else 1
        V[:, k] = vec[:, i]
    return V


# --------------------------------------------------------------------------
# standardisation (wrapper_MLARM_batch_compile_N128.py:4119-4283)
# --------------------------------------------------------------------------

def rotation_op(X, theta, c):
    """rotationOperator (:4226-4239)."""
    N = X.shape[0] // 2
    x, y = X[:N] - c[0], X[N:] - c[1]
    ct, st = np.cos(theta), np.sin(theta)
    return np.vstack([x * ct - y * st + c[0], x * st + y * ct + c[1]])


def translate_op(X, t):
    """translateOp (:4241-4248)."""
    N = X.shape[0] // 2
    return np.vstack([X[:N] + t[0], X[N:] + t[1]])


def reference_values(X):
    """referenceValues (:4179-4223): translation, rotation, rotation centre,
    scaling and sort index (nv, N)."""
    N, nv = X.shape[0] // 2, X.shape[1]
    rc = O.physical_center(X)
    V = princ_axes(X, rc)
    rot = np.arctan2(V[0], V[1])
    Xr = rotation_op(X, rot, rc)
    trans = -O.physical_center(Xr)
    Xr = translate_op(Xr, trans)
    theta = np.arctan2(Xr[N:], Xr[:N])
    start = np.argmin(np.where(theta < 0, 100.0, theta), axis=0)
    sort_idx = ((start[None, :] + np.arange(N)[:, None]) % N).T
    _, _, length = O.geom_prop(Xr)
    return trans, rot, rc, 1.0 / length, sort_idx


def standardize(X, trans, rot, rc, scaling, sort_idx):
    """standardize (:4140-4152): rotate about rc, translate, reorder, scale."""
    N, nv = X.shape[0] // 2, X.shape[1]
    Xr = rotation_op(X, rot, rc)
    Xr = np.vstack([Xr[:N] + trans[0], Xr[N:] + trans[1]])
    cols = np.arange(nv)[None, :]
    return scaling * np.vstack([Xr[sort_idx.T, cols], Xr[sort_idx.T + N, cols]])


def destandardize(Xs, sv):
    """destandardize (:4154-4177)."""
    scaling, rot, rc, trans, sort_idx = sv
    N, nv = Xs.shape[0] // 2, Xs.shape[1]
    Xs = Xs / scaling
    X = np.zeros_like(Xs)
    cols = np.arange(nv)[None, :]
    X[sort_idx.T, cols] = Xs[:N]
    X[sort_idx.T + N, cols] = Xs[N:]
    X = translate_op(X, -trans)
    return rotation_op(X, -rot, rc)


def standardization_step(X):
    """standardizationStep (:4119-4138): five redistribution passes (no early
    exit), then the reference values."""
    X = X.copy()
    for _ in range(5):
        X, _ = O.redistribute_arc_length(X)
    trans, rot, rc, scaling, sort_idx = reference_values(X)
    Xs = standardize(X, trans, rot, rc, scaling, sort_idx)
    return Xs, (scaling, rot, rc, trans, sort_idx)


def _stand_velocity_fft(v, sv):
    """fft of the velocity/force rotated by the shape's angle and reordered,
    without translation or scaling (the ``standardize(..., 0, rot, 0, 1, idx)``
    calls at :1829, :3603, :3653)."""
    _, rot, _, _, sort_idx = sv
    nv = v.shape[1]
    vs = standardize(v, np.zeros((2, nv)), rot, np.zeros((2, nv)), 1.0, sort_idx)
    N = vs.shape[0] // 2
    zh = np.fft.fft(vs[:N] + 1j * vs[N:], axis=0)
    return zh.real, zh.imag


def _unsort(vals, sort_idx):
    """out[sort_idx[v, j], v] = vals[j, v]."""
    out = np.zeros_like(vals)
    out[sort_idx.T, np.arange(vals.shape[1])[None, :]] = vals
    return out


# --------------------------------------------------------------------------
# network wrappers (model_zoo/get_network_torch.py) and MLARM glue
# --------------------------------------------------------------------------

class Nets:
    """The five networks with their normalisation constants (float64)."""

    def __init__(self, state_dicts, norms):
        from ves2dpy_gb300.mlarm_weights import NETS
        self.spec = NETS
        self.sd = state_dicts
        self.nrm = {k: np.asarray(v, dtype=np.float64) for k, v in norms.items()}

    def run(self, name, x):
        return net_forward(self.spec[name], self.sd[name], x)

    def relax(self, Xin, dt):
        """RelaxNetwork.forward (get_network_torch.py:71-80)."""
        N, nv = Xin.shape[0] // 2, Xin.shape[1]
        p, q = self.nrm["relax_in"], self.nrm["relax_out"]
        inp = np.zeros((nv, 2, 128))
        inp[:, 0] = ((Xin[:N] - p[0]) / p[1]).T
        inp[:, 1] = ((Xin[N:] - p[2]) / p[3]).T
        out = self.run("relax", inp)
        DX = np.vstack([(out[:, 0] * q[1] + q[0]).T, (out[:, 1] * q[3] + q[2]).T])
        return Xin + DX / RELAX_DT_SCALE * dt

    def adv(self, Xs):
        """MergedAdvNetwork.forward (:150-203): (127, nv, 2, 256) per-mode blocks."""
        N, nv = Xs.shape[0] // 2, Xs.shape[1]
        rep = 127
        p = self.nrm["adv_in"].copy()
        p[63, 1] = 1.0  # x_std[63] = 1 (:163-167)
        p[63, 3] = 1.0
        cx = (Xs[:N, :, None] - p[:, 0]) / p[:, 1]     # (N, nv, rep)
        cy = (Xs[N:, :, None] - p[:, 2]) / p[:, 3]
        coords = np.concatenate([cx.transpose(1, 2, 0), cy.transpose(1, 2, 0)], axis=-1)  # (nv, rep, 2N)
        th = np.arange(N) / N * 2 * np.pi
        k = np.arange(1, N)
        basis = np.concatenate([np.cos(np.outer(th, k)) / N, np.sin(np.outer(th, k)) / N], axis=0).T  # (rep, 2N)
        inp = np.stack([coords, np.broadcast_to(basis, coords.shape)], axis=2).reshape(nv, 2 * rep, 2 * N)
        out = self.run("adv", inp).reshape(nv, rep, 2, 2 * N).transpose(1, 0, 2, 3)
        q = self.nrm["adv_out"]
        res = np.empty_like(out)
        res[:, :, 0] = out[:, :, 0] * q[:, 1, None, None] + q[:, 0, None, None]
        res[:, :, 1] = out[:, :, 1] * q[:, 3, None, None] + q[:, 2, None, None]
        res[63] = 0.0
        return res

    def _per_mode_input(self, Xs, p, modes):
        N, nv = Xs.shape[0] // 2, Xs.shape[1]
        x = (Xs[:N, :, None] - p[:, 0]) / p[:, 1]       # (N, nv, modes)
        y = (Xs[N:, :, None] - p[:, 2]) / p[:, 3]
        inp = np.stack([x, y], axis=0)                  # (2, N, nv, modes)
        return inp.transpose(2, 3, 0, 1).reshape(nv, 2 * modes, N)

    def advten(self, Xs):
        """MergedTenAdvNetwork pre/forward/post (:337-357): (127, nv, 2, 128)."""
        N, nv = Xs.shape[0] // 2, Xs.shape[1]
        inp = self._per_mode_input(Xs, self.nrm["advten_in"], 127)
        out = self.run("advten", inp).reshape(nv, 127, 2, N).transpose(2, 3, 0, 1)  # (2, N, nv, 127)
        q = self.nrm["advten_out"]
        res = np.empty_like(out)
        res[0] = out[0] * q[:, 1] + q[:, 0]
        res[1] = out[1] * q[:, 3] + q[:, 2]
        return res.transpose(3, 2, 0, 1)

    def selften(self, Xs):
        """TenSelfNetwork pre/forward/post (:229-278): (N, nv) standardised tension."""
        N, nv = Xs.shape[0] // 2, Xs.shape[1]
        p, q = self.nrm["selften_in"], self.nrm["selften_out"]
        inp = np.zeros((nv, 2, 128))
        inp[:, 0] = ((Xs[:N] - p[0]) / p[1]).T
        inp[:, 1] = ((Xs[N:] - p[2]) / p[3]).T
        out = self.run("selften", inp)[:, 0]            # (nv, N)
        return out.T * q[1] + q[0]


def tension_term(X, sig):
    return O.Capsule(X).tension_term(sig)


def bending_upsampled(X, kappa=1.0):
    """fBend of the step (:1007-1013): bending of the upsampled shape on
    Nup = N*ceil(sqrt(N)) points, truncated back to N modes."""
    N = X.shape[0] // 2
    Nup = N * math.ceil(math.sqrt(N))
    Xup = O.interpft_vec(X, Nup)
    cup = O.Capsule(Xup, kappa)
    return O.interpft_vec(cup.bending_term(Xup), N)


def exact_targets(Xs, dt=1e-5, kappa=1.0):
    """Training targets of the four trained networks for standardised shapes
    Xs (2N, nv), from the BIEM operators of each isolated vesicle (FP64):
    relax (2N, nv) = X+ - Xs of the implicit step without flow
    (tstep_biem.py:181-428 with one vesicle; its bending operator is the
    fourth power of the matvec's arc derivative, capsules.py:62-68); selften (N, nv) =
    A^-1 Div G fBend, A = Div G Ten; advten (nv, 254, N) and adv (nv, 254, 2N):
    A^-1 Div b and G Ten A^-1 Div b for the Fourier basis velocities
    b_{k,0} = (cos k th, sin k th)/N, b_{k,1} = (-sin k th, cos k th)/N,
    channel 2(k-1) + c, k = 1..127."""
    N, nv = Xs.shape[0] // 2, Xs.shape[1]
    tab = O.PotenTables(N)
    G = O.stokes_sl_matrix(Xs, tab)
    cap = O.Capsule(Xs, kappa)
    Ben, Ten, Div = cap.compute_derivs()
    fB = bending_upsampled(Xs, kappa)
    th = 2 * np.pi * np.arange(N) / N
    Bm = np.zeros((2 * N, 254))
    for m in range(127):
        c, s_ = np.cos((m + 1) * th) / N, np.sin((m + 1) * th) / N
        Bm[:N, 2 * m], Bm[N:, 2 * m] = c, s_
        Bm[:N, 2 * m + 1], Bm[N:, 2 * m + 1] = -s_, c
    relax = np.zeros((2 * N, nv))
    selften = np.zeros((N, nv))
    advten = np.zeros((nv, 254, N))
    adv = np.zeros((nv, 254, 2 * N))
    divx = cap.surface_div(Xs)
    D1 = np.real(O.fourier_diff(N))
    for k in range(nv):
        # the matvec's bending operator: the fourth power of its arc derivative
        Ar = cap.isa[:, k][:, None] * D1
        D4 = np.linalg.matrix_power(Ar, 4)
        Bk = np.zeros((2 * N, 2 * N))
        Bk[:N, :N] = Bk[N:, N:] = D4
        M = np.zeros((3 * N, 3 * N))
        M[:2 * N, :2 * N] = np.eye(2 * N) + dt * kappa * G[:, :, k] @ Bk
        M[:2 * N, 2 * N:] = -dt * G[:, :, k] @ Ten[:, :, k]
        M[2 * N:, :2 * N] = Div[:, :, k]
        sol = np.linalg.solve(M, np.concatenate([Xs[:, k], divx[:, k]]))
        relax[:, k] = sol[:2 * N] - Xs[:, k]
        GT = G[:, :, k] @ Ten[:, :, k]
        A = Div[:, :, k] @ GT
        selften[:, k] = np.linalg.solve(A, Div[:, :, k] @ (G[:, :, k] @ fB[:, k]))
        Z = np.linalg.solve(A, Div[:, :, k] @ Bm)
        advten[k] = Z.T
        adv[k] = (GT @ Z).T
    return {"relax": relax, "selften": selften, "advten": advten, "adv": adv}


def far_field(X, f, excl=None):
    """computeStokesInteractions_noinfo far field (:2495-2675) without
    repulsion: upsampled sources, coarse targets, near pairs (< 1/N) of the
    first call excluded in both calls."""
    N = X.shape[0] // 2
    Nup = N * math.ceil(math.sqrt(N))
    Xup = O.interpft_vec(X, Nup)
    jac, _, _ = O.diff_prop(Xup)
    fup = O.interpft_vec(f, Nup)
    if excl is None:
        excl = O.compare1_exclusions(Xup, X, length=1.0)
    return O.all_exact_stokes_sl_target(Xup, jac, fup, X, excl), excl


def inv_ten_mat_on_vback(nets, Xs, sv, vinf):
    """invTenMatOnVback (:3632-3669)."""
    out = nets.advten(Xs)                     # (127, nv, 2, N)
    V1, V2 = _stand_velocity_fft(vinf, sv)   # (N, nv)
    Z1 = out[:, :, 0].transpose(2, 0, 1)      # (N, 127, nv): Z1[j, k-1, v]
    Z2 = out[:, :, 1].transpose(2, 0, 1)
    mv = np.einsum("jkv,kv->jv", Z1, V1[1:]) + np.einsum("jkv,kv->jv", Z2, V2[1:])
    return _unsort(mv, sv[4])


def inv_ten_mat_on_self_bend(nets, Xs, sv):
    """invTenMatOnSelfBend (:3672-3688)."""
    scaling = sv[0]
    return _unsort(nets.selften(Xs) / scaling ** 2, sv[4])


def translate_vinf(nets, Xold, Xs, sv, vinf, dt):
    """translateVinfwTorch (:3584-3620)."""
    N, nv = Xs.shape[0] // 2, Xs.shape[1]
    P = nets.adv(Xs)                          # (127, nv, 2, 2N)
    V1, V2 = _stand_velocity_fft(vinf, sv)
    Z11 = P[:, :, 0, :N].transpose(2, 0, 1)   # (N, 127, nv)
    Z21 = P[:, :, 0, N:].transpose(2, 0, 1)
    Z12 = P[:, :, 1, :N].transpose(2, 0, 1)
    Z22 = P[:, :, 1, N:].transpose(2, 0, 1)
    mx = np.einsum("jkv,kv->jv", Z11, V1[1:]) + np.einsum("jkv,kv->jv", Z12, V2[1:])
    my = np.einsum("jkv,kv->jv", Z21, V1[1:]) + np.einsum("jkv,kv->jv", Z22, V2[1:])
    mv = np.vstack([_unsort(mx, sv[4]), _unsort(my, sv[4])])
    mv = rotation_op(mv, -sv[1], np.zeros((2, nv)))
    return Xold + dt * vinf - dt * mv


def relax_w_net(nets, Xmid, dt):
    """relaxWTorchNet (:3622-3629)."""
    Xin, sv = standardization_step(Xmid)
    return destandardize(nets.relax(Xin, dt), sv)


def mlarm_step(nets, Xold, ten_old, area0, len0, dt=1e-5, speed=2.0, kappa=1.0, record=None):
    """time_step_many_noinfo (:986-1206) with shear background flow
    ``speed * (y, 0)`` and no repulsion.  Returns (Xnew, tenNew)."""
    rec = record if record is not None else {}
    N, nv = Xold.shape[0] // 2, Xold.shape[1]
    vback = O.bg_flow(Xold, "shear", speed)
    f_ten = tension_term(Xold, ten_old)
    f_bend = bending_upsampled(Xold, kappa)
    Xs, sv = standardization_step(Xold)
    rec["stand_X"], rec["sv"] = Xs, sv
    far1, excl = far_field(Xold, f_bend + f_ten)
    rec["far1"], rec["excl"] = far1, excl
    far1 = O.filter_shape(far1, 16)
    vback_solve = inv_ten_mat_on_vback(nets, Xs, sv, vback + far1)
    selfbend_solve = inv_ten_mat_on_self_bend(nets, Xs, sv)
    rec["vback_solve"], rec["selfbend_solve"] = vback_solve, selfbend_solve
    ten_new = -(vback_solve + selfbend_solve)
    trac = f_bend + tension_term(Xold, ten_new)
    far2, _ = far_field(Xold, trac, excl)
    rec["far2"] = far2
    far2 = O.filter_shape(far2, 16)
    Xadv = translate_vinf(nets, Xold, Xs, sv, vback + far2, dt)
    rec["Xadv"] = Xadv
    Xadv = O.filter_shape(Xadv, 16)
    Xnew = relax_w_net(nets, Xadv, dt)
    rec["Xrelax"] = Xnew
    XnewC = Xnew.copy()
    for _ in range(5):
        Xnew, good = O.redistribute_arc_length(Xnew)
        if good:
            break
    Xnew = O.align_center_angle(XnewC, Xnew)
    rec["Xalign"] = Xnew
    Xnew = O.correct_area_length(Xnew, area0, len0)
    rec["Xcorr"] = Xnew
    return O.filter_shape(Xnew, 16), ten_new
