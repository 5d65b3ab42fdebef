"""Pin the FP64 oracle against fixtures recorded from the reference itself.

The fixtures were produced by ``tests/golden/make_golden.py`` running the
reference ``mytorch/`` code with its FP32 casts promoted to FP64; the oracle
must reproduce them to round-off.  The ``*_mixed`` fixtures are the
reference's own mixed FP32/FP64 arithmetic and are compared at FP32 level.
"""
import numpy as np
import pytest

from oracle import ves2d_oracle as O


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("N", [16, 32])
def test_capsule_ops(golden, N):
    g = golden("capsules_fp64")
    X, sig, f = g[f"X{N}"], g[f"sig{N}"], g[f"f{N}"]
    ves = O.Capsule(X)
    assert rel(ves.sa, g[f"sa{N}"]) < 1e-13
    assert rel(ves.xt, g[f"xt{N}"]) < 1e-13
    assert rel(ves.cur, g[f"cur{N}"]) < 1e-12
    assert rel(ves.trac_jump(X, sig), g[f"trac{N}"]) < 1e-11
    assert rel(ves.surface_div(f), g[f"sdiv{N}"]) < 1e-12
    Ben, Ten, Div = ves.compute_derivs()
    assert rel(Ben, g[f"Ben{N}"]) < 1e-10
    assert rel(Ten, g[f"Ten{N}"]) < 1e-12
    assert rel(Div, g[f"Div{N}"]) < 1e-12
    ra, area, length = O.geom_prop(X)
    assert rel(area, g[f"area{N}"]) < 1e-13 and rel(length, g[f"len{N}"]) < 1e-13
    tab = O.PotenTables(N)
    assert rel(O.interpft_vec(X, tab.Nup), g[f"up{N}"]) < 1e-13


@pytest.mark.parametrize("N", [16, 32])
def test_alpert_matrix(golden, N):
    g = golden("capsules_fp64")
    tab = O.PotenTables(N)
    assert rel(tab.qw, g[f"qw{N}"]) < 1e-14
    assert rel(tab.qp, g[f"qp{N}"]) < 1e-12
    assert rel(tab.R, g[f"Rlp{N}"]) < 1e-12
    assert rel(tab.P, g[f"Plp{N}"]) < 1e-12
    G = O.stokes_sl_matrix(g[f"X{N}"], tab)
    assert rel(G, g[f"G{N}"]) < 1e-11


def test_alpert_matrix_vs_mixed_reference(golden):
    """The reference's own FP32 G agrees with the FP64 restatement at FP32 level."""
    g = golden("capsules_mixed")
    G = O.stokes_sl_matrix(g["X32"], O.PotenTables(32))
    assert rel(G, g["G32"]) < 1e-4  # the reference builds G in FP32


def test_near_zone_and_far_field(golden):
    g = golden("far_fp64")
    X, f = g["X"], g["f"]
    N = X.shape[0] // 2
    tab = O.PotenTables(N)
    Xup = O.interpft_vec(X, tab.Nup)
    assert rel(Xup, g["Xup"]) < 1e-13
    near = O.naive_near_zone_info(X, Xup)
    for got, key in [(near[2][0], "id1"), (near[2][1], "id2"), (near[3][0], "id1_hh"),
                     (near[3][1], "id2_hh"), (near[4][0], "ids0"), (near[4][1], "ids1"), (near[4][2], "ids2")]:
        np.testing.assert_array_equal(got, g[key])
    np.testing.assert_array_equal(near[1], g["idx_closest"])
    # torch.cdist uses the |x|^2+|y|^2-2x.y form, accurate to ~sqrt(eps)*|x| absolute
    assert np.max(np.abs(near[0] - g["closest_dist"])) < 1e-7
    sa_up = O.diff_prop(Xup)[0]
    fup = O.interpft_vec(f, tab.Nup)
    far2 = O.all_exact_stokes_sl_target(Xup, sa_up, fup, X, near[4])
    assert rel(far2, g["far2"]) < 1e-12
    far0 = O.all_exact_stokes_sl_target(Xup, sa_up, fup, X, None)
    assert rel(far0, g["far_noexcl"]) < 1e-12
    c1 = O.compare1_exclusions(Xup, X)
    for got, key in zip(c1, ["c1_ids0", "c1_ids1", "c1_ids2"]):
        np.testing.assert_array_equal(got, g[key])
    far1 = O.all_exact_stokes_sl_target(Xup, sa_up, fup, X, c1)
    assert rel(far1, g["far1"]) < 1e-12
    sl = O.exact_stokes_sl_points(X, O.diff_prop(X)[0], f, X[:, :1], list(range(1, X.shape[1])))
    assert rel(sl, g["exact_sl_col0"]) < 1e-12


def test_near_sing_int_hh(golden):
    g = golden("step_near_fp64")
    X, f = g["X0"], g["f_near"]
    N = X.shape[0] // 2
    tab = O.PotenTables(N)
    G = O.stokes_sl_matrix(X, tab)
    vself = O.exact_stokes_sl_diag(G, f)
    near = O.naive_near_zone_info(X, O.interpft_vec(X, tab.Nup))
    assert len(near[4][0]) == int(g["n_near"]) and len(near[3][0]) == int(g["n_hh"])
    LP, nearf = O.near_sing_int_hh(X, f, vself, near, tab)
    assert rel(nearf, g["nearField"]) < 1e-11
    assert rel(LP, g["LP_near"]) < 1e-11


@pytest.mark.parametrize("fixture", ["step_c1_fp64", "step_near_fp64"])
def test_time_step(golden, fixture):
    g = golden(fixture)
    X = g["X0"]
    N, nv = X.shape[0] // 2, X.shape[1]
    prm = O.StepParams(dt=float(g["dt"]), speed=float(g["speed"]), gmres_tol=1e-10, gmres_maxiter=200)
    tab = O.PotenTables(N)
    sig = np.zeros((N, nv))
    nsteps = sum(1 for k in g.files if k.startswith("iter"))   # config 1: its 10 steps
    for s in range(1, nsteps + 1):
        res = O.time_step(X, sig, prm, tab)
        assert res.iters == int(g[f"iter{s}"])
        assert not res.iflag
        assert rel(res.X, g[f"X{s}"]) < 1e-12
        assert rel(res.sigma, g[f"sig{s}"]) < 1e-8
        X, sig = res.X, res.sigma


def test_time_step_vs_mixed_reference(golden):
    """The reference's native mixed-precision step is within FP32 error of FP64."""
    g = golden("step_c1_mixed")
    X = g["X0"]
    N, nv = X.shape[0] // 2, X.shape[1]
    prm = O.StepParams(dt=float(g["dt"]), speed=float(g["speed"]))
    res = O.time_step(X, np.zeros((N, nv)), prm, O.PotenTables(N))
    assert rel(res.X, g["X1"]) < 1e-6


@pytest.mark.parametrize("tag", ["unit", "big"])
def test_post_step_conditioning(golden, tag):
    g = golden("post_fp64")
    X = g[f"X_{tag}"]
    assert rel(O.physical_center(X), g[f"center_{tag}"]) < 1e-12
    assert np.max(np.abs(O.inc_angle(X) - g[f"incangle_{tag}"])) < 1e-12
    X1, _ = O.redistribute_arc_length(X)
    X5 = X.copy()
    for _ in range(5):
        X5, _ = O.redistribute_arc_length(X5)
    tol = 1e-10 if tag == "unit" else 1e-6
    assert rel(X1, g[f"redist1_{tag}"]) < tol
    assert rel(X5, g[f"redist5_{tag}"]) < tol
    assert rel(O.align_center_angle(X, g[f"redist5_{tag}"]), g[f"align_{tag}"]) < 1e-10
    Xc = O.correct_area_length(g[f"pert_{tag}"], g[f"a0_{tag}"], g[f"l0_{tag}"])
    assert rel(Xc, g[f"corrected_{tag}"]) < 1e-9


def test_bg_flow(golden):
    """bg_flow (mytorch/tstep_biem.py:849-952), every unconfined kind."""
    g = golden("bgflow_fp64")
    for kind in g["kinds"]:
        v = O.bg_flow(g["X"], str(kind), speed=1.7, chan_width=2.3, vortex_size=1.9)
        assert rel(v, g[f"v_{kind}"]) < 1e-14, kind
