"""Double layer of vesicles with a viscosity contrast: the oracle's
restatements against the reference (golden dl_fp64), CPU only."""
import numpy as np

from oracle import ves2d_oracle as O


def rel(a, b):
    return np.max(np.abs(np.asarray(a) - b)) / max(np.max(np.abs(b)), 1e-300)


def test_oracle_dl_matches_reference(golden):
    g = golden("dl_fp64")
    for tag in ("n32", "n128"):
        X, visc, f = g[f"X_{tag}"], g[f"visc_{tag}"], g[f"f_{tag}"]
        N = X.shape[0] // 2
        tab = O.PotenTables(N)
        D = O.stokes_dl_matrix(X, visc, tab)
        assert rel(D, g[f"D_{tag}"]) < 1e-11, tag
        # D vanishes exactly for the vesicles without a contrast
        for k, v in enumerate(visc):
            if v == 1:
                assert np.all(g[f"D_{tag}"][:, :, k] == 0) and np.all(D[:, :, k] == 0)
        assert rel(O.exact_stokes_sl_diag(D, f), g[f"DLdiag_{tag}"]) < 1e-11
        sa, tang, _ = O.diff_prop(X)
        assert rel(O.exact_stokes_dl(X, tang, sa, f, visc, g[f"Xtar_{tag}"]), g[f"DL_{tag}"]) < 1e-12
        # nearSingInt's far-field loop over the upsampled sources (no near pairs here)
        assert rel(O.near_sing_int_dl(X, f, None, visc, tab, "none"), g[f"far_{tag}"]) < 1e-12


def test_oracle_dl_schemes_reduce_to_far_field_without_near_pairs(golden):
    """Both near-field rules leave the far field untouched when no pair is near."""
    g = golden("dl_fp64")
    X, visc, f = g["X_n32"], g["visc_n32"], g["f_n32"]
    N = X.shape[0] // 2
    tab = O.PotenTables(N)
    vself = f * (0.5 * (1 - visc))[None, :] + O.exact_stokes_sl_diag(O.stokes_dl_matrix(X, visc, tab), f)
    near = O.naive_near_zone_info(X, O.interpft_vec(X, tab.Nup))
    entries, h = O.get_zone(X)
    assert len(near[4][0]) == 0 and len(entries) == 0
    far = g["far_n32"]
    assert rel(O.near_sing_int_dl(X, f, vself, visc, tab, "py_hh", near=near), far) < 1e-12
    assert rel(O.near_sing_int_dl(X, f, vself, visc, tab, "matlab", entries=entries, h=h), far) < 1e-12
