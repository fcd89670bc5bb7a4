"""Comparison helpers shared by the parity tests."""
import numpy as np


def interior(a):
    """Interior cells 2..imax of a padded array (k, j, i, v) laid out -1..imax+3."""
    return a[3:-3, 3:-3, 3:-3]


def field_err(x, y, axis_var=-1):
    """Max over variables of max|x - y| / max(max|y|, tiny), per variable scale."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    nv = y.shape[axis_var]
    errs = []
    for v in range(nv):
        yv = np.take(y, v, axis=axis_var)
        xv = np.take(x, v, axis=axis_var)
        scale = max(np.abs(yv).max(), 1e-300)
        if not np.any(yv) and not np.any(xv):
            errs.append(0.0)
            continue
        errs.append(np.abs(xv - yv).max() / scale)
    return np.array(errs)


def rel_err(x, y, floor=1e-300):
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    return np.abs(x - y) / np.maximum(np.abs(y), floor)


# the update's EOS against the oracle's at the same state (as the pointwise EOS test)
TOL_EOS = 1e-11
# stiffened water + ideal vapour: the sound-speed denominator cancels (all dh/dp = 0)
TOL_EOS_STIFFENED = 2e-9


def dv_eos_err(pv_interior, dv_interior, cfg):
    """The largest relative difference between an engine's interior dv and the oracle's
    EOS of the same engine's pv.  Iterated states are compared this way rather than dv
    against dv: the mixture sound speed of a cell holding a trace of vapour (y1 ~ 1e-11)
    moves with y1 far more than y1 itself does, so two trajectories whose pv agree to
    rounding may hold sound speeds further apart while each dv is the EOS of its state.
    Returns (error, tolerance)."""
    from oracle import oracle_py
    npv = pv_interior.shape[-1]
    pv = np.asarray(pv_interior).reshape(-1, npv)
    pref = float(cfg["pref"])
    dv_eos, _ = oracle_py.eos(pv[:, 0] + pref, pv[:, 4], pv[:, 5], pv[:, 6], fluid=int(cfg["fluid"]),
                              prop=int(cfg["iturb"]) != -3)
    dv = np.asarray(dv_interior).reshape(-1, dv_eos.shape[-1])
    tol = TOL_EOS_STIFFENED if int(cfg["fluid"]) == 1 else TOL_EOS
    return float(np.max(rel_err(dv, dv_eos, floor=1e-30))), tol
