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
