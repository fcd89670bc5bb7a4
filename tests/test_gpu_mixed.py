"""The mixed-precision form (CFD3D_MIXED) against the CPU oracle.

FP32 reconstruction, limiter and flux arithmetic on a gauge shadow of the state, IF97
sums in df64, FP64 mixture EOS, accumulation, implicit operator and update.  The bar is
the residual on an identical state: max over cells of |R_mixed - R_oracle| divided by the
largest |R_oracle| of the same variable, at most 1e-5.  Iterated states are compared only
loosely: a precision change moves states across the discrete switches of the scheme
(limiter branches, y1 = 0 clips, upwind direction), so trajectories separate by more
than the per-evaluation error.
"""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native
from tests.helpers import field_err

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-5

CASES = {
    "plain_roe_tvd": ("plain_small", dict(scale=2), {}),
    "plain_roem_mlp": ("plain_small", dict(scale=2), dict(nscheme=2, nmuscl=2, nlim=8)),
    "plain_ausmpw_vl": ("plain_small", dict(scale=2), dict(nscheme=3, nmuscl=1, nlim=3)),
    "plain_ausmup_first": ("plain_small", dict(scale=2), dict(nscheme=4, nmuscl=0)),
    "cavitating": ("cavitating", dict(scale=4), dict(fix_cav_clamp=1)),
    "adjoint_sst": ("adjoint", dict(scale=4), dict(fix_cav_clamp=1)),
    "large_sst_bdf2": ("large", dict(scale=8), dict(fix_cav_clamp=1)),
    "batched_multiblock": ("batched", dict(scale=4, nblocks=6), dict(fix_cav_clamp=1)),
}


def make(name):
    base, kw, over = CASES[name]
    c = cases.make(base, **kw)
    c["cfg"].update(over)
    return c


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_residual_within_tolerance(oracle, name):
    c = make(name)
    e = native.Engine(c, precision=abi.MIXED)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    worst = 0.0
    for b in range(len(c["blocks"])):
        err = field_err(e.residual(b)["res"], o.residual(b)["res"]).max()
        worst = max(worst, err)
    assert worst < TOL_MIXED, (name, worst)


@pytest.mark.parametrize("name", ["cavitating", "large_sst_bdf2", "batched_multiblock"])
def test_mixed_iterations_follow_fp64(oracle, name):
    c = make(name)
    e = native.Engine(c, precision=abi.MIXED)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    for it in range(5):
        _, resg, _ = e.iterate(1, it + 1, 0.0)
        _, reso, _ = o.iterate(1, it + 1, 0.0)
        assert np.all(np.isfinite(resg))
        big = reso > 1e-6 * reso.max()
        assert np.allclose(resg[big], reso[big], rtol=2e-2), (it, resg, reso)
