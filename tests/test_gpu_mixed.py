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


# mixed against FP64 form, one iteration from the same state: per-cell state difference,
# normalised by each variable's largest value.  The FP32 neighbour products and FP32 diagonal
# correction of the sweeps, the FP32 fluxes and the FP32 time step move dq by a small
# fraction of itself; a missing or misplaced neighbour contribution moves it by its whole
# size (~1e-2 of the state's scale), which this bound catches.
TOL_FIELD_ONE_ITERATION = 2e-3


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_state_follows_fp64(name):
    c = make(name)
    e64 = native.Engine(c, precision=abi.FP64)
    emx = native.Engine(c, precision=abi.MIXED)
    e64.initialize(c["pv0"])
    emx.initialize(c["pv0"])
    e64.iterate(1, 1, 0.0)
    emx.iterate(1, 1, 0.0)
    worst = 0.0
    for b in range(len(c["blocks"])):
        a = emx.download(b)["pv"][3:-3, 3:-3, 3:-3]
        r = e64.download(b)["pv"][3:-3, 3:-3, 3:-3]
        worst = max(worst, field_err(a, r).max())
    print(f"{name}: mixed vs FP64 state after one iteration {worst:.2e}")
    assert worst < TOL_FIELD_ONE_ITERATION, worst


def test_mixed_iterations_are_deterministic():
    """two engines, same state, same iterations: the same state bit for bit (the tile
    sweeps' result does not depend on which warp took which tile when)"""
    c = make("batched_multiblock")
    out = []
    for _ in range(2):
        e = native.Engine(c, precision=abi.MIXED)
        e.initialize(c["pv0"])
        for it in range(3):
            e.iterate(1, it + 1, 0.0)
        out.append([e.download(b)["pv"] for b in range(len(c["blocks"]))])
        e.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
