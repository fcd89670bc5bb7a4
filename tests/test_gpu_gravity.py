"""The gravity source (rhs%gravity, src/gravity_module.f90): a constant acceleration along an
axis (gravity = +-1..+-3) or the history of gravity.dat (gravity = 4, read at the
residual's time), through the C ABI against the CPU oracle, in both forms, and through
the discrete adjoint."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native
from tests.helpers import field_err, interior

pytestmark = pytest.mark.gpu

TOL_RES = 1e-9
TOL_STATE = 1e-9
TOL_MIXED = 1e-5

BASES = {
    "plain": ("plain_small", dict(scale=4), {}),
    "cavitating": ("cavitating", dict(scale=8, fix_cav_clamp=1), {}),
    "sst_bdf2": ("large", dict(scale=16), dict(fix_cav_clamp=1)),
}


def make(base, gravity, history=None):
    name, kw, over = BASES[base]
    c = cases.make(name, **kw)
    c["cfg"].update(over)
    c["cfg"]["gravity"] = gravity
    if history is not None:
        c["cfg"]["gravity_data"] = np.asarray(history, dtype=np.float64)
    return c


def _compare(oracle, c, steps):
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    assert field_err(e.residual(0)["res"], o.residual(0)["res"]).max() < TOL_RES
    for it, nt_phy in enumerate(steps):
        _, resg, _ = e.iterate(nt_phy, it + 1, 0.0)
        _, reso, _ = o.iterate(nt_phy, it + 1, 0.0)
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    for b in range(len(c["blocks"])):
        assert field_err(interior(e.download(b)["pv"]), interior(o.get_state(b)["pv"])).max() < TOL_STATE
    return e


@pytest.mark.parametrize("gravity", [-2, 3])
@pytest.mark.parametrize("base", list(BASES))
def test_constant_gravity_matches(oracle, base, gravity):
    _compare(oracle, make(base, gravity), [1, 1, 1])


def test_gravity_history_matches(oracle):
    """the history read at dt_phy nt_phy: between rows, then past the last row"""
    c = make("sst_bdf2", 4)
    dtp = c["cfg"]["dt_phy"]
    c["cfg"]["gravity_data"] = np.array([[0.0, 0.0, -9.8, 0.0], [1.5 * dtp, 2.0, -4.0, 1.0], [3.0 * dtp, 0.0, 0.0, 5.0]])
    _compare(oracle, c, [1, 2, 4])


def test_gravity_changes_the_momentum_residual():
    c0, c1 = make("plain", 0), make("plain", -2)
    r = []
    for c in (c0, c1):
        e = native.Engine(c)
        e.initialize(c["pv0"])
        r.append(e.residual(0)["res"])
    d = r[1] - r[0]
    assert np.abs(d[..., 2]).max() > 0.0          # the y-momentum row
    assert np.abs(d[..., 1]).max() == 0.0 and np.abs(d[..., 3]).max() == 0.0


def test_mixed_gravity_residual(oracle):
    c = make("sst_bdf2", -2)
    e = native.Engine(c, precision=abi.MIXED)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    assert field_err(e.residual(0)["res"], o.residual(0)["res"]).max() < TOL_MIXED


def test_gravity_rejects_bad_settings():
    for g, hist in ((5, None), (4, None), (4, [[1.0, 0, 0, 0], [0.5, 0, 0, 0]])):
        with pytest.raises(native.Cfd3dError) as ei:
            native.Engine(make("plain", g, hist))
        assert ei.value.code == abi.ERR_ARG


def test_vjp_with_gravity():
    from cfd3d_gb300 import adjoint
    from tests.test_gpu_adjoint import _check, _entries, _state
    c = _state(4)
    c["cfg"]["gravity"] = -2
    e = native.Engine(c)
    e.initialize(c["pv0"])
    s = adjoint.StateSetter(e)
    pv = s.interior(0)
    res = s.residual([pv])[0]
    rng = np.random.default_rng(13)
    scale_v = np.abs(res).reshape(-1, res.shape[-1]).max(axis=0)
    lam = rng.normal(size=res.shape) / np.maximum(scale_v, 1e-300)
    g, _ = e.residual_vjp([lam])
    d = dict(pv=pv, lam=lam, g=g[0])
    entries = _entries(pv.shape[:-1], pv.shape[-1], 18, 7)
    used, errs, rows = _check(lambda p: s.residual([p])[0], d, entries)
    print(f"gravity rows: {used}/{len(entries)} entries, max relative error {errs.max():.2e}")
    assert used >= len(entries) - 2, rows
    assert errs.max() <= 1e-6, (errs, rows)
