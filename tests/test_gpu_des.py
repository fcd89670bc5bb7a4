"""DES length scales of the SST destruction term (ides 1-4: sst_des, sst_ddes, sst_iddes,
sst_s_iddes; src/turbsource_module.f90:416-576) through the C ABI against the CPU oracle,
in both arithmetic forms, and the discrete adjoint through them against finite
differences."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native
from tests.helpers import field_err, interior

pytestmark = pytest.mark.gpu

TOL_RES = 1e-9
TOL_STATE = 1e-9
TOL_MIXED = 1e-5


def make(ides):
    """the SST block with omega lowered 20-fold, so that the RANS length sqrt(k)/(0.09 omega)
    exceeds the LES length 0.61 h in places and every variant changes the destruction"""
    c = cases.make("adjoint", scale=8)
    c["cfg"].update(ides=ides, fix_cav_clamp=1)
    c["pv0"][0][..., 8] /= 20.0
    return c


@pytest.mark.parametrize("ides", [1, 2, 3, 4])
def test_des_residual_and_iterations_match(oracle, ides):
    c = make(ides)
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    rg, ro = e.residual(0), o.residual(0)
    assert field_err(rg["res"], ro["res"]).max() < TOL_RES
    assert field_err(rg["itt"], ro["itt"]).max() < TOL_RES
    for it in range(3):
        _, resg, _ = e.iterate(1, it + 1, 0.0)
        _, reso, _ = o.iterate(1, it + 1, 0.0)
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    assert field_err(interior(e.download(0)["pv"]), interior(o.get_state(0)["pv"])).max() < TOL_STATE


def test_des_changes_the_destruction():
    """every DES variant differs from the RANS length scale on this state"""
    r0 = None
    for ides in range(5):
        c = make(ides)
        e = native.Engine(c)
        e.initialize(c["pv0"])
        r = e.residual(0)["res"][..., 7]
        if r0 is None:
            r0 = r
        else:
            assert np.abs(r - r0).max() > 1e-9 * np.abs(r0).max(), ides


@pytest.mark.parametrize("ides", [2, 3])
def test_des_mixed_residual(oracle, ides):
    c = make(ides)
    e = native.Engine(c, precision=abi.MIXED)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    assert field_err(e.residual(0)["res"], o.residual(0)["res"]).max() < TOL_MIXED


def test_des_rejects_an_unknown_variant():
    with pytest.raises(native.Cfd3dError) as ei:
        native.Engine(make(5))
    assert ei.value.code == abi.ERR_ARG


def test_vjp_through_ddes():
    """(dR/dpv)^T lambda with the DDES length scale against central differences of the GPU
    residual, at the k and omega rows where the destruction term acts"""
    from cfd3d_gb300 import adjoint
    from tests.test_gpu_adjoint import _check, _entries, _state
    c = _state(4)
    c["cfg"]["ides"] = 2
    c["pv0"][0][..., 8] /= 20.0
    e = native.Engine(c)
    e.initialize(c["pv0"])
    s = adjoint.StateSetter(e)
    pv = s.interior(0)
    res = s.residual([pv])[0]
    rng = np.random.default_rng(9)
    scale_v = np.abs(res).reshape(-1, res.shape[-1]).max(axis=0)
    lam = rng.normal(size=res.shape) / np.maximum(scale_v, 1e-300)
    g, _ = e.residual_vjp([lam])
    d = dict(pv=pv, lam=lam, g=g[0])
    entries = [(k, j, i, 7 + (q % 2)) for q, (k, j, i, _) in enumerate(_entries(pv.shape[:-1], pv.shape[-1], 14, 6))]
    used, errs, rows = _check(lambda p: s.residual([p])[0], d, entries)
    print(f"DDES rows: {used}/{len(entries)} entries, max relative error {errs.max():.2e}")
    assert used >= len(entries) - 2, rows
    assert errs.max() <= 1e-6, (errs, rows)
