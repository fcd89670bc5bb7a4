"""The k-epsilon model (iturb = -1): kepsilon source (src/turbsource_module.f90:170-267),
its low-Re eddy viscosity (src/eddy_module.f90), sigma_k = 1, sigma_eps = 1.3 in the
viscous flux (src/vsflux_module.f90:69-75), the bcwallviscouske wall and the k-epsilon
reference values of config%setref, through the C ABI against the CPU oracle."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native
from tests.helpers import field_err, interior

pytestmark = pytest.mark.gpu

TOL_RES = 1e-9
TOL_STATE = 1e-9
TOL_MIXED = 1e-5


def make(name, **kw):
    """an SST case turned k-epsilon: eps = 0.09 k omega for the state and the free stream"""
    c = cases.make(name, **kw)
    cfg = c["cfg"]
    cfg.update(iturb=-1, fix_cav_clamp=1)
    if cfg.get("kinf", 0) > 0 and cfg.get("oinf", 0) > 0:
        cfg["oinf"] = 0.09 * cfg["kinf"] * cfg["oinf"]
    for pv in c["pv0"]:
        pv[..., 8] = 0.09 * pv[..., 7] * pv[..., 8]
    return c


CASES = {"steady_block": ("adjoint", dict(scale=8)), "bdf2_wall": ("large", dict(scale=16))}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("timemethod", [3, 2])
def test_ke_matches_oracle(oracle, name, timemethod):
    c = make(CASES[name][0], **CASES[name][1])
    c["cfg"]["timemethod"] = timemethod
    if timemethod != 3:
        c["cfg"]["cfl"] = 0.5
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
        assert np.all(np.isfinite(resg))
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    sg, so = e.download(0), o.get_state(0)
    assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL_STATE
    assert field_err(interior(sg["tv"]), interior(so["tv"])).max() < TOL_STATE
    # the wall's ghost layers (j = -1, 0, 1) of the bcwallviscouske patch
    assert field_err(sg["pv"][3:-3, :3, 3:-3], so["pv"][3:-3, :3, 3:-3]).max() < TOL_STATE


def test_ke_mixed_residual(oracle):
    c = make("large", scale=16)
    e = native.Engine(c, precision=abi.MIXED)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    assert field_err(e.residual(0)["res"], o.residual(0)["res"]).max() < TOL_MIXED
    for it in range(3):
        _, resg, _ = e.iterate(1, it + 1, 0.0)
        _, reso, _ = o.iterate(1, it + 1, 0.0)
        big = reso > 1e-6 * reso.max()
        assert np.allclose(resg[big], reso[big], rtol=2e-2), (it, resg, reso)


def test_ke_reference_values():
    """config%setref: k = 1.5 (1e-4 U)^2, mu_t = 1e-5 mu, eps = 0.09 rho k^2 / mu_t -- the
    initial eddy viscosity is the reference mu_t"""
    c = make("adjoint", scale=8)
    c["cfg"].update(kinf=0.0, oinf=0.0)
    e = native.Engine(c)
    e.initialize(None)
    s = e.download(0)
    mu = interior(s["tv"])[..., 0]
    mut = interior(s["tv"])[..., 2]
    assert np.allclose(mut, 1e-5 * mu.mean(), rtol=1e-6)
    u = c["cfg"]["uref"]
    assert np.allclose(interior(s["pv"])[..., 7], 1.5 * (1e-4 * u) ** 2, rtol=1e-12)


def test_ke_unsupported_paths():
    c = make("adjoint", scale=8)
    e = native.Engine(c)
    e.initialize(c["pv0"])
    with pytest.raises(native.Cfd3dError) as ei:
        e.residual_vjp([np.zeros(abi.interior_shape(c["blocks"][0], 9))])
    assert ei.value.code == abi.ERR_ARG
    c2 = make("adjoint", scale=8)
    b = c2["blocks"][0]
    im, jm, km = b["imax"], b["jmax"], b["kmax"]
    b["bc"] = [(abi.BC_WALL_COUNTERROTATING if tuple(p) == (1, 1, 1, im, 1, km) else k, p) for k, p in b["bc"]]
    with pytest.raises(native.Cfd3dError) as ei:
        native.Engine(c2)
    assert ei.value.code == abi.ERR_DESCRIPTOR
