"""The surface-tension source (csf = 1; src/csf_module.f90:97-175, the volume-fraction
gradient of src/variable_module.f90:304-377 and its halo setbc_vfg, src/bc_module.f90
:1398-1804) through the C ABI against the CPU oracle: the residual and the stored source,
iterations, the two-block halo, the mixed form, the checkpoint record and the adjoint's
refusal.  The cavitating start's vapour sphere gives |grad vf| well above the reference's
interface threshold 0.04, so the source is active there."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native
from oracle import oracle_checkpoint as ock
from tests.helpers import dv_eos_err, field_err, interior

pytestmark = pytest.mark.gpu

TOL = 1e-9
# mixed form against the FP64 form on the same state, as the mixed-form tests bound it
TOL_MIXED = 1e-5


def _case(base="cavitating", **kw):
    kw.setdefault("scale", 8)
    c = cases.make(base, **kw)
    c["cfg"]["csf"] = 1
    c["cfg"]["fix_cav_clamp"] = 1
    return c


def _pair(c):
    from oracle import oracle_py
    e = native.Engine(c)
    o = oracle_py.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    return e, o


@pytest.mark.parametrize("base,kw", [("cavitating", {}), ("batched", dict(scale=4, nblocks=6)),
                                     ("large", dict(scale=16))])
def test_residual_and_source_match(base, kw):
    c = _case(base, **kw)
    e, o = _pair(c)
    active = 0.0
    for b in range(len(c["blocks"])):
        rg, ro = e.residual(b), o.residual(b)
        assert field_err(rg["res"], ro["res"]).max() < TOL
        cg, co = e.download_csf(b), o.get_csf(b)["csf"]
        scale = max(np.abs(co).max(), 1e-300)
        assert np.abs(cg - co).max() <= TOL * scale
        active = max(active, np.abs(co).max())
    if base == "cavitating":
        assert active > 0.0


def test_iterations_match():
    c = _case()
    e, o = _pair(c)
    for it in range(3):
        _, resg, _ = e.iterate(1, it + 1, 0.0)
        _, reso, _ = o.iterate(1, it + 1, 0.0)
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    sg, so = e.download(0), o.get_state(0)
    assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL
    err, tol = dv_eos_err(interior(sg["pv"]), interior(sg["dv"]), c["cfg"])
    assert err < tol
    assert np.abs(e.download_csf(0) - o.get_csf(0)["csf"]).max() <= TOL * np.abs(o.get_csf(0)["csf"]).max()


def test_mixed_form_residual():
    c = _case()
    e64 = native.Engine(c)
    emx = native.Engine(c, precision=abi.MIXED)
    for e in (e64, emx):
        e.initialize(c["pv0"])
    r64, rmx = e64.residual(0)["res"], emx.residual(0)["res"]
    assert field_err(rmx, r64).max() < TOL_MIXED
    # The source itself is not compared cell by cell: the reference's curvature sums the
    # unit normals vfg / |vfg| of the six neighbours, and next to the interface a neighbour's
    # vfg is a rounding-level vector whose direction the two forms' last bits decide; only
    # that the source is there is checked (the residual bound above covers its effect).
    assert np.abs(emx.download_csf(0)).max() > 0.0


def test_checkpoint_carries_the_source(tmp_path):
    c = _case()
    e = native.Engine(c)
    e.initialize(c["pv0"])
    t, _, _ = e.iterate(1, 1, 0.0)
    path = tmp_path / "out_00000001.dat"
    e.checkpoint_write(str(path), 1, 1, t)
    s = e.download(0)
    want = ock.write_checkpoint(tmp_path / "oracle.dat", c["cfg"], c["blocks"], e.npv, e.nqq, 1, 1, t,
                                [dict(pv=s["pv"], tv=s["tv"], qq=s["qq"][..., :e.nqq * e.npv], rcav=s["rcav"],
                                      csf=e.download_csf(0))])
    assert path.read_bytes() == want
    # the reader restores the stored source with the state
    r = native.Engine(c)
    r.checkpoint_read(str(path))
    assert np.array_equal(r.download_csf(0), e.download_csf(0))


def test_adjoint_declines_and_csf_download_needs_the_source():
    c = _case()
    e = native.Engine(c)
    e.initialize(c["pv0"])
    lam = np.ones(e.residual(0)["res"].shape)
    with pytest.raises(native.Cfd3dError) as ei:
        e.residual_vjp([lam])
    assert ei.value.code == abi.ERR_ARG
    plain = native.Engine(cases.make("cavitating", scale=8))
    with pytest.raises(native.Cfd3dError) as ei:
        plain.download_csf(0)
    assert ei.value.code == abi.ERR_ARG
