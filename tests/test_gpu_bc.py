"""Characteristic inflow / outflow boundaries through the C ABI against the CPU oracle:
bcinflowsubsonic, bcoutflowsubsonic and bcinflowsupersonic (src/bc_module.f90:2464-2869),
on single-phase Euler, cavitating laminar and SST cases, in both arithmetic forms."""
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
    "sst": ("large", dict(scale=16), dict(fix_cav_clamp=1, nsteady=0)),
}
BCSETS = {
    "subsonic": {"imin": abi.BC_INFLOW_SUBSONIC, "imax": abi.BC_OUTFLOW_SUBSONIC},
    "supersonic_in": {"imin": abi.BC_INFLOW_SUPERSONIC, "imax": abi.BC_EXTRAPOLATE},
    "out_only": {"imin": abi.BC_FARFIELD, "imax": abi.BC_OUTFLOW_SUBSONIC},
    # bcmassflowratein at the inlet; counter-rotating walls (the SST case's wall, and the
    # others' j faces); bcshiftedperiodic on the k faces (their 16-cell shift needs 17 cells)
    "massflow_crwall": {"imin": abi.BC_MASSFLOWRATE_IN, "jmin": abi.BC_WALL_COUNTERROTATING},
}
SHIFTED = {"kmin": abi.BC_SHIFTED_PERIODIC, "kmax": abi.BC_SHIFTED_PERIODIC}


def replace_faces(c, kinds):
    """the case with the BC of the named faces of every block replaced"""
    for b in c["blocks"]:
        im, jm, km = b["imax"], b["jmax"], b["kmax"]
        faces = {"imin": (1, 1, 1, 1, jm, km), "imax": (im, 1, 1, im, jm, km),
                 "jmin": (1, 1, 1, im, 1, km), "jmax": (1, jm, 1, im, jm, km),
                 "kmin": (1, 1, 1, im, jm, 1), "kmax": (1, 1, km, im, jm, km)}
        bc = []
        for kind, pnts in b["bc"]:
            face = next((f for f, p in faces.items() if tuple(p) == tuple(pnts)), None)
            bc.append((kinds[face], pnts) if face in kinds else (kind, pnts))
        b["bc"] = bc
    return c


def make(base, bcset):
    name, kw, over = BASES[base]
    c = cases.make(name, **kw)
    c["cfg"].update(over)
    return replace_faces(c, BCSETS[bcset])


@pytest.mark.parametrize("bcset", list(BCSETS))
@pytest.mark.parametrize("base", list(BASES))
def test_residual_and_iterations_match(oracle, base, bcset):
    c = make(base, bcset)
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    for b in range(len(c["blocks"])):
        assert field_err(e.residual(b)["res"], o.residual(b)["res"]).max() < TOL_RES
    for it in range(3):
        _, resg, _ = e.iterate(1, it + 1, 0.0)
        _, reso, _ = o.iterate(1, it + 1, 0.0)
        assert np.all(np.isfinite(resg))
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    for b in range(len(c["blocks"])):
        sg, so = e.download(b), o.get_state(b)
        assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL_STATE
        # the ghost layers the boundary program writes
        assert field_err(sg["pv"][3:-3, 3:-3, :3], so["pv"][3:-3, 3:-3, :3]).max() < TOL_STATE
        assert field_err(sg["pv"][3:-3, 3:-3, -3:], so["pv"][3:-3, 3:-3, -3:]).max() < TOL_STATE


@pytest.mark.parametrize("bcset", ["subsonic", "supersonic_in"])
def test_mixed_residual(oracle, bcset):
    c = make("sst", bcset)
    e = native.Engine(c, precision=abi.MIXED)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    assert field_err(e.residual(0)["res"], o.residual(0)["res"]).max() < TOL_MIXED


@pytest.mark.parametrize("base", ["plain", "sst"])
def test_shifted_periodic_matches(oracle, base):
    name, kw, over = BASES[base]
    c = cases.make(name, scale=kw["scale"] // 2, **{k: v for k, v in kw.items() if k != "scale"})
    c["cfg"].update(over)
    c = replace_faces(c, SHIFTED)
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    assert field_err(e.residual(0)["res"], o.residual(0)["res"]).max() < TOL_RES
    for it in range(2):
        e.iterate(1, it + 1, 0.0)
        o.iterate(1, it + 1, 0.0)
    sg, so = e.download(0), o.get_state(0)
    assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL_STATE
    assert field_err(sg["pv"][:3, 3:-3, 3:-3], so["pv"][:3, 3:-3, 3:-3]).max() < TOL_STATE
    assert field_err(sg["pv"][-3:, 3:-3, 3:-3], so["pv"][-3:, 3:-3, 3:-3]).max() < TOL_STATE


def test_shifted_periodic_rejects_a_source_outside_the_block():
    """24 cells along i (so the shift applies) but 8 along k: the source k + 16 of a kmin
    ghost lies beyond the padded block"""
    c = cases.make("plain_small", scale=4)
    xyz = cases.box_nodes(24, 8, 8, 2.0, 1.0, 1.0, shear=0.02, seed=0)
    c["blocks"] = [dict(imax=25, jmax=9, kmax=9, xyz=xyz, con=[],
                        bc=cases.face_patches(25, 9, 9, {"imin": abi.BC_FARFIELD, "imax": abi.BC_FARFIELD,
                                                         "jmin": abi.BC_SYMMETRY, "jmax": abi.BC_SYMMETRY,
                                                         "kmin": abi.BC_SHIFTED_PERIODIC,
                                                         "kmax": abi.BC_SHIFTED_PERIODIC}))]
    with pytest.raises(native.Cfd3dError) as ei:
        native.Engine(c)
    assert ei.value.code == abi.ERR_DESCRIPTOR
    assert "shifted periodic" in str(ei.value)


def with_heatflux(c, times, fluxes):
    """the SST case with its jmin wall a HeatFlux-family wall carrying the given history"""
    c = replace_faces(c, {"jmin": abi.BC_WALL_HEATFLUX})
    for b in c["blocks"]:
        q = next(n for n, (kind, _) in enumerate(b["bc"]) if kind == abi.BC_WALL_HEATFLUX)
        b["heatflux"] = {q: (np.asarray(times, dtype=np.float64), np.asarray(fluxes, dtype=np.float64))}
    return c


@pytest.mark.parametrize("nsteady", [0, 2])
def test_heatflux_wall_matches(oracle, nsteady):
    """bcheatfluxwallviscouskw: the history is read at bcinfo%time -- dt_phy nt_phy when
    unsteady (stepping through its segments), the accumulated pseudo time when steady"""
    name, kw, over = BASES["sst"]
    c = cases.make(name, **kw)
    c["cfg"].update(over)
    c["cfg"]["nsteady"] = nsteady
    dtp = c["cfg"]["dt_phy"]
    c = with_heatflux(c, [0.0, 1.5 * dtp, 3.0 * dtp], [50.0, 300.0, 100.0])   # a few K at the wall
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    assert field_err(e.residual(0)["res"], o.residual(0)["res"]).max() < TOL_RES
    for it, nt_phy in enumerate([1, 2, 4]):
        _, resg, _ = e.iterate(nt_phy, it + 1, 0.0)
        _, reso, _ = o.iterate(nt_phy, it + 1, 0.0)
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    sg, so = e.download(0), o.get_state(0)
    assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL_STATE
    # the wall's ghost layers (j = -1, 0, 1)
    assert field_err(sg["pv"][3:-3, :3, 3:-3], so["pv"][3:-3, :3, 3:-3]).max() < TOL_STATE


def test_heatflux_wall_needs_sst():
    c = cases.make("cavitating", scale=8)
    c = with_heatflux(replace_faces(c, {"jmin": abi.BC_WALL}), [0.0], [1.0e4])
    with pytest.raises(native.Cfd3dError) as ei:
        native.Engine(c)
    assert ei.value.code == abi.ERR_DESCRIPTOR


@pytest.mark.parametrize("base", ["plain", "cavitating", "sst"])
def test_totalpressure_inlet_matches(oracle, base):
    """bctotalpressurein: the patch's area-weighted averages, the reference's Newton solve for
    (p, T) at its fixed totals, and the ghost state from them"""
    name, kw, over = BASES[base]
    c = cases.make(name, **kw)
    c["cfg"].update(over)
    c = replace_faces(c, {"imin": abi.BC_TOTALPRESSURE_IN})
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    assert field_err(e.residual(0)["res"], o.residual(0)["res"]).max() < TOL_RES
    for it in range(3):
        _, resg, _ = e.iterate(1, it + 1, 0.0)
        _, reso, _ = o.iterate(1, it + 1, 0.0)
        assert np.all(np.isfinite(resg))
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    sg, so = e.download(0), o.get_state(0)
    assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL_STATE
    assert field_err(sg["pv"][3:-3, 3:-3, :3], so["pv"][3:-3, 3:-3, :3]).max() < TOL_STATE
    with pytest.raises(native.Cfd3dError):
        e.residual_vjp([np.zeros(abi.interior_shape(c["blocks"][0], e.npv))])


def test_totalpressure_inlet_pooled_over_blocks(oracle):
    """a total-pressure inlet on the k face of the SST case split in two along i: one pooled
    reduction and Newton solve for both blocks' patches (the reference's communicator of
    every rank carrying the inlet)"""
    name, kw, over = BASES["sst"]
    c = cases.make(name, **kw)
    c["cfg"].update(over)
    c = replace_faces(cases.split_i(c, 2), {"kmin": abi.BC_TOTALPRESSURE_IN})
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    for b in range(2):
        assert field_err(e.residual(b)["res"], o.residual(b)["res"]).max() < TOL_RES
    for it in range(3):
        _, resg, _ = e.iterate(1, it + 1, 0.0)
        _, reso, _ = o.iterate(1, it + 1, 0.0)
        assert np.all(np.isfinite(resg))
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    for b in range(2):
        sg, so = e.download(b), o.get_state(b)
        assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL_STATE
        assert field_err(sg["pv"][:3, 3:-3, 3:-3], so["pv"][:3, 3:-3, 3:-3]).max() < TOL_STATE
