"""The rotating frame (rotation, rpm; src/rotation_module.f90:75-97, the rothalpy of
src/flux_module.f90:697-721, src/lhs_module.f90:573-584, src/jacobian_module.f90:486-495,
and the grid velocity of the counter-rotating walls, the mass-flow and the total-pressure
inlets, src/bc_module.f90:3299-4012) through the C ABI against the CPU oracle, FP64 form.
The cases turn at 30 rpm about +z or -x, so omega x r is a few m/s across the grid: the
Coriolis and centrifugal source, the rothalpy in the fluxes and the implicit operator, and
the ghost velocities all carry it."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native
from tests.helpers import dv_eos_err, field_err, interior
from tests.test_gpu_bc import BASES, replace_faces

pytestmark = pytest.mark.gpu

TOL_RES = 1e-9
TOL_STATE = 1e-9


def make(base, rotation, bcs, timemethod=3):
    name, kw, over = BASES[base]
    c = cases.make(name, **kw)
    c["cfg"].update(over)
    c["cfg"].update(rotation=rotation, rpm=30.0, timemethod=timemethod)
    if timemethod != 3:
        c["cfg"]["cfl"] = 0.5
    return replace_faces(c, bcs)


def _parity(oracle, c, nit=3):
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    for b in range(len(c["blocks"])):
        assert field_err(e.residual(b)["res"], o.residual(b)["res"]).max() < TOL_RES
    for it in range(nit):
        _, resg, _ = e.iterate(1, it + 1, 0.0)
        _, reso, _ = o.iterate(1, it + 1, 0.0)
        assert np.all(np.isfinite(resg))
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    for b in range(len(c["blocks"])):
        sg, so = e.download(b), o.get_state(b)
        assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL_STATE
        err, tol = dv_eos_err(interior(sg["pv"]), interior(sg["dv"]), c["cfg"])
        assert err < tol
        # the ghost layers of the rotating-frame boundaries (i faces: inlet; j faces: wall)
        assert field_err(sg["pv"][3:-3, 3:-3, :3], so["pv"][3:-3, 3:-3, :3]).max() < TOL_STATE
        assert field_err(sg["pv"][3:-3, :3, 3:-3], so["pv"][3:-3, :3, 3:-3]).max() < TOL_STATE
    return e, o


WALL_INLET = {"imin": abi.BC_MASSFLOWRATE_IN, "jmin": abi.BC_WALL_COUNTERROTATING}


@pytest.mark.parametrize("rotation", [3, -1])
@pytest.mark.parametrize("base", list(BASES))
def test_rotating_frame_matches(oracle, base, rotation):
    """Euler (the inviscid counter-rotating wall), laminar (the viscous one) and SST (its
    k-omega variant) with a mass-flow inlet, LU-SGS"""
    _parity(oracle, make(base, rotation, WALL_INLET))


def test_rotating_frame_totalpressure_inlet(oracle):
    """the total-pressure inlet's averages take u + omega x r and its ghost -omega x r"""
    _parity(oracle, make("sst", 3, {"imin": abi.BC_TOTALPRESSURE_IN, "jmin": abi.BC_WALL_COUNTERROTATING}))


@pytest.mark.parametrize("base", ["plain", "sst"])
@pytest.mark.parametrize("timemethod", [1, 2])
def test_rotating_frame_explicit(oracle, timemethod, base):
    """the explicit schemes' diagonal solve takes the rothalpy too.  (On the cavitating
    start with the reflecting mass-flow inlet, RK3 reaches NaN at its third iteration in
    the oracle as on the GPU, so the explicit cases are the Euler and SST ones.)"""
    _parity(oracle, make(base, 3, WALL_INLET, timemethod=timemethod))


def test_rotation_changes_the_residual_and_is_refused_where_not_built():
    c0 = make("sst", 0, WALL_INLET)
    c1 = make("sst", 3, WALL_INLET)
    e0, e1 = native.Engine(c0), native.Engine(c1)
    e0.initialize(c0["pv0"])
    e1.initialize(c1["pv0"])
    r0, r1 = e0.residual(0)["res"], e1.residual(0)["res"]
    assert field_err(r1, r0).max() > 1e-3
    with pytest.raises(native.Cfd3dError) as ei:
        native.Engine(c1, precision=abi.MIXED)
    assert ei.value.code == abi.ERR_ARG
    with pytest.raises(native.Cfd3dError) as ei:
        e1.residual_vjp([np.zeros(abi.interior_shape(b, e1.npv)) for b in c1["blocks"]])
    assert ei.value.code == abi.ERR_ARG
