"""ctypes mirror of include/cfd3d.h (descriptor structs and constants).

The structs follow the reference's input and grid descriptors: `cfd3d_config` holds the
fields `config%construct` reads from input.inp (src/config_module.f90:100-119),
`cfd3d_bc_patch` / `cfd3d_connection` hold what `grid%construct` reads from the CGNS
file (src/grid_module.f90:151-300).
"""
import ctypes as C

import numpy as np

OK = 0
ERR_ARG, ERR_CUDA, ERR_NONFINITE, ERR_VOLUME, ERR_TIMEOUT, ERR_DESCRIPTOR, ERR_NOMEM, ERR_NODEVICE, ERR_IO = range(1, 10)

FP64, MIXED = 0, 1

BC_WALL, BC_SYMMETRY, BC_FARFIELD, BC_EXTRAPOLATE, BC_DEGENERATE, BC_INFLOW = range(1, 7)
BC_INFLOW_SUBSONIC, BC_OUTFLOW_SUBSONIC, BC_INFLOW_SUPERSONIC, BC_OUTFLOW = range(7, 11)
BC_WALL_COUNTERROTATING, BC_WALL_HEATFLUX, BC_MASSFLOWRATE_IN, BC_SHIFTED_PERIODIC = 11, 12, 13, 14
BC_TOTALPRESSURE_IN = 15
BC_NAMES = {
    "BCWall": BC_WALL,
    "BCSymmetryPlane": BC_SYMMETRY,
    "BCFarfield": BC_FARFIELD,
    "BCExtrapolate": BC_EXTRAPOLATE,
    "BCOutflowSupersonic": BC_EXTRAPOLATE,
    "BCDegeneratePoint": BC_DEGENERATE,
    "BCDegenerateLine": BC_DEGENERATE,
    "BCInflow": BC_INFLOW,
    "BCInflowSubsonic": BC_INFLOW_SUBSONIC,
    "BCOutflowSubsonic": BC_OUTFLOW_SUBSONIC,
    "BCInflowSupersonic": BC_INFLOW_SUPERSONIC,
    "BCOutflow": BC_OUTFLOW,
    "BCMassflowrateIn": BC_MASSFLOWRATE_IN,
    "BCShiftedPeriodic": BC_SHIFTED_PERIODIC,
    "BCTotalPressureIn": BC_TOTALPRESSURE_IN,
}


class Config(C.Structure):
    _fields_ = [
        ("nsteady", C.c_int), ("npmax", C.c_int), ("ntmax", C.c_int), ("bond", C.c_int),
        ("dt_phy", C.c_double),
        ("iturb", C.c_int), ("ides", C.c_int),
        ("nscheme", C.c_int), ("nmuscl", C.c_int), ("nlim", C.c_int),
        ("timemethod", C.c_int), ("local", C.c_int), ("prec", C.c_int),
        ("cfl", C.c_double),
        ("fluid", C.c_int), ("ngas", C.c_int),
        ("ncav", C.c_int), ("c_v", C.c_double), ("c_c", C.c_double),
        ("pref", C.c_double), ("uref", C.c_double), ("aoa", C.c_double), ("aos", C.c_double),
        ("tref", C.c_double), ("y1ref", C.c_double), ("y2ref", C.c_double),
        ("l_chord", C.c_double), ("l_character", C.c_double), ("scale", C.c_double),
        ("l_domain", C.c_double),
        ("fix_cav_clamp", C.c_int), ("precision", C.c_int),
        ("kinf", C.c_double), ("oinf", C.c_double),
        ("gravity", C.c_int), ("ngravity", C.c_int), ("gravity_data", C.POINTER(C.c_double)),
        ("csf", C.c_int), ("rotation", C.c_int), ("rpm", C.c_double),
    ]


class BcPatch(C.Structure):
    _fields_ = [("type", C.c_int), ("pnts", C.c_int * 6), ("ndata", C.c_int),
                ("tdata", C.POINTER(C.c_double)), ("heatflux", C.POINTER(C.c_double))]


class Connection(C.Structure):
    _fields_ = [("donor", C.c_int), ("pnts", C.c_int * 6), ("pnts_donor", C.c_int * 6),
                ("transform", C.c_int * 3)]


class BlockDesc(C.Structure):
    _fields_ = [("imax", C.c_int), ("jmax", C.c_int), ("kmax", C.c_int),
                ("xyz", C.POINTER(C.c_double)),
                ("nbc", C.c_int), ("bc", C.POINTER(BcPatch)),
                ("ncon", C.c_int), ("con", C.POINTER(Connection))]


def config_from_dict(d):
    cfg = Config()
    defaults = dict(nsteady=0, npmax=1, ntmax=1, bond=12, dt_phy=1.0, iturb=-3, ides=0, nscheme=1,
                    nmuscl=1, nlim=1, timemethod=3, local=1, prec=1, cfl=1.0, fluid=2, ngas=1, ncav=0,
                    c_v=0.0, c_c=0.0, pref=101325.0, uref=10.0, aoa=0.0, aos=0.0, tref=300.0,
                    y1ref=0.0, y2ref=1e-7, l_chord=1.0, l_character=1.0, scale=1.0, l_domain=1.0,
                    fix_cav_clamp=0, precision=FP64, kinf=0.0, oinf=0.0, gravity=0, csf=0, rotation=0,
                    rpm=0.0)
    defaults.update(d)
    table = defaults.pop("gravity_data", None)
    for k, v in defaults.items():
        if k in ("ngravity",):
            continue
        setattr(cfg, k, v)
    if table is not None:
        # the gravity history (t, gx, gy, gz) rows; kept alive with the struct
        arr = np.ascontiguousarray(table, dtype=np.float64).reshape(-1, 4)
        cfg._gravity_keep = arr
        cfg.ngravity = arr.shape[0]
        cfg.gravity_data = arr.ctypes.data_as(C.POINTER(C.c_double))
    return cfg


class BlockSet:
    """Keeps the numpy buffers of a list of block descriptors alive for the C call."""

    def __init__(self, blocks):
        self._keep = []
        arr = (BlockDesc * len(blocks))()
        for n, b in enumerate(blocks):
            xyz = np.ascontiguousarray(b["xyz"], dtype=np.float64)
            assert xyz.shape == (b["kmax"], b["jmax"], b["imax"], 3)
            bcs = (BcPatch * max(1, len(b["bc"])))()
            # heat-flux histories: {patch index: (times, fluxes)}
            tables = b.get("heatflux", {})
            for q, (t, p) in enumerate(b["bc"]):
                bcs[q].type = t
                for r in range(6):
                    bcs[q].pnts[r] = p[r]
                if q in tables:
                    td = np.ascontiguousarray(tables[q][0], dtype=np.float64)
                    hf = np.ascontiguousarray(tables[q][1], dtype=np.float64)
                    assert td.shape == hf.shape and td.ndim == 1
                    self._keep += [td, hf]
                    bcs[q].ndata = td.size
                    bcs[q].tdata = td.ctypes.data_as(C.POINTER(C.c_double))
                    bcs[q].heatflux = hf.ctypes.data_as(C.POINTER(C.c_double))
            cons = (Connection * max(1, len(b.get("con", []))))()
            for q, cc in enumerate(b.get("con", [])):
                cons[q].donor = cc["donor"]
                for r in range(6):
                    cons[q].pnts[r] = cc["pnts"][r]
                    cons[q].pnts_donor[r] = cc["pnts_donor"][r]
                for r in range(3):
                    cons[q].transform[r] = cc["transform"][r]
            arr[n].imax, arr[n].jmax, arr[n].kmax = b["imax"], b["jmax"], b["kmax"]
            arr[n].xyz = xyz.ctypes.data_as(C.POINTER(C.c_double))
            arr[n].nbc = len(b["bc"])
            arr[n].bc = bcs
            arr[n].ncon = len(b.get("con", []))
            arr[n].con = cons
            self._keep += [xyz, bcs, cons]
        self.arr = arr
        self.n = len(blocks)


def sizes(cfg_dict):
    """(npv, ntv, nqq, ngrd) for a config (config%construct, src/config_module.f90:144-161)."""
    it = cfg_dict.get("iturb", -3)
    npv = 9 if it in (-1, 0) else 7
    ntv = {-3: 0, -2: 2}.get(it, 3)
    nqq = 2 if cfg_dict.get("nsteady", 0) >= 1 else 0
    ngrd = 5 if it in (-1, 0) else 4
    return npv, ntv, nqq, ngrd


def padded_shape(b, nvar):
    """Shape (k, j, i, var) of a padded cell array pv(nvar, -1:imax+3, ...)."""
    return (b["kmax"] + 5, b["jmax"] + 5, b["imax"] + 5, nvar)


def interior_shape(b, nvar):
    return (b["kmax"] - 1, b["jmax"] - 1, b["imax"] - 1, nvar)
