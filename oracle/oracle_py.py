"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/liboracle.so (built by `make -C oracle`) and exposes the restated
reference path on the same descriptors the product takes.  Imported only by tests/,
by __graft_entry__.smoke() (to verify the GPU path) and by bench.py's CPU-baseline arm (timed
as the CPU baseline); never by the product path.

parity unpinned: the reference (Fortran + MPI + CGNS) cannot be built here and has no
tests or golden vectors; see oracle_physics.h.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from cfd3d_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
# the same source built for speed (-O3, multiply-add contraction): times the CPU baseline
# only, never a parity check
LIB_FAST = os.path.join(HERE, "_build", "liboracle_fast.so")
_libs = {}


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib(fast=False):
    path = LIB_FAST if fast else LIB
    if path not in _libs:
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(abi.Config), C.c_int, C.POINTER(abi.BlockDesc), C.c_char_p, C.c_int]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_initialize.argtypes = [C.c_void_p, C.c_int, dp]
        L.orc_set_state.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp]
        L.orc_get_state.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp, dp]
        L.orc_get_csf.argtypes = [C.c_void_p, C.c_int, dp, dp]
        L.orc_metrics.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp]
        L.orc_residual.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp]
        L.orc_iterate.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, dp, dp, C.POINTER(C.c_int)]
        L.orc_unsteady_shift.argtypes = [C.c_void_p]
        L.orc_eos.argtypes = [C.c_int, C.c_int, C.c_int, C.c_long, dp, dp, dp, dp, dp, dp]
        L.orc_refs.argtypes = [C.c_void_p, dp]
        L.orc_pww.restype = C.c_double
        L.orc_pww.argtypes = [C.c_double]
        L.orc_tww.restype = C.c_double
        L.orc_tww.argtypes = [C.c_double]
        L.orc_snd2_fallbacks.restype = C.c_long
        _libs[path] = L
    return _libs[path]


def _p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def eos(p, t, y1, y2, fluid=2, prop=False):
    p, t, y1, y2 = (np.ascontiguousarray(a, dtype=np.float64) for a in (p, t, y1, y2))
    n = p.size
    dv = np.zeros((n, 18))
    tv = np.zeros((n, 2))
    lib().orc_eos(fluid, 1, 1 if prop else 0, n, _p(p), _p(t), _p(y1), _p(y2), _p(dv), _p(tv))
    return dv, tv


class Oracle:
    """One oracle instance over a case (see cfd3d_gb300.cases)."""

    def __init__(self, case, threads=1, fast=False):
        """fast: the speed build (CPU-baseline timing only)"""
        self.case = case
        self._L = lib(fast)
        self.cfgd = dict(case["cfg"])
        self.npv, self.ntv, self.nqq, self.ngrd = abi.sizes(self.cfgd)
        self._cfg = abi.config_from_dict(self.cfgd)
        self._bs = abi.BlockSet(case["blocks"])
        err = C.create_string_buffer(512)
        self.h = self._L.orc_create(C.byref(self._cfg), self._bs.n, self._bs.arr, err, 512)
        if not self.h:
            raise RuntimeError("oracle create failed: " + err.value.decode())
        self._L.orc_set_threads(self.h, threads)

    def __del__(self):
        if getattr(self, "h", None):
            self._L.orc_destroy(self.h)
            self.h = None

    def blocks(self):
        return self.case["blocks"]

    def initialize(self, pv0=None):
        for n in range(len(self.case["blocks"])):
            a = None if pv0 is None else np.ascontiguousarray(pv0[n], dtype=np.float64)
            self._L.orc_initialize(self.h, n, _p(a))

    def refs(self):
        out = np.zeros(6)
        self._L.orc_refs(self.h, _p(out))
        return dict(zip(["rhoref", "visref", "kref", "oref", "emutref", "str"], out))

    def get_state(self, n):
        b = self.case["blocks"][n]
        pv = np.zeros(abi.padded_shape(b, self.npv))
        dv = np.zeros(abi.padded_shape(b, 18))
        tv = np.zeros(abi.padded_shape(b, max(self.ntv, 1)))
        qq = np.zeros(abi.interior_shape(b, max(self.npv * self.nqq, 1)))
        rc = np.zeros(abi.interior_shape(b, 2))
        self._L.orc_get_state(self.h, n, _p(pv), _p(dv), _p(tv), _p(qq), _p(rc))
        return dict(pv=pv, dv=dv, tv=tv[..., :self.ntv], qq=qq, rcav=rc)

    def get_csf(self, n):
        """csf = 1: the volume-fraction gradient vfg (k, j, i, 3) over the cells 1..imax+1
        and the surface-tension source csf (interior, 3) of the last residual."""
        b = self.case["blocks"][n]
        vfg = np.zeros((b["kmax"] + 1, b["jmax"] + 1, b["imax"] + 1, 3))
        csf = np.zeros(abi.interior_shape(b, 3))
        if self._L.orc_get_csf(self.h, n, _p(vfg), _p(csf)) != 0:
            raise ValueError("the case has no surface-tension source")
        return dict(vfg=vfg, csf=csf)

    def set_state(self, n, pv=None, dv=None, tv=None, qq=None):
        b = self.case["blocks"][n]
        if tv is not None and self.ntv:
            tv = np.ascontiguousarray(tv, dtype=np.float64)
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (pv, dv, tv, qq)]
        self._L.orc_set_state(self.h, n, *[_p(a) for a in args])
        del b

    def metrics(self, n):
        b = self.case["blocks"][n]
        im, jm, km = b["imax"], b["jmax"], b["kmax"]
        cx = np.zeros((km + 1, jm + 1, im, 3))
        ex = np.zeros((km + 1, jm, im + 1, 3))
        tx = np.zeros((km, jm + 1, im + 1, 3))
        grd = np.zeros((km + 1, jm + 1, im + 1, self.ngrd))
        self._L.orc_metrics(self.h, n, _p(cx), _p(ex), _p(tx), _p(grd))
        return cx, ex, tx, grd

    def residual(self, n=0):
        b = self.case["blocks"][n]
        res = np.zeros(abi.interior_shape(b, self.npv))
        icav = np.zeros(abi.interior_shape(b, 4))
        itt = np.zeros(abi.interior_shape(b, 4))
        oc = np.zeros(abi.interior_shape(b, 1))
        self._L.orc_residual(self.h, n, _p(res), _p(icav), _p(itt), _p(oc))
        return dict(res=res, icav=icav, itt=itt, omega_cut=oc[..., 0])

    def iterate(self, nt_phy=1, nt=1, timeprev=0.0):
        t = C.c_double(0.0)
        res = np.zeros(self.npv)
        loc = (C.c_int * 4)()
        self._L.orc_iterate(self.h, nt_phy, nt, timeprev, C.byref(t), _p(res), loc)
        return t.value, res, tuple(loc)

    def unsteady_shift(self):
        self._L.orc_unsteady_shift(self.h)
