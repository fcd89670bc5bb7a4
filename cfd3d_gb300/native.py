"""ctypes binding of the engine's C ABI (include/cfd3d.h) and the host driver.

`Engine` wraps one `cfd3d_handle`; `Solver` mirrors the reference's
`t_solve%solve_equation` (src/solve_module.f90:119-153): physical-time loop, pseudo-time
loop of `update%timeinteg` + `resi%residual`, convergence test on res(1)/res(2) against
10^-bond, BDF history shift after each physical step, and the `res.plt` Tecplot log
(src/residual_module.f90:47-69,168-174).

There is no CPU fallback: if the CUDA library is missing or no GPU is visible, every
entry point raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from . import build as _build

_lib = None


class Cfd3dError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cfd3d error {code}: {msg}")
        self.code = code


def lib():
    """Load libcfd3d_gb300.so (building it in-tree if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        _build.build()
    L = C.CDLL(path)
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    H = C.c_void_p
    L.cfd3d_create.argtypes = [C.POINTER(abi.Config), C.c_int, C.POINTER(abi.BlockDesc), C.POINTER(H)]
    L.cfd3d_destroy.argtypes = [H]
    L.cfd3d_last_error.restype = C.c_char_p
    L.cfd3d_last_error.argtypes = [H]
    L.cfd3d_sizes.argtypes = [H, ip, ip, ip, ip, ip]
    L.cfd3d_initialize.argtypes = [H, C.c_int, dp]
    L.cfd3d_upload_state.argtypes = [H, C.c_int, dp, dp, dp, dp]
    L.cfd3d_download_state.argtypes = [H, C.c_int, dp, dp, dp, dp, dp]
    L.cfd3d_download_csf.argtypes = [H, C.c_int, dp]
    L.cfd3d_upload_primitives.argtypes = [H, C.c_int, dp, dp]
    pp = C.POINTER(dp)
    L.cfd3d_upload_primitives_all.argtypes = [H, pp, pp]
    L.cfd3d_download_state_all.argtypes = [H, pp, pp, pp]
    L.cfd3d_checkpoint_write.argtypes = [H, C.c_char_p, C.c_int, C.c_int, C.c_double]
    L.cfd3d_checkpoint_read.argtypes = [H, C.c_char_p, C.c_int, ip, ip, dp]
    L.cfd3d_iterate.argtypes = [H, C.c_int, C.c_int, C.c_double, dp, dp, ip]
    L.cfd3d_iterate_n.argtypes = [H, C.c_int, C.c_int, C.c_int, C.c_double, dp, dp]
    L.cfd3d_unsteady_shift.argtypes = [H]
    L.cfd3d_residual.argtypes = [H, C.c_int, dp, dp, dp, dp]
    L.cfd3d_grid_metrics.argtypes = [H, C.c_int, dp, dp, dp, dp]
    L.cfd3d_residual_vjp.argtypes = [H, dp, dp, dp]
    L.cfd3d_sweep_stall_test.argtypes = [H]
    L.cfd3d_autotune.argtypes = [H, C.c_int, ip]
    L.cfd3d_eos_eval.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, dp, dp, dp, dp, dp, dp]
    L.cfd3d_eos_eval_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, dp, dp, dp, dp, dp, dp]
    L.cfd3d_stats.argtypes = [H, C.POINTER(C.c_int64), ip]
    L.cfd3d_launch_shapes.argtypes = [H, ip]
    L.cfd3d_set_launch_shapes.argtypes = [H, ip]
    L.cfd3d_convert_selftest.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
    L.cfd3d_convert_rate.argtypes = [dp]
    L.cfd3d_time_iterate.argtypes = [H, C.c_int, dp]
    L.cfd3d_profile_iterate.argtypes = [H, dp]
    L.cfd3d_set_device.argtypes = [C.c_int]
    L.cfd3d_fp64_peak.argtypes = [C.c_double, dp]
    _lib = L
    return L


EXPORTS = ["cfd3d_create", "cfd3d_destroy", "cfd3d_last_error", "cfd3d_sizes", "cfd3d_initialize",
           "cfd3d_upload_state", "cfd3d_download_state", "cfd3d_upload_primitives", "cfd3d_upload_primitives_all", "cfd3d_download_state_all", "cfd3d_download_csf", "cfd3d_checkpoint_write", "cfd3d_checkpoint_read",
           "cfd3d_iterate", "cfd3d_iterate_n",
           "cfd3d_unsteady_shift", "cfd3d_residual", "cfd3d_residual_vjp", "cfd3d_sweep_stall_test", "cfd3d_autotune", "cfd3d_grid_metrics", "cfd3d_eos_eval", "cfd3d_eos_eval_noalloc", "cfd3d_stats", "cfd3d_launch_shapes", "cfd3d_set_launch_shapes", "cfd3d_convert_selftest", "cfd3d_convert_rate",
           "cfd3d_time_iterate", "cfd3d_profile_iterate", "cfd3d_set_device", "cfd3d_fp64_peak"]
STAGES = ["timestep", "boundary", "face_flux", "residual", "sweep_fwd", "sweep_bwd", "update_eos", "eddy_norms"]


def set_device(dev):
    """Select the CUDA device for the engines created afterwards on this thread."""
    rc = lib().cfd3d_set_device(int(dev))
    if rc:
        raise Cfd3dError(rc, "cfd3d_set_device failed")


def _p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def fp64_peak(seconds=1.0):
    """cfd3d_fp64_peak: the current device's FP64 FMA throughput in TFLOP/s"""
    out = C.c_double(0.0)
    rc = lib().cfd3d_fp64_peak(float(seconds), C.byref(out))
    if rc:
        raise Cfd3dError(rc, "cfd3d_fp64_peak failed")
    return out.value


def convert_selftest(n, seed=1):
    """cfd3d_convert_selftest: (double -> float, float -> double) mismatch counts of the
    integer-pipe conversions against the hardware's over n seeded bit patterns."""
    out = (C.c_longlong * 2)()
    rc = lib().cfd3d_convert_selftest(int(n), int(seed), out)
    if rc:
        raise Cfd3dError(rc, "cfd3d_convert_selftest failed")
    return out[0], out[1]


def convert_rate():
    """cfd3d_convert_rate: G conversions/s of double -> float (hardware, integer pipes) and
    float -> double (hardware, integer pipes) on the current device."""
    out = (C.c_double * 4)()
    rc = lib().cfd3d_convert_rate(out)
    if rc:
        raise Cfd3dError(rc, "cfd3d_convert_rate failed")
    return {"d2f_hw": out[0], "d2f_int": out[1], "f2d_hw": out[2], "f2d_int": out[3]}


def eos_eval(p, t, y1, y2, fluid=2, prop=False):
    """Pointwise mixture EOS on the device: dv (n, 18) and tv (n, 2)."""
    p, t, y1, y2 = (np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (p, t, y1, y2))
    n = p.size
    dv = np.zeros((n, 18))
    tv = np.zeros((n, 2))
    rc = lib().cfd3d_eos_eval(fluid, 1, 1 if prop else 0, n, _p(p), _p(t), _p(y1), _p(y2), _p(dv), _p(tv))
    if rc:
        raise Cfd3dError(rc, "cfd3d_eos_eval failed")
    return dv, tv


EOS_NOALLOC_MAX = 4096   # CFD3D_EOS_NOALLOC_MAX


def eos_eval_noalloc(p, t, y1, y2, fluid=2, prop=False):
    """eos_eval through the library's static device buffer (no device allocation);
    at most EOS_NOALLOC_MAX points per call, calls on one device must not overlap."""
    p, t, y1, y2 = (np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (p, t, y1, y2))
    n = p.size
    dv = np.zeros((n, 18))
    tv = np.zeros((n, 2))
    rc = lib().cfd3d_eos_eval_noalloc(fluid, 1, 1 if prop else 0, n, _p(p), _p(t), _p(y1), _p(y2), _p(dv), _p(tv))
    if rc:
        raise Cfd3dError(rc, "cfd3d_eos_eval_noalloc failed (n = %d, limit %d)" % (n, EOS_NOALLOC_MAX))
    return dv, tv


class Engine:
    """One engine handle over a case (cfd3d_gb300.cases format)."""

    def __init__(self, case, precision=abi.FP64):
        self.case = case
        cfgd = dict(case["cfg"])
        cfgd["precision"] = precision
        self.cfgd = cfgd
        self._cfg = abi.config_from_dict(cfgd)
        self._bs = abi.BlockSet(case["blocks"])
        h = C.c_void_p()
        rc = lib().cfd3d_create(C.byref(self._cfg), self._bs.n, self._bs.arr, C.byref(h))
        self.h = h
        if rc:
            msg = lib().cfd3d_last_error(h).decode() if h else "create failed"
            lib().cfd3d_destroy(h)
            self.h = None
            raise Cfd3dError(rc, msg)
        npv, ndv, ntv, nqq, ngrd = (C.c_int() for _ in range(5))
        lib().cfd3d_sizes(self.h, C.byref(npv), C.byref(ndv), C.byref(ntv), C.byref(nqq), C.byref(ngrd))
        self.npv, self.ntv, self.nqq, self.ngrd = npv.value, ntv.value, nqq.value, ngrd.value

    def close(self):
        if getattr(self, "h", None):
            lib().cfd3d_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, rc):
        if rc:
            raise Cfd3dError(rc, lib().cfd3d_last_error(self.h).decode())

    def initialize(self, pv0=None):
        for n in range(len(self.case["blocks"])):
            a = None if pv0 is None else np.ascontiguousarray(pv0[n], dtype=np.float64)
            self._check(lib().cfd3d_initialize(self.h, n, _p(a)))

    def upload(self, n, pv=None, dv=None, tv=None, qq=None):
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (pv, dv, tv, qq)]
        self._check(lib().cfd3d_upload_state(self.h, n, *[_p(a) for a in args]))

    def upload_primitives(self, n, pv, qq=None):
        """cfd3d_upload_primitives: padded pv (and the history qq); dv and tv follow on the
        device from the EOS and the eddy viscosity."""
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (pv, qq)]
        self._check(lib().cfd3d_upload_primitives(self.h, n, *[_p(a) for a in args]))

    def _ptrs(self, arrays, writable=False):
        """an array of per-block pointers (NULL for None entries, or None for no list)"""
        if arrays is None:
            return None
        arr = (C.POINTER(C.c_double) * len(arrays))()
        for q, a in enumerate(arrays):
            if a is not None:
                assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] and (a.flags["WRITEABLE"] or not writable)
                arr[q] = _p(a)
        return arr

    def upload_primitives_all(self, pv, qq=None):
        """cfd3d_upload_primitives_all: per-block padded pv (and qq) lists, contiguous float64"""
        self._check(lib().cfd3d_upload_primitives_all(self.h, self._ptrs(pv), self._ptrs(qq)))

    def download_state_all(self, pv=None, dv=None, tv=None):
        """cfd3d_download_state_all into caller-owned per-block arrays (None skips)"""
        self._check(lib().cfd3d_download_state_all(self.h, self._ptrs(pv, True), self._ptrs(dv, True),
                                                   self._ptrs(tv, True) if self.ntv else None))

    def download_csf(self, n):
        """The surface-tension source csf(3, interior) of block n from the last residual."""
        out = np.zeros(abi.interior_shape(self.case["blocks"][n], 3))
        self._check(lib().cfd3d_download_csf(self.h, n, _p(out)))
        return out

    def download(self, n, out=None):
        b = self.case["blocks"][n]
        if out is None:
            out = dict(pv=np.zeros(abi.padded_shape(b, self.npv)), dv=np.zeros(abi.padded_shape(b, 18)),
                       tv=np.zeros(abi.padded_shape(b, max(self.ntv, 1))),
                       qq=np.zeros(abi.interior_shape(b, max(2 * self.npv * (1 if self.nqq else 0), 1))),
                       rcav=np.zeros(abi.interior_shape(b, 2)))
        self._check(lib().cfd3d_download_state(self.h, n, _p(out["pv"]), _p(out["dv"]),
                                               _p(out["tv"]) if self.ntv else None,
                                               _p(out["qq"]) if self.nqq else None, _p(out["rcav"])))
        if self.ntv:
            out["tv"] = out["tv"][..., :self.ntv]
        return out

    def download_arrays(self, n, pv=None, dv=None, tv=None, qq=None, rcav=None):
        """Download into caller-owned contiguous float64 arrays (None skips a field)."""
        for a in (pv, dv, tv, qq, rcav):
            assert a is None or (a.dtype == np.float64 and a.flags["C_CONTIGUOUS"])
        self._check(lib().cfd3d_download_state(self.h, n, _p(pv), _p(dv), _p(tv) if self.ntv else None,
                                               _p(qq) if self.nqq else None, _p(rcav)))

    def checkpoint_write(self, path, nt_phy, nt, time):
        """variable%export_variable: write the state to `path` in the reference's layout."""
        self._check(lib().cfd3d_checkpoint_write(self.h, os.fsencode(path), nt_phy, nt, float(time)))

    def checkpoint_read(self, path, steady_start=False):
        """t_ini_restart%restart: load the state from `path`; returns (nps, nts, timeprev)."""
        nps, nts, tp = C.c_int(), C.c_int(), C.c_double()
        self._check(lib().cfd3d_checkpoint_read(self.h, os.fsencode(path), 1 if steady_start else 0,
                                                C.byref(nps), C.byref(nts), C.byref(tp)))
        return nps.value, nts.value, tp.value

    def residual(self, n=0):
        b = self.case["blocks"][n]
        res = np.zeros(abi.interior_shape(b, self.npv))
        icav = np.zeros(abi.interior_shape(b, 4))
        itt = np.zeros(abi.interior_shape(b, 4))
        oc = np.zeros(abi.interior_shape(b, 1))
        self._check(lib().cfd3d_residual(self.h, n, _p(res), _p(icav), _p(itt), _p(oc)))
        return dict(res=res, icav=icav, itt=itt, omega_cut=oc[..., 0])

    def residual_vjp(self, cot):
        """Discrete adjoint of the FP64 residual on the current state.

        cot: one residual-shaped array per block (interior_shape(block, npv)).  Returns
        (g, g_params): g = (dR/dpv)^T cot per block, same shapes, and g_params =
        cot . dR/d(uref, c_v, c_c)."""
        blocks = self.case["blocks"]
        shapes = [abi.interior_shape(b, self.npv) for b in blocks]
        flat = np.concatenate([np.ascontiguousarray(c, dtype=np.float64).reshape(-1) for c in cot])
        assert flat.size == sum(int(np.prod(s)) for s in shapes)
        out = np.zeros_like(flat)
        gpar = np.zeros(3)
        self._check(lib().cfd3d_residual_vjp(self.h, _p(flat), _p(out), _p(gpar)))
        g, off = [], 0
        for s in shapes:
            m = int(np.prod(s))
            g.append(out[off:off + m].reshape(s))
            off += m
        return g, gpar

    def autotune(self, reps=3):
        """cfd3d_autotune: returns (face threads per CTA, residual threads per CTA, sweep
        CTAs per SM) chosen by timing on the current state."""
        ch = (C.c_int * 3)()
        self._check(lib().cfd3d_autotune(self.h, reps, ch))
        return tuple(ch)

    def launch_shapes(self):
        """cfd3d_launch_shapes: (face threads per CTA, residual threads per CTA, sweep CTAs
        per SM, face / residual pipeline groups) in use."""
        sh = (C.c_int * 4)()
        self._check(lib().cfd3d_launch_shapes(self.h, sh))
        return tuple(sh)

    def set_launch_shapes(self, shapes):
        """cfd3d_set_launch_shapes: the four shapes of launch_shapes()."""
        sh = (C.c_int * 4)(*[int(x) for x in shapes])
        self._check(lib().cfd3d_set_launch_shapes(self.h, sh))

    def sweep_stall_test(self):
        """cfd3d_sweep_stall_test: the status code (CFD3D_ERR_TIMEOUT expected)."""
        return lib().cfd3d_sweep_stall_test(self.h)

    def metrics(self, n):
        b = self.case["blocks"][n]
        im, jm, km = b["imax"], b["jmax"], b["kmax"]
        cx = np.zeros((km + 1, jm + 1, im, 3))
        ex = np.zeros((km + 1, jm, im + 1, 3))
        tx = np.zeros((km, jm + 1, im + 1, 3))
        grd = np.zeros((km + 1, jm + 1, im + 1, self.ngrd))
        self._check(lib().cfd3d_grid_metrics(self.h, n, _p(cx), _p(ex), _p(tx), _p(grd)))
        return cx, ex, tx, grd

    def iterate(self, nt_phy=1, nt=1, timeprev=0.0):
        t = C.c_double(0.0)
        res = np.zeros(self.npv)
        loc = (C.c_int * 4)()
        self._check(lib().cfd3d_iterate(self.h, nt_phy, nt, timeprev, C.byref(t), _p(res), loc))
        return t.value, res, tuple(loc)

    def iterate_n(self, niter, nt_phy=1, nt0=1, timeprev=0.0):
        t = C.c_double(0.0)
        res = np.zeros(self.npv)
        self._check(lib().cfd3d_iterate_n(self.h, niter, nt_phy, nt0, timeprev, C.byref(t), _p(res)))
        return t.value, res

    def unsteady_shift(self):
        self._check(lib().cfd3d_unsteady_shift(self.h))

    def time_iterate(self, niter):
        ms = C.c_double(0.0)
        self._check(lib().cfd3d_time_iterate(self.h, niter, C.byref(ms)))
        return ms.value

    def profile_iterate(self):
        out = np.zeros(len(STAGES))
        self._check(lib().cfd3d_profile_iterate(self.h, _p(out)))
        return dict(zip(STAGES, out))

    def stats(self):
        fb = C.c_int64()
        nl = C.c_int()
        self._check(lib().cfd3d_stats(self.h, C.byref(fb), C.byref(nl)))
        return dict(snd2_fallbacks=fb.value, launches_per_iter=nl.value)


class Solver:
    """The reference's solve loop (src/solve_module.f90:119-153) over an Engine."""

    def __init__(self, case, precision=abi.FP64, log_path=None):
        self.engine = Engine(case, precision)
        self.cfg = case["cfg"]
        self.case = case
        self.log_path = log_path
        self.history = []

    def solve(self, npmax=None, ntmax=None, pv0=None, export_dir=None, restart=None, steady_start=False):
        """Run the physical / pseudo-time loops.

        export_dir: write checkpoints out_########.dat there where solve_equation calls
        variable%export_variable (src/solve_module.f90:127-150): the initial state as
        out_00000000.dat, then for a steady run every nexport pseudo-iterations and at
        convergence, for an unsteady run every nexport physical steps (after the history
        shift, with nt - 1 as its nt).  The tag is nt_phy for unsteady runs, else nt.
        restart: a checkpoint to start from (iread >= 1) instead of the initial state; the
        loops resume from the counters it yields.  steady_start reads it as the steadyini
        variant (no qq section)."""
        e = self.engine
        nsteady = self.cfg.get("nsteady", 0)
        if restart is not None:
            nps, nts, timeprev = e.checkpoint_read(restart, steady_start)
        else:
            e.initialize(self.case.get("pv0") if pv0 is None else pv0)
            nps, nts, timeprev = 1, 1, 0.0
        npmax = npmax or self.cfg.get("npmax", 1)
        ntmax = ntmax or self.cfg.get("ntmax", 1)
        nexport = max(int(self.cfg.get("nexport", 0) or 0), 0)
        bond = 10.0 ** (-self.cfg.get("bond", 12))

        def export(nt_phy, nt, time):
            if export_dir is None:
                return
            tag = nt_phy if nsteady >= 1 else nt
            e.checkpoint_write(os.path.join(export_dir, "out_%08d.dat" % tag), nt_phy, nt, time)

        if restart is None:
            export(0, 0, 0.0)
        log = open(self.log_path, "a" if restart is not None else "w") if self.log_path else None
        if log:
            names = ["nt", "resp", "resu", "resv", "resw", "rest", "resy1", "resy2"] + (["resk", "reso"] if e.npv == 9 else [])
            zone = "restart" if restart is not None else "newstart"
            log.write(" variables=" + ",".join('"%s"' % x for x in names) + "\n zone t =\"%s\"\n" % zone)
        time = timeprev
        for nt_phy in range(nps, npmax + 1):
            nt = nts
            for nt in range(nts, ntmax + 1):
                time, res, loc = e.iterate(nt_phy, nt, timeprev)
                it = ntmax * (nt_phy - 1) + nt
                self.history.append((it, time, res.copy(), loc))
                if log:
                    log.write("%10d" % it + "".join("%30.12f" % r for r in res) + "\n")
                if res[0] < bond or res[1] < bond:
                    if nsteady == 0:
                        export(nt_phy, nt, time)
                    break
                if nexport and nt % nexport == 0 and nsteady == 0:
                    export(nt_phy, nt, time)
            else:
                nt = ntmax + 1   # a completed Fortran do loop leaves its index one past the end
            if nsteady >= 1:
                e.unsteady_shift()
                if nexport and nt_phy % nexport == 0:
                    export(nt_phy, nt - 1, time)
        if log:
            log.close()
        return self.history
