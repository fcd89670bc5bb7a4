"""CPU restatement of the reference's checkpoint file (TEST INFRASTRUCTURE ONLY).

The file out_########.dat written by `variable%export_variable`
(src/variable_module.f90:116-182) and read by `t_ini_restart%restart`
(src/initial_module.f90:245-389; the steadyini variant :103-242).  Imported only by
tests/, to verify the engine's cfd3d_checkpoint_write / cfd3d_checkpoint_read.

Each MPI rank r owns block r and writes its record at a displacement equal to the sizes
of the records of ranks 0..r-1 (src/variable_module.f90:80-91, with intsize = 4 and
realsize = 8 from mpi_type_size).  A record is, in native byte order:

    nt_phy (int32), nt (int32), time (float64)                   :127-137
    pv(npv, -1:imax+3, -1:jmax+3, -1:kmax+3)                      :139-142
    emut(-1:imax+3, ..) = tv(3, ..)          if iturb >= -1        :144-158
    qq(npv, nqq, 2:imax, 2:jmax, 2:kmax)                          :160-163
    rcav(2, 2:imax, ..)                      if ncav != 0          :165-170
    csf(3, 2:imax, ..)                       if csf != 0           :172-177

Arrays here use the engine's host shapes: a padded array is (kmax+5, jmax+5, imax+5, nv)
in C order, an interior one (kmax-1, jmax-1, imax-1, nv): the same bytes as the Fortran
arrays above.  parity unpinned: the reference cannot run here (no Fortran, MPI or CGNS),
so the layout is pinned by the record formula of the reference's own displacement code,
which the tests check independently.
"""
import numpy as np

INTSIZE, REALSIZE = 4, 8


def flags(cfg):
    """l_turb, l_cav of t_variable%construct (src/variable_module.f90:65-66)."""
    return cfg.get("iturb", -3) >= -1, cfg.get("ncav", 0) != 0


def csf_flag(cfg):
    """l_csf of t_variable%construct (src/variable_module.f90:67)."""
    return cfg.get("csf", 0) != 0


def record_size(npv, nqq, imax, jmax, kmax, turb, cav, with_qq=True, csf=False):
    """Bytes of one block's record: the summand of the displacement loop
    (src/variable_module.f90:84-89; without the qq term for steadyini, initial_module :130-136)."""
    npad = (imax + 5) * (jmax + 5) * (kmax + 5)
    nint = (imax - 1) * (jmax - 1) * (kmax - 1)
    s = INTSIZE * 2 + REALSIZE + REALSIZE * npv * npad
    if with_qq:
        s += REALSIZE * nqq * npv * nint
    if turb:
        s += REALSIZE * npad
    if cav:
        s += REALSIZE * 2 * nint
    if csf:
        s += REALSIZE * 3 * nint
    return s


def displacements(cfg, blocks, npv, nqq, with_qq=True):
    """Displacement of each block's record (rank r = block r)."""
    turb, cav = flags(cfg)
    out, d = [], 0
    for b in blocks:
        out.append(d)
        d += record_size(npv, nqq, b["imax"], b["jmax"], b["kmax"], turb, cav, with_qq, csf_flag(cfg))
    return out, d


def encode_record(cfg, b, npv, nqq, nt_phy, nt, time, pv, tv=None, qq=None, rcav=None, with_qq=True, csf=None):
    """The bytes of one record, in export_variable's order."""
    turb, cav = flags(cfg)
    pad = (b["kmax"] + 5, b["jmax"] + 5, b["imax"] + 5)
    inner = (b["kmax"] - 1, b["jmax"] - 1, b["imax"] - 1)
    parts = [np.array([nt_phy, nt], dtype="<i4").tobytes(), np.array([time], dtype="<f8").tobytes()]
    pv = np.asarray(pv, dtype="<f8")
    assert pv.shape == pad + (npv,)
    parts.append(pv.tobytes())
    if turb:
        tv = np.asarray(tv, dtype="<f8")
        assert tv.shape[:3] == pad and tv.shape[3] >= 3
        parts.append(np.ascontiguousarray(tv[..., 2]).tobytes())
    if with_qq and nqq:
        qq = np.asarray(qq, dtype="<f8")
        assert qq.shape == inner + (nqq * npv,)
        parts.append(qq.tobytes())
    if cav:
        rcav = np.asarray(rcav, dtype="<f8")
        assert rcav.shape == inner + (2,)
        parts.append(rcav.tobytes())
    if csf_flag(cfg):
        csf = np.asarray(csf, dtype="<f8")
        assert csf.shape == inner + (3,)
        parts.append(csf.tobytes())
    return b"".join(parts)


def write_checkpoint(path, cfg, blocks, npv, nqq, nt_phy, nt, time, states):
    """export_variable for every rank: `states[r]` holds pv, tv, qq, rcav (and csf) of block r."""
    data = b"".join(encode_record(cfg, b, npv, nqq, nt_phy, nt, time, s["pv"], s.get("tv"), s.get("qq"),
                                  s.get("rcav"), csf=s.get("csf")) for b, s in zip(blocks, states))
    with open(path, "wb") as f:
        f.write(data)
    return data


def read_checkpoint(path, cfg, blocks, npv, nqq, with_qq=True):
    """restart's reads: per block the header and the arrays (None where absent)."""
    turb, cav = flags(cfg)
    raw = open(path, "rb").read()
    disp, total = displacements(cfg, blocks, npv, nqq, with_qq)
    if len(raw) < total:
        raise ValueError("checkpoint shorter than the case's records")
    out = []
    for b, d in zip(blocks, disp):
        pad = (b["kmax"] + 5, b["jmax"] + 5, b["imax"] + 5)
        inner = (b["kmax"] - 1, b["jmax"] - 1, b["imax"] - 1)

        def take(count, dtype):
            nonlocal d
            a = np.frombuffer(raw, dtype=dtype, count=count, offset=d)
            d += count * np.dtype(dtype).itemsize
            return a

        nt_phy, nt = (int(x) for x in take(2, "<i4"))
        time = float(take(1, "<f8")[0])
        rec = dict(nt_phy=nt_phy, nt=nt, time=time)
        rec["pv"] = take(int(np.prod(pad)) * npv, "<f8").reshape(pad + (npv,))
        rec["emut"] = take(int(np.prod(pad)), "<f8").reshape(pad) if turb else None
        rec["qq"] = take(int(np.prod(inner)) * nqq * npv, "<f8").reshape(inner + (nqq * npv,)) if (with_qq and nqq) else None
        rec["rcav"] = take(int(np.prod(inner)) * 2, "<f8").reshape(inner + (2,)) if cav else None
        rec["csf"] = take(int(np.prod(inner)) * 3, "<f8").reshape(inner + (3,)) if csf_flag(cfg) else None
        out.append(rec)
    return out


def restart_counters(nt_phy, nt, time, nsteady, steady_start=False):
    """nps, nts, timeprev after restart (src/initial_module.f90:238-240 steadyini, :373-381)."""
    if steady_start:
        return 1, 1, 0.0
    nts, nps = nt + 1, nt_phy + 1
    if nsteady >= 1:
        nts = 1
    else:
        nps = 1
    return nps, nts, time
