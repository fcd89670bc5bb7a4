"""Checkpoints through the C ABI: cfd3d_checkpoint_write must produce the reference's
out_########.dat bytes (the oracle's restatement of variable%export_variable, fed with the
engine's own downloaded state), and cfd3d_checkpoint_read must restart the run so that the
next pseudo-iteration is the one the uninterrupted run takes."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native
from oracle import oracle_checkpoint as ock

pytestmark = pytest.mark.gpu

CASES = {
    # steady Euler: no emut, no qq, no rcav
    "plain": ("plain_small", dict(scale=8), {}),
    # steady laminar with cavitation: rcav
    "cavitating": ("cavitating", dict(scale=8), {}),
    # SST, cavitation, BDF2: emut, qq (nqq = 2), rcav
    "large": ("large", dict(scale=16), dict(fix_cav_clamp=1)),
    # six blocks: per-block displacements
    "batched": ("batched", dict(scale=4, nblocks=6), dict(fix_cav_clamp=1)),
}


def make(name):
    base, kw, over = CASES[name]
    c = cases.make(base, **kw)
    c["cfg"].update(over)
    return c


def _run(e, c, n):
    nsteady = c["cfg"].get("nsteady", 0)
    t = 0.0
    for it in range(1, n + 1):
        t, _, _ = e.iterate(1, it, 0.0)
    if nsteady:
        e.unsteady_shift()
    return t


def _states(e, c):
    return [e.download(b) for b in range(len(c["blocks"]))]


@pytest.mark.parametrize("name", list(CASES))
def test_written_file_matches_the_reference_layout(name, tmp_path):
    c = make(name)
    e = native.Engine(c)
    e.initialize(c["pv0"])
    t = _run(e, c, 2)
    path = tmp_path / "out_00000002.dat"
    e.checkpoint_write(str(path), 1, 2, t)
    got = path.read_bytes()
    st = _states(e, c)
    want = ock.write_checkpoint(tmp_path / "oracle.dat", c["cfg"], c["blocks"], e.npv, e.nqq, 1, 2, t,
                                [dict(pv=s["pv"], tv=s["tv"], qq=s["qq"][..., :e.nqq * e.npv], rcav=s["rcav"])
                                 for s in st])
    assert len(got) == len(want) == ock.displacements(c["cfg"], c["blocks"], e.npv, e.nqq)[1]
    assert got == want


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_restart_continues_the_run(name, precision, tmp_path):
    c = make(name)
    nsteady = c["cfg"].get("nsteady", 0)
    a = native.Engine(c, precision=precision)
    a.initialize(c["pv0"])
    t = _run(a, c, 3)
    path = str(tmp_path / "out.dat")
    a.checkpoint_write(path, 1, 3, t)
    b = native.Engine(c, precision=precision)
    nps, nts, tp = b.checkpoint_read(path)
    assert (nps, nts, tp) == ock.restart_counters(1, 3, t, nsteady)
    for blk in range(len(c["blocks"])):
        sa, sb = a.download(blk), b.download(blk)
        for k in ("pv", "dv", "tv", "qq", "rcav"):
            ia, ib = sa[k], sb[k]
            if k in ("pv", "dv", "tv"):
                ia, ib = ia[3:-3, 3:-3, 3:-3], ib[3:-3, 3:-3, 3:-3]
            assert np.array_equal(ia, ib), (blk, k)
    # the next pseudo-iteration of both runs
    ta, ra, _ = a.iterate(nps, nts, 0.0)
    tb, rb, _ = b.iterate(nps, nts, tp if nsteady == 0 else 0.0)
    assert np.array_equal(ra, rb)
    for blk in range(len(c["blocks"])):
        assert np.array_equal(a.download(blk)["pv"][3:-3, 3:-3, 3:-3], b.download(blk)["pv"][3:-3, 3:-3, 3:-3])


def test_steady_start_rebuilds_the_history(tmp_path):
    """The steadyini variant: a steady run's file (no qq) starts an unsteady run."""
    steady = make("large")
    steady["cfg"].update(nsteady=0)
    a = native.Engine(steady)
    a.initialize(steady["pv0"])
    t = _run(a, steady, 2)
    path = str(tmp_path / "out_00000002.dat")
    a.checkpoint_write(path, 1, 2, t)
    c = make("large")
    b = native.Engine(c)
    assert b.checkpoint_read(path, steady_start=True) == (1, 1, 0.0)
    sa, sb = a.download(0), b.download(0)
    assert np.array_equal(sa["pv"][3:-3, 3:-3, 3:-3], sb["pv"][3:-3, 3:-3, 3:-3])
    q = sb["qq"]
    npv = b.npv
    # both histories hold the conservative state of the read pv
    assert np.array_equal(q[..., :npv], q[..., npv:2 * npv])
    rho = sb["dv"][3:-3, 3:-3, 3:-3, 0]
    assert np.array_equal(q[..., 0], rho)
    assert np.array_equal(q[..., 1], rho * sb["pv"][3:-3, 3:-3, 3:-3, 1])


def test_errors_and_no_truncation(tmp_path):
    c = make("plain")
    e = native.Engine(c)
    e.initialize(c["pv0"])
    with pytest.raises(native.Cfd3dError) as ei:
        e.checkpoint_read(str(tmp_path / "missing.dat"))
    assert ei.value.code == abi.ERR_IO
    path = tmp_path / "out.dat"
    size = ock.displacements(c["cfg"], c["blocks"], e.npv, e.nqq)[1]
    # mpi_mode_create without truncation: bytes past the records stay
    path.write_bytes(b"\xab" * (size + 100))
    e.checkpoint_write(str(path), 0, 0, 0.0)
    raw = path.read_bytes()
    assert len(raw) == size + 100 and raw[size:] == b"\xab" * 100
    path.write_bytes(raw[:size - 8])
    with pytest.raises(native.Cfd3dError) as ei:
        e.checkpoint_read(str(path))
    assert ei.value.code == abi.ERR_IO
    e.iterate(1, 1, 0.0)   # the handle stays usable
