"""Error paths of the C ABI on a GPU, made on the host: a non-finite uploaded state,
out-of-range arguments, a grid with a collapsed cell.  Nothing here faults the device; the
handle stays usable."""
import numpy as np
import pytest

from cfd3d_gb300 import abi, cases, native
from cfd3d_gb300.native import Cfd3dError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_nonfinite_state_is_reported_and_the_handle_recovers(precision):
    c = cases.make("plain_small", scale=8)
    e = native.Engine(c, precision=precision)
    e.initialize(c["pv0"])
    clean = e.download(0)
    bad = {k: v.copy() for k, v in clean.items()}
    bad["pv"][5, 5, 5, 0] = np.nan
    e.upload(0, pv=bad["pv"])
    with pytest.raises(Cfd3dError) as ei:
        e.iterate(1, 1, 0.0)
    assert ei.value.code == abi.ERR_NONFINITE
    e.upload(0, pv=clean["pv"], dv=clean["dv"], tv=clean["tv"] if e.ntv else None)
    _, res, _ = e.iterate(1, 2, 0.0)
    assert np.all(np.isfinite(res))


def test_block_index_out_of_range():
    c = cases.make("plain_small", scale=8)
    e = native.Engine(c)
    e.initialize(c["pv0"])
    lib = native.lib()
    assert lib.cfd3d_residual(e.h, 3, None, None, None, None) == abi.ERR_ARG
    assert lib.cfd3d_download_state(e.h, -1, None, None, None, None, None) == abi.ERR_ARG
    assert b"block" in lib.cfd3d_last_error(e.h)
    e.residual(0)   # still usable


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_sweep_wait_runs_out_and_the_handle_recovers(precision):
    """A dataflow sweep in which one chunk of cells never signals: its dependents' bounded
    waits run out, the launch completes and the host gets CFD3D_ERR_TIMEOUT; the next
    iteration is normal."""
    c = cases.make("cavitating", scale=8, fix_cav_clamp=1)
    e = native.Engine(c, precision=precision)
    e.initialize(c["pv0"])
    assert e.sweep_stall_test() == abi.ERR_TIMEOUT
    e.initialize(c["pv0"])
    _, res, _ = e.iterate(1, 1, 0.0)
    assert np.all(np.isfinite(res))


def test_dataflow_sweeps_equal_hyperplane_sweeps(monkeypatch):
    """The dataflow sweeps run each cell's arithmetic on the same inputs as the one-launch-
    per-hyperplane sweeps: the FP64 states agree to rounding (the two kernels may contract
    multiply-adds differently), and two dataflow runs agree bit for bit (the result does
    not depend on which CTA took which chunk)."""
    c = cases.make("batched", scale=8)
    c["cfg"]["fix_cav_clamp"] = 1
    out = []
    for mode in ("planes", "dataflow", "dataflow"):
        monkeypatch.setenv("CFD3D_SWEEP", mode)
        e = native.Engine(c, precision=abi.FP64)
        e.initialize(c["pv0"])
        for it in range(3):
            e.iterate(1, it + 1, 0.0)
        out.append([e.download(n)["pv"] for n in range(len(c["blocks"]))])
        e.close()
    for a, b, b2 in zip(*out):
        scale = np.abs(a).reshape(-1, a.shape[-1]).max(axis=0)
        assert (np.abs(a - b).reshape(-1, a.shape[-1]).max(axis=0) <= 1e-12 * scale).all()
        assert np.array_equal(b, b2)


def test_collapsed_cell_is_rejected_at_create():
    """The device metrics find a cell of zero volume (two node planes made to coincide) and
    create fails with a descriptor error, as the host check did; a good grid still builds."""
    c = cases.make("plain_small", scale=8)
    xyz = c["blocks"][0]["xyz"]
    xyz[3] = xyz[2]          # node planes k = 3 and k = 4 (Fortran numbering) coincide
    with pytest.raises(Cfd3dError) as ei:
        native.Engine(c)
    assert ei.value.code == abi.ERR_DESCRIPTOR
    assert "volume" in str(ei.value)
    native.Engine(cases.make("plain_small", scale=8))
