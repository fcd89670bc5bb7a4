"""The checkpoint file's layout (oracle) and the solve loop's export / restart points,
on the CPU.  The engine's own writer and reader are compared with the oracle byte for byte
in test_gpu_checkpoint.py."""
import numpy as np
import pytest

from cfd3d_gb300 import native
from oracle import oracle_checkpoint as ock

DIMS = [(9, 5, 7), (4, 6, 5), (13, 3, 4)]


def _blocks(dims):
    return [dict(imax=i, jmax=j, kmax=k) for i, j, k in dims]


def _reference_disp(rank, dims, npv, nqq, turb, cav, with_qq=True, csf=False):
    """The displacement loop of t_variable%construct (src/variable_module.f90:80-91),
    term by term, with intsize = 4 and realsize = 8."""
    intsize, realsize = 4, 8
    disp = 0
    for i in range(rank):
        im, jm, km = dims[i]
        disp += intsize * 2 + realsize + realsize * npv * (im + 5) * (jm + 5) * (km + 5)
        if with_qq:
            disp += realsize * nqq * npv * (im - 1) * (jm - 1) * (km - 1)
        if turb:
            disp += realsize * (im + 5) * (jm + 5) * (km + 5)
        if cav:
            disp += realsize * 2 * (im - 1) * (jm - 1) * (km - 1)
        if csf:
            disp += realsize * 3 * (im - 1) * (jm - 1) * (km - 1)
    return disp


CFGS = [dict(iturb=-3, ncav=0, nsteady=0), dict(iturb=-2, ncav=1, nsteady=0), dict(iturb=-2, ncav=1, nsteady=0, csf=1),
        dict(iturb=0, ncav=1, nsteady=2), dict(iturb=0, ncav=0, nsteady=1)]


@pytest.mark.parametrize("cfg", CFGS)
@pytest.mark.parametrize("with_qq", [True, False])
def test_displacements_follow_the_reference_formula(cfg, with_qq):
    npv = 9 if cfg["iturb"] == 0 else 7
    nqq = 2 if cfg["nsteady"] else 0
    turb, cav = ock.flags(cfg)
    csf = ock.csf_flag(cfg)
    disp, total = ock.displacements(cfg, _blocks(DIMS), npv, nqq, with_qq)
    for r in range(len(DIMS)):
        assert disp[r] == _reference_disp(r, DIMS, npv, nqq, turb, cav, with_qq, csf)
    assert total == _reference_disp(len(DIMS), DIMS, npv, nqq, turb, cav, with_qq, csf)


def _random_states(cfg, blocks, npv, nqq, rng):
    states = []
    for b in blocks:
        pad = (b["kmax"] + 5, b["jmax"] + 5, b["imax"] + 5)
        inner = (b["kmax"] - 1, b["jmax"] - 1, b["imax"] - 1)
        states.append(dict(pv=rng.standard_normal(pad + (npv,)), tv=rng.standard_normal(pad + (3,)),
                           qq=rng.standard_normal(inner + (max(nqq, 1) * npv,))[..., :nqq * npv],
                           rcav=rng.standard_normal(inner + (2,)), csf=rng.standard_normal(inner + (3,))))
    return states


@pytest.mark.parametrize("cfg", CFGS)
def test_oracle_write_read_round_trip(cfg, tmp_path):
    rng = np.random.default_rng(7)
    npv = 9 if cfg["iturb"] == 0 else 7
    nqq = 2 if cfg["nsteady"] else 0
    blocks = _blocks(DIMS)
    states = _random_states(cfg, blocks, npv, nqq, rng)
    path = tmp_path / "out_00000012.dat"
    data = ock.write_checkpoint(path, cfg, blocks, npv, nqq, 3, 12, 0.625, states)
    assert len(data) == ock.displacements(cfg, blocks, npv, nqq)[1]
    turb, cav = ock.flags(cfg)
    recs = ock.read_checkpoint(path, cfg, blocks, npv, nqq)
    for rec, s in zip(recs, states):
        assert (rec["nt_phy"], rec["nt"], rec["time"]) == (3, 12, 0.625)
        assert np.array_equal(rec["pv"], s["pv"])
        assert (rec["emut"] is not None) == turb
        if turb:
            assert np.array_equal(rec["emut"], s["tv"][..., 2])
        if nqq:
            assert np.array_equal(rec["qq"], s["qq"])
        assert (rec["rcav"] is not None) == cav
        if cav:
            assert np.array_equal(rec["rcav"], s["rcav"])
        assert (rec["csf"] is not None) == ock.csf_flag(cfg)
        if ock.csf_flag(cfg):
            assert np.array_equal(rec["csf"], s["csf"])
    with open(path, "r+b") as f:
        f.truncate(len(data) - 8)
    with pytest.raises(ValueError):
        ock.read_checkpoint(path, cfg, blocks, npv, nqq)


def test_restart_counters():
    assert ock.restart_counters(1, 40, 2.5, nsteady=0) == (1, 41, 2.5)
    assert ock.restart_counters(5, 30, 0.1, nsteady=2) == (6, 1, 0.1)
    assert ock.restart_counters(5, 30, 0.1, nsteady=2, steady_start=True) == (1, 1, 0.0)


class _FakeEngine:
    """Stands in for the device engine: records the solve loop's calls."""

    def __init__(self, npv, converge_at=None):
        self.npv = npv
        self.calls = []
        self.converge_at = converge_at or set()

    def initialize(self, pv0):
        self.calls.append(("init",))

    def checkpoint_write(self, path, nt_phy, nt, time):
        self.calls.append(("export", path.rsplit("/", 1)[-1], nt_phy, nt))

    def checkpoint_read(self, path, steady_start=False):
        self.calls.append(("restart", steady_start))
        return 2, 1, 0.5

    def iterate(self, nt_phy, nt, timeprev):
        self.calls.append(("iter", nt_phy, nt))
        res = np.ones(self.npv)
        if (nt_phy, nt) in self.converge_at:
            res[0] = 0.0
        return timeprev + nt, res, (0, 2, 2, 2)

    def unsteady_shift(self):
        self.calls.append(("shift",))


def _solver(cfg, engine):
    s = native.Solver.__new__(native.Solver)
    s.engine, s.cfg, s.case, s.log_path, s.history = engine, cfg, dict(cfg=cfg), None, []
    return s


def _exports(engine):
    return [c[1:] for c in engine.calls if c[0] == "export"]


def test_steady_export_points():
    cfg = dict(nsteady=0, npmax=1, ntmax=7, nexport=3, bond=12)
    e = _FakeEngine(7)
    _solver(cfg, e).solve(export_dir="d")
    assert _exports(e) == [("out_00000000.dat", 0, 0), ("out_00000003.dat", 1, 3), ("out_00000006.dat", 1, 6)]
    e = _FakeEngine(7, converge_at={(1, 5)})
    _solver(cfg, e).solve(export_dir="d")
    assert _exports(e) == [("out_00000000.dat", 0, 0), ("out_00000003.dat", 1, 3), ("out_00000005.dat", 1, 5)]
    assert [c for c in e.calls if c[0] == "iter"][-1] == ("iter", 1, 5)


def test_unsteady_export_points_and_restart():
    cfg = dict(nsteady=2, npmax=4, ntmax=3, nexport=2, bond=12)
    e = _FakeEngine(9, converge_at={(4, 2)})
    _solver(cfg, e).solve(export_dir="d")
    # after the history shift of every second physical step, with nt - 1 as nt: ntmax after
    # a full pseudo loop, one less than the converged iteration after an early exit
    assert _exports(e) == [("out_00000000.dat", 0, 0), ("out_00000002.dat", 2, 3), ("out_00000004.dat", 4, 1)]
    assert sum(1 for c in e.calls if c[0] == "shift") == 4
    e = _FakeEngine(9)
    _solver(cfg, e).solve(export_dir="d", restart="d/out_00000001.dat")
    assert e.calls[0] == ("restart", False)
    assert not any(c[0] == "init" for c in e.calls)
    assert [c for c in e.calls if c[0] == "iter"][0] == ("iter", 2, 1)
    assert _exports(e)[0] == ("out_00000002.dat", 2, 3)
