"""GPU parity: the CUDA engine (through the C ABI) against the CPU oracle.

Every case is one of the seeded synthetic configurations at a reduced size; the FP64
engine must reproduce the oracle's metrics, residual, implicit-source Jacobians and
updated state to the stated relative tolerances (normalised by each field's maximum,
since residuals are flux differences that pass through zero).
"""
import numpy as np
import pytest

from cfd3d_gb300 import cases, native
from tests.helpers import field_err, interior, rel_err

pytestmark = pytest.mark.gpu

# FP64 tolerances: rounding differs (FMA contraction, re-associated IF97 sums)
TOL_EOS = 1e-11
# stiffened water + ideal vapour: the sound-speed denominator cancels (all dh/dp = 0)
TOL_EOS_STIFFENED = 2e-9
TOL_METRIC = 1e-13
TOL_RES = 1e-9
TOL_STATE = 1e-9

CASES = {
    "plain_roe_tvd": ("plain_small", dict(scale=4), {}),
    "plain_roem_mlp": ("plain_small", dict(scale=4), dict(nscheme=2, nmuscl=2, nlim=8)),
    "plain_ausmpw_vl": ("plain_small", dict(scale=4), dict(nscheme=3, nmuscl=1, nlim=3)),
    "plain_ausmup_first": ("plain_small", dict(scale=4), dict(nscheme=4, nmuscl=0)),
    "cavitating": ("cavitating", dict(scale=8), {}),
    "cavitating_fixed": ("cavitating", dict(scale=8, fix_cav_clamp=1), {}),
    "adjoint_sst": ("adjoint", dict(scale=8), dict(fix_cav_clamp=1)),
    "large_sst_bdf2": ("large", dict(scale=16), dict(fix_cav_clamp=1)),
    "batched_multiblock": ("batched", dict(scale=4, nblocks=6), dict(fix_cav_clamp=1)),
    # the batched workload's 24 uneven blocks in four chains, at 1/8 of its extents
    "batched_24": ("batched", dict(scale=8, nblocks=24), dict(fix_cav_clamp=1)),
}


def make(name):
    base, kw, over = CASES[name]
    c = cases.make(base, **kw)
    c["cfg"].update(over)
    return c


def test_eos_matches_oracle(oracle):
    rng = np.random.default_rng(7)
    n = 20000
    p = rng.uniform(2e3, 3e5, n)
    t = rng.uniform(280.0, 320.0, n)
    y1 = rng.uniform(0.0, 0.5, n) * (rng.uniform(size=n) < 0.5)
    y2 = 10.0 ** rng.uniform(-7, -3, n)
    for prop in (False, True):
        dv, tv = native.eos_eval(p, t, y1, y2, fluid=2, prop=prop)
        dvo, tvo = oracle.eos(p, t, y1, y2, fluid=2, prop=prop)
        assert rel_err(dv, dvo, floor=1e-30).max() < TOL_EOS
        if prop:
            assert rel_err(tv, tvo).max() < TOL_EOS
    dv, tv = native.eos_eval(p, t, y1, y2, fluid=1, prop=True)
    dvo, tvo = oracle.eos(p, t, y1, y2, fluid=1, prop=True)
    assert rel_err(dv, dvo, floor=1e-30).max() < TOL_EOS_STIFFENED
    assert rel_err(tv, tvo).max() < TOL_EOS


@pytest.mark.parametrize("name", list(CASES))
def test_metrics_match(oracle, name):
    c = make(name)
    e = native.Engine(c)
    o = oracle.Oracle(c)
    for b in range(len(c["blocks"])):
        for x, y in zip(e.metrics(b), o.metrics(b)):
            assert field_err(x, y).max() < TOL_METRIC


@pytest.mark.parametrize("name", list(CASES))
def test_residual_matches(oracle, name):
    c = make(name)
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    for b in range(len(c["blocks"])):
        rg = e.residual(b)
        ro = o.residual(b)
        assert field_err(rg["res"], ro["res"]).max() < TOL_RES, name
        if c["cfg"].get("ncav", 0):
            assert field_err(rg["icav"], ro["icav"]).max() < TOL_RES
        if c["cfg"].get("iturb", -3) == 0:
            assert field_err(rg["itt"], ro["itt"]).max() < TOL_RES
            assert field_err(rg["omega_cut"][..., None], ro["omega_cut"][..., None]).max() < TOL_RES


@pytest.mark.parametrize("name", list(CASES))
def test_iterations_match(oracle, name):
    c = make(name)
    e = native.Engine(c)
    o = oracle.Oracle(c)
    e.initialize(c["pv0"])
    o.initialize(c["pv0"])
    nit = 3
    for it in range(nit):
        tg, resg, locg = e.iterate(1, it + 1, 0.0)
        to, reso, loco = o.iterate(1, it + 1, 0.0)
        assert abs(tg - to) <= 1e-9 * abs(to)
        assert np.allclose(resg, reso, rtol=1e-7, atol=1e-9 * np.abs(reso).max()), (it, resg, reso)
    for b in range(len(c["blocks"])):
        sg = e.download(b)
        so = o.get_state(b)
        assert field_err(interior(sg["pv"]), interior(so["pv"])).max() < TOL_STATE
        assert field_err(interior(sg["dv"]), interior(so["dv"])).max() < TOL_STATE
        if e.ntv:
            assert field_err(interior(sg["tv"]), interior(so["tv"])).max() < TOL_STATE
