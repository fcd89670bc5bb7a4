"""Discrete adjoint (cfd3d_residual_vjp) against central finite differences.

R(pv) is the FP64 residual with each interior cell's dv and tv(1:2) its EOS and the eddy
viscosity tv(3) and history held (cfd3d_gb300.adjoint.StateSetter).  The state is the
cavitating SST block of cases.adjoint (pressure, velocity and vapour fraction noisy) with
noise added to T, y2, k and omega as well, so that no limiter, min / max or clip sits on
a tie, and two bands of cells just below and above the vapour pressure, where vaporisation
and condensation are active.  Checks, each at <= 1e-6 relative:
  * entries of (dR/dpv)^T lambda at cells across the block (boundary rows included)
    against lambda . (R(pv + h e) - R(pv - h e)) / 2h of the GPU residual, h = 1e-6 |x|;
  * the same against the oracle's residual (CPU restatement of the reference);
  * the parameter gradients (uref, c_v, c_c) against differences of engines built with
    the perturbed parameter;
  * the torch.autograd.Function wrapper's backward equals the ABI's result.
An entry whose difference quotient changes between h and h/2 by more than 1e-7 sits on a
switch (limiter branch, upwinding) within the step and is skipped; at most a few may be.
"""
import numpy as np
import pytest

from cfd3d_gb300 import abi, adjoint, cases, native

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _state(scale, seed=11):
    c = cases.adjoint(scale=scale)
    # the intended cavitation clamp: with the reference's (temperature-indexed) clamp the
    # vaporisation rate is its clamp value and does not depend on c_v
    c["cfg"]["fix_cav_clamp"] = 1
    rng = np.random.default_rng(seed)
    pv = c["pv0"][0].copy()
    sh = pv.shape[:-1]
    pv[..., 4] = 300.0 + rng.normal(0.0, 0.05, size=sh)
    pv[..., 6] = 1e-7 * (1.0 + 0.1 * rng.normal(size=sh))
    # two bands of cells 0.2-0.8 % below and above the vapour pressure: vaporisation and
    # condensation are active there and below their clamps, so that they depend on c_v, c_c
    w = max(sh[2] // 8, 2)
    for b0, sgn in ((0, -1.0), (w, 1.0)):
        band = pv[:, :, b0:b0 + w, 4]
        dev = 0.002 + 0.006 * rng.random(size=band.shape)
        pv[:, :, b0:b0 + w, 0] = np.vectorize(cases.pww_iapws)(band) * (1.0 + sgn * dev) - c["cfg"]["pref"]
    pv[..., 7] *= 1.0 + 0.05 * rng.normal(size=sh)
    pv[..., 8] *= 1.0 + 0.05 * rng.normal(size=sh)
    c["pv0"] = [pv]
    return c


def _engine(c, cfg=None):
    cc = dict(c)
    if cfg is not None:
        cc["cfg"] = cfg
    return native.Engine(cc, precision=abi.FP64)


def _with_inout(c):
    """subsonic inflow at imin and subsonic outflow at imax instead of the far field"""
    for b in c["blocks"]:
        im, jm, km = b["imax"], b["jmax"], b["kmax"]
        repl = {(1, 1, 1, 1, jm, km): abi.BC_INFLOW_SUBSONIC, (im, 1, 1, im, jm, km): abi.BC_OUTFLOW_SUBSONIC}
        b["bc"] = [(repl.get(tuple(p), k), p) for k, p in b["bc"]]
    return c


def _with_massflow_crwall(c):
    """bcmassflowratein at imin and the counter-rotating SST wall at jmin"""
    for b in c["blocks"]:
        im, jm, km = b["imax"], b["jmax"], b["kmax"]
        repl = {(1, 1, 1, 1, jm, km): abi.BC_MASSFLOWRATE_IN, (1, 1, 1, im, 1, km): abi.BC_WALL_COUNTERROTATING}
        b["bc"] = [(repl.get(tuple(p), k), p) for k, p in b["bc"]]
    return c


def _with_heatflux(c):
    """the jmin wall a HeatFlux-family wall with a constant history"""
    for b in c["blocks"]:
        im, jm, km = b["imax"], b["jmax"], b["kmax"]
        b["bc"] = [(abi.BC_WALL_HEATFLUX if tuple(p) == (1, 1, 1, im, 1, km) else k, p) for k, p in b["bc"]]
        q = next(n for n, (k, _) in enumerate(b["bc"]) if k == abi.BC_WALL_HEATFLUX)
        b["heatflux"] = {q: (np.array([0.0, 1.0]), np.array([150.0, 150.0]))}
    return c


def _prepared(scale, inout=False, massflow=False, heatflux=False, ncav=None):
    c = _state(scale)
    if ncav is not None:
        c["cfg"]["ncav"] = ncav
    if inout:
        c = _with_inout(c)
    if massflow:
        c = _with_massflow_crwall(c)
    if heatflux:
        c = _with_heatflux(c)
    e = _engine(c)
    e.initialize(c["pv0"])
    s = adjoint.StateSetter(e)
    pv = s.interior(0)
    res = s.residual([pv])[0]
    rng = np.random.default_rng(5)
    scale_v = np.abs(res).reshape(-1, res.shape[-1]).max(axis=0)
    lam = rng.normal(size=res.shape) / np.maximum(scale_v, 1e-300)
    g, gpar = e.residual_vjp([lam])
    return dict(case=c, e=e, s=s, pv=pv, lam=lam, g=g[0], gpar=gpar)


@pytest.fixture(scope="module")
def c4():
    return _prepared(1)


@pytest.fixture(scope="module")
def c4_small():
    return _prepared(4)


@pytest.fixture(scope="module")
def c4_inout():
    return _prepared(4, inout=True)


@pytest.fixture(scope="module")
def c4_massflow():
    return _prepared(4, massflow=True)


@pytest.fixture(scope="module")
def c4_heatflux():
    return _prepared(4, heatflux=True)


@pytest.fixture(scope="module", params=[2, 3, 4, 5], ids=["kunz", "singhal", "schnerr_sauer", "lee"])
def c4_model(request):
    return _prepared(4, ncav=request.param)


def _typical(pv, v):
    """typical magnitude of variable v: the floor of its finite-difference step"""
    return np.abs(pv[..., v]).mean()


def _entries(shape, nv, n, seed):
    rng = np.random.default_rng(seed)
    km, jm, im = shape
    out = []
    for q in range(n):
        k = int(rng.integers(0, km)); j = int(rng.integers(0, jm)); i = int(rng.integers(0, im))
        if q % 3 == 0:   # boundary rows: ghosts of the far-field, wall and symmetry patches
            i = 0 if q % 2 == 0 else im - 1
        if q % 3 == 1:
            j = 0 if q % 2 == 0 else jm - 1
        out.append((k, j, i, q % nv))
    return out


def _fd(resid, pv, lam, k, j, i, v, h):
    p = pv.copy()
    p[k, j, i, v] += h
    rp = resid(p)
    p[k, j, i, v] -= 2.0 * h
    rm = resid(p)
    return float(np.sum(lam * (rp - rm)) / (2.0 * h))


def _check(resid, d, entries):
    pv, lam, g = d["pv"], d["lam"], d["g"]
    gmax = np.abs(g).max()
    used, errs, rows = 0, [], []
    for (k, j, i, v) in entries:
        h = 1e-6 * max(abs(pv[k, j, i, v]), _typical(pv, v))
        f1 = _fd(resid, pv, lam, k, j, i, v, h)
        f2 = _fd(resid, pv, lam, k, j, i, v, 0.5 * h)
        ga = g[k, j, i, v]
        rows.append((k, j, i, v, f1, f2, ga))
        if abs(f1 - f2) > 1e-7 * max(abs(f1), abs(f2), 1e-4 * gmax):
            continue
        used += 1
        errs.append(abs(f2 - ga) / max(abs(ga), abs(f2), 1e-4 * gmax))
    return used, np.array(errs), rows


def test_vjp_state_against_fd_of_gpu_residual(c4):
    d = c4
    s = d["s"]
    entries = _entries(d["pv"].shape[:-1], d["pv"].shape[-1], 27, 1)
    used, errs, rows = _check(lambda p: s.residual([p])[0], d, entries)
    print(f"GPU residual: {used}/{len(entries)} entries, max relative error {errs.max():.2e}")
    assert used >= len(entries) - 3, rows
    assert errs.max() <= TOL, (errs, rows)


def test_vjp_state_against_fd_of_oracle_residual(c4_small):
    from oracle import oracle_py
    d = c4_small
    c = d["case"]
    base = d["s"].base[0]
    o = oracle_py.Oracle(c)
    o.initialize(c["pv0"])
    o.set_state(0, pv=base["pv"], dv=base["dv"], tv=base["tv"], qq=base["qq"])
    pref = float(c["cfg"]["pref"])
    prop = int(c["cfg"]["iturb"]) != -3

    def resid(p):
        pv = base["pv"].copy()
        dv = base["dv"].copy()
        tv = base["tv"].copy()
        pv[3:-3, 3:-3, 3:-3, :] = p
        flat = p.reshape(-1, p.shape[-1])
        dd, tt = oracle_py.eos(flat[:, 0] + pref, flat[:, 4], flat[:, 5], flat[:, 6], fluid=2, prop=prop)
        dv[3:-3, 3:-3, 3:-3, :] = dd.reshape(p.shape[:-1] + (18,))
        tv[3:-3, 3:-3, 3:-3, :2] = tt.reshape(p.shape[:-1] + (2,))
        o.set_state(0, pv=pv, dv=dv, tv=tv)
        return o.residual(0)["res"]

    entries = _entries(d["pv"].shape[:-1], d["pv"].shape[-1], 18, 2)
    used, errs, rows = _check(resid, d, entries)
    print(f"oracle residual: {used}/{len(entries)} entries, max relative error {errs.max():.2e}")
    assert used >= len(entries) - 2, rows
    assert errs.max() <= TOL, (errs, rows)


def test_vjp_parameters_against_fd(c4_small):
    d = c4_small
    c, lam = d["case"], d["lam"]
    base = d["s"].base[0]
    for q, name in enumerate(["uref", "c_v", "c_c"]):
        x0 = float(c["cfg"][name])
        h = 1e-6 * abs(x0)
        r = []
        for sgn in (1.0, -1.0):
            cfg = dict(c["cfg"])
            cfg[name] = x0 + sgn * h
            e2 = _engine(c, cfg)
            e2.upload(0, pv=base["pv"], dv=base["dv"], tv=base["tv"], qq=base["qq"] if e2.nqq else None)
            r.append(e2.residual(0)["res"])
            e2.close()
        fd = float(np.sum(lam * (r[0] - r[1])) / (2.0 * h))
        ga = d["gpar"][q]
        assert ga != 0.0, name
        print(f"d/d{name}: vjp {ga:.12e} fd {fd:.12e} relative error {abs(fd - ga) / max(abs(fd), abs(ga)):.2e}")
        assert abs(fd - ga) <= TOL * max(abs(fd), abs(ga)), (name, fd, ga)


def test_autograd_function_backward_is_the_vjp(c4_small):
    torch = pytest.importorskip("torch")
    d = c4_small
    fn = adjoint.residual_function()
    x = torch.tensor(d["pv"].reshape(-1), dtype=torch.float64, requires_grad=True)
    r = fn.apply(x, d["s"])
    lam = torch.tensor(d["lam"].reshape(-1), dtype=torch.float64)
    (r * lam).sum().backward()
    got = x.grad.numpy().reshape(d["pv"].shape)
    # the reverse pass accumulates with atomics: equal up to the order of the sums
    assert np.abs(got - d["g"]).max() <= 1e-12 * np.abs(d["g"]).max()


def test_vjp_is_linear_in_the_cotangent(c4_small):
    d = c4_small
    e = d["e"]
    d["s"].apply([d["pv"]])
    lam2 = np.random.default_rng(9).normal(size=d["lam"].shape) * np.abs(d["lam"]).mean()
    g1, p1 = e.residual_vjp([d["lam"]])
    g2, p2 = e.residual_vjp([lam2])
    g3, p3 = e.residual_vjp([2.0 * d["lam"] - 3.0 * lam2])
    ref = 2.0 * g1[0] - 3.0 * g2[0]
    assert np.abs(g3[0] - ref).max() <= 1e-9 * np.abs(ref).max()
    assert np.allclose(p3, 2.0 * p1 - 3.0 * p2, rtol=1e-9, atol=1e-9 * np.abs(p3).max())


def test_vjp_through_subsonic_inflow_and_outflow(c4_inout):
    """boundary rows next to bcinflowsubsonic / bcoutflowsubsonic ghosts"""
    d = c4_inout
    s = d["s"]
    km, jm, im = d["pv"].shape[:-1]
    entries = [(k, j, 0 if q % 2 == 0 else im - 1, v)
               for q, (k, j, _, v) in enumerate(_entries(d["pv"].shape[:-1], d["pv"].shape[-1], 18, 3))]
    used, errs, rows = _check(lambda p: s.residual([p])[0], d, entries)
    print(f"in/outflow rows: {used}/{len(entries)} entries, max relative error {errs.max():.2e}")
    assert used >= len(entries) - 2, rows
    assert errs.max() <= TOL, (errs, rows)


def test_vjp_through_massflow_inlet_and_counterrotating_wall(c4_massflow):
    """rows next to bcmassflowratein (i = 0) and the counter-rotating SST wall (j = 0)"""
    d = c4_massflow
    s = d["s"]
    km, jm, im = d["pv"].shape[:-1]
    base = _entries(d["pv"].shape[:-1], d["pv"].shape[-1], 18, 4)
    entries = [(k, j, 0, v) if q % 2 == 0 else (k, 0, i, v) for q, (k, j, i, v) in enumerate(base)]
    used, errs, rows = _check(lambda p: s.residual([p])[0], d, entries)
    print(f"mass-flow / counter-rotating rows: {used}/{len(entries)} entries, max relative error {errs.max():.2e}")
    assert used >= len(entries) - 2, rows
    assert errs.max() <= TOL, (errs, rows)


def test_vjp_through_heatflux_wall(c4_heatflux):
    """rows next to the heat-flux wall (j = 0), whose ghost temperature depends on the
    boundary cell's temperature, velocity and transport properties"""
    d = c4_heatflux
    s = d["s"]
    entries = [(k, 0, i, v) for (k, j, i, v) in _entries(d["pv"].shape[:-1], d["pv"].shape[-1], 18, 5)]
    used, errs, rows = _check(lambda p: s.residual([p])[0], d, entries)
    print(f"heat-flux wall rows: {used}/{len(entries)} entries, max relative error {errs.max():.2e}")
    assert used >= len(entries) - 2, rows
    assert errs.max() <= TOL, (errs, rows)


def test_vjp_cavitation_models(c4_model):
    """Kunz, Singhal, Schnerr-Sauer and Lee (src/cav_module.f90:173-357): rows of p, T, y1
    and y2 in the two bands next to the vapour pressure, where vaporisation and condensation
    are active, against finite differences of the GPU residual; and the gradients with
    respect to c_v and c_c against engines built with the perturbed coefficient"""
    d = c4_model
    s = d["s"]
    km, jm, im = d["pv"].shape[:-1]
    w = max(im // 8, 2)
    rng = np.random.default_rng(6)
    entries = [(int(rng.integers(0, km)), int(rng.integers(0, jm)), int(rng.integers(0, 2 * w)), v)
               for v in (0, 4, 5, 6) for _ in range(4)]
    used, errs, rows = _check(lambda p: s.residual([p])[0], d, entries)
    print(f"ncav {d['case']['cfg']['ncav']}: {used}/{len(entries)} entries, max relative error {errs.max():.2e}")
    assert used >= len(entries) - 2, rows
    assert errs.max() <= TOL, (errs, rows)
    c, lam = d["case"], d["lam"]
    base = d["s"].base[0]
    for q, name in ((1, "c_v"), (2, "c_c")):
        x0 = float(c["cfg"][name])
        h = 1e-6 * abs(x0)
        r = []
        for sgn in (1.0, -1.0):
            cfg = dict(c["cfg"])
            cfg[name] = x0 + sgn * h
            e2 = _engine(c, cfg)
            e2.upload(0, pv=base["pv"], dv=base["dv"], tv=base["tv"], qq=base["qq"] if e2.nqq else None)
            r.append(e2.residual(0)["res"])
            e2.close()
        fd = float(np.sum(lam * (r[0] - r[1])) / (2.0 * h))
        ga = d["gpar"][q]
        assert abs(fd - ga) <= TOL * max(abs(fd), abs(ga), 1e-12 * np.abs(d["g"]).max()), (name, fd, ga)
