"""The CPU oracle (test infrastructure): self-consistency properties and golden fixtures.

Parity with the Fortran reference is unpinned (it cannot be built here and ships no
tests); these properties guard the restatement itself."""
import os

import numpy as np
import pytest

from cfd3d_gb300 import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_eos_reference_state(oracle):
    dv, tv = oracle.eos([101325.0], [300.0], [0.0], [0.0], prop=True)
    # IF97 region 1 liquid at 300 K / 0.101325 MPa; IAPWS viscosity ~8.5e-4 Pa s
    assert 996.0 < dv[0, 2] < 997.0
    assert 8.0e-4 < tv[0, 0] < 9.0e-4
    assert abs(oracle.lib().orc_pww(300.0) - 3536.6) < 1.0


def test_eos_derivatives_consistent(oracle):
    """dv(7,8) = d rho/d(p,T) and dv(11,12) = d h/d(p,T) of the mixture, by central differences."""
    rng = np.random.default_rng(0)
    n = 200
    p = rng.uniform(5e3, 3e5, n)
    t = rng.uniform(285.0, 315.0, n)
    y1 = rng.uniform(0.0, 1e-3, n)
    y2 = np.full(n, 1e-6)
    dv, _ = oracle.eos(p, t, y1, y2)
    hp, ht = p * 1e-6, 1e-4
    dpp, _ = oracle.eos(p + hp, t, y1, y2)
    dpm, _ = oracle.eos(p - hp, t, y1, y2)
    dtp, _ = oracle.eos(p, t + ht, y1, y2)
    dtm, _ = oracle.eos(p, t - ht, y1, y2)
    # only points whose vapour phase stays on one side of p_sat in the stencil
    psat = np.array([oracle.lib().orc_pww(x) for x in t])
    ok = np.abs(p - psat) > 10 * hp
    fd_rp = (dpp[:, 0] - dpm[:, 0]) / (2 * hp)
    fd_rt = (dtp[:, 0] - dtm[:, 0]) / (2 * ht)
    fd_hp = (dpp[:, 1] - dpm[:, 1]) / (2 * hp)
    fd_ht = (dtp[:, 1] - dtm[:, 1]) / (2 * ht)
    assert np.allclose(fd_rp[ok], dv[ok, 6], rtol=2e-4)
    assert np.allclose(fd_rt[ok], dv[ok, 7], rtol=2e-4)
    assert np.allclose(fd_hp[ok], dv[ok, 10], rtol=1e-3, atol=1e-9)
    assert np.allclose(fd_ht[ok], dv[ok, 11], rtol=2e-4)


def test_saturation_inverse(oracle):
    for t in (280.0, 300.0, 330.0, 400.0):
        p = oracle.lib().orc_pww(t)
        assert abs(oracle.lib().orc_tww(p) - t) < 1e-6


@pytest.mark.parametrize("over", [dict(), dict(nscheme=2, nmuscl=2, nlim=8), dict(nscheme=3, nlim=3),
                                  dict(nscheme=4, nmuscl=0), dict(iturb=-2)])
def test_uniform_flow_preserved(oracle, over):
    """A uniform free stream on the sheared grid gives a zero residual to roundoff
    (discrete geometric conservation + flux consistency + free-stream ghosts).  Viscous
    stencils reach the edge ghosts, which the reference fills as wall-wall edges, so
    the check covers the cells one layer away from the j/k boundaries."""
    c = cases.make("plain_small", scale=8)
    c["cfg"].update(over)
    npv = 7
    pv = np.zeros_like(c["pv0"][0])
    pv[..., 1] = c["cfg"]["uref"]
    pv[..., 4] = 300.0
    pv[..., 6] = 1e-7
    o = oracle.Oracle(c)
    o.initialize([pv])
    r = o.residual(0)["res"][1:-1, 1:-1, :]
    # scale: momentum flux through a face ~ (p + rho u^2) * area
    area = (1.0 / c["blocks"][0]["jmax"]) ** 2
    assert np.abs(r[..., 1:4]).max() < 1e-8 * (101325.0 + 1e5) * area
    assert np.abs(r[..., 0]).max() < 1e-9 * 1e4 * area
    del npv


def test_iterations_reduce_residual(oracle):
    c = cases.make("plain_small", scale=4)
    o = oracle.Oracle(c)
    o.initialize(c["pv0"])
    r = [o.iterate(1, n + 1)[1][0] for n in range(12)]
    assert r[-1] < 0.5 * r[0]


def test_multiblock_split_matches_single_block_residual(oracle):
    """Two point-matched blocks reproduce the single block's residual away from the
    block-edge ghost regions (3-layer halos + metric halos)."""
    from cfd3d_gb300.abi import BC_FARFIELD, BC_SYMMETRY
    single = cases.make("plain_small", scale=4)
    xyz = single["blocks"][0]["xyz"]
    nk, nj, ni, _ = xyz.shape
    h = (ni - 1) // 2
    a, b = xyz[:, :, : h + 1], xyz[:, :, h:]
    J, K = nj, nk
    Ia, Ib = a.shape[2], b.shape[2]
    ba = {"imax": Ia, "jmax": J, "kmax": K, "xyz": a,
          "bc": cases.face_patches(Ia, J, K, {"imin": BC_FARFIELD, "jmin": BC_SYMMETRY, "jmax": BC_SYMMETRY,
                                              "kmin": BC_SYMMETRY, "kmax": BC_SYMMETRY}),
          "con": [{"donor": 1, "pnts": (Ia, 1, 1, Ia, J, K), "pnts_donor": (1, 1, 1, 1, J, K), "transform": (1, 2, 3)}]}
    bb = {"imax": Ib, "jmax": J, "kmax": K, "xyz": b,
          "bc": cases.face_patches(Ib, J, K, {"imax": BC_FARFIELD, "jmin": BC_SYMMETRY, "jmax": BC_SYMMETRY,
                                              "kmin": BC_SYMMETRY, "kmax": BC_SYMMETRY}),
          "con": [{"donor": 0, "pnts": (1, 1, 1, 1, J, K), "pnts_donor": (Ia, 1, 1, Ia, J, K), "transform": (1, 2, 3)}]}
    split = {"cfg": dict(single["cfg"]), "blocks": [ba, bb]}
    pv = single["pv0"][0]
    o1 = oracle.Oracle(single)
    o1.initialize([pv])
    o2 = oracle.Oracle(split)
    o2.initialize([pv[:, :, : Ia - 1], pv[:, :, Ia - 1:]])
    r1 = o1.residual(0)["res"]
    r2a = o2.residual(0)["res"]
    r2b = o2.residual(1)["res"]
    r2 = np.concatenate([r2a, r2b], axis=2)
    core = (slice(2, -2), slice(2, -2), slice(None))
    scale = np.maximum(np.abs(r1).max(axis=(0, 1, 2)), 1e-300)
    err = np.abs(r1[core] - r2[core]).max(axis=(0, 1, 2)) / scale
    assert err.max() < 1e-12, err


def _split_i(single, kinds_a, kinds_b):
    """The single block of `single` cut into two point-matched blocks along i."""
    xyz = single["blocks"][0]["xyz"]
    nk, nj, ni, _ = xyz.shape
    h = (ni - 1) // 2
    a, b = xyz[:, :, : h + 1], xyz[:, :, h:]
    J, K = nj, nk
    Ia, Ib = a.shape[2], b.shape[2]
    ba = {"imax": Ia, "jmax": J, "kmax": K, "xyz": a, "bc": cases.face_patches(Ia, J, K, kinds_a),
          "con": [{"donor": 1, "pnts": (Ia, 1, 1, Ia, J, K), "pnts_donor": (1, 1, 1, 1, J, K), "transform": (1, 2, 3)}]}
    bb = {"imax": Ib, "jmax": J, "kmax": K, "xyz": b, "bc": cases.face_patches(Ib, J, K, kinds_b),
          "con": [{"donor": 0, "pnts": (1, 1, 1, 1, J, K), "pnts_donor": (Ia, 1, 1, Ia, J, K), "transform": (1, 2, 3)}]}
    pv = single["pv0"][0]
    return {"cfg": dict(single["cfg"]), "blocks": [ba, bb], "pv0": [pv[:, :, : Ia - 1], pv[:, :, Ia - 1:]]}


def test_surface_tension_split_matches_single_block(oracle):
    """The surface-tension source (csf = 1) on the cavitating start, whose vapour sphere
    straddles the cut: two point-matched blocks reproduce the single block's residual and
    source, which needs the volume-fraction gradient's halo (setbc_vfg) at the cut.  The
    source is not zero, and uniform flow (no interface) gets none."""
    from cfd3d_gb300.abi import BC_FARFIELD, BC_SYMMETRY
    single = cases.make("cavitating", scale=8, fix_cav_clamp=1)
    single["cfg"]["csf"] = 1
    sym = {"jmin": BC_SYMMETRY, "jmax": BC_SYMMETRY, "kmin": BC_SYMMETRY, "kmax": BC_SYMMETRY}
    split = _split_i(single, dict(sym, imin=BC_FARFIELD), dict(sym, imax=BC_FARFIELD))
    o1 = oracle.Oracle(single)
    o1.initialize(single["pv0"])
    o2 = oracle.Oracle(split)
    o2.initialize(split["pv0"])
    r1 = o1.residual(0)["res"]
    c1 = o1.get_csf(0)["csf"]
    r2 = np.concatenate([o2.residual(0)["res"], o2.residual(1)["res"]], axis=2)
    c2 = np.concatenate([o2.get_csf(0)["csf"], o2.get_csf(1)["csf"]], axis=2)
    assert np.abs(c1).max() > 0.0
    core = (slice(2, -2), slice(2, -2), slice(None))
    scale = np.maximum(np.abs(r1).max(axis=(0, 1, 2)), 1e-300)
    assert (np.abs(r1[core] - r2[core]).max(axis=(0, 1, 2)) / scale).max() < 1e-12
    assert np.abs(c1[core] - c2[core]).max() <= 1e-12 * np.abs(c1).max()
    uni = cases.make("cavitating", scale=8, fix_cav_clamp=1)
    uni["cfg"]["csf"] = 1
    ou = oracle.Oracle(uni)
    pv = uni["pv0"][0].copy()
    pv[..., :] = pv[0, 0, 0, :]
    pv[..., 5] = 0.0
    ou.initialize([pv])
    ou.residual(0)
    assert np.abs(ou.get_csf(0)["csf"]).max() == 0.0


def test_totalpressure_inlet_pooled_across_blocks(oracle):
    """A total-pressure inlet on a k face split over two blocks: the reference reduces its
    averages over every rank carrying the inlet (one communicator), so the split case
    reproduces the single block's residual next to the inlet, not per-block averages."""
    from cfd3d_gb300.abi import BC_TOTALPRESSURE_IN
    single = cases.make("large", scale=16)
    single["cfg"].update(fix_cav_clamp=1, nsteady=0)
    for b in single["blocks"]:
        im, jm, km = b["imax"], b["jmax"], b["kmax"]
        b["bc"] = [(BC_TOTALPRESSURE_IN if tuple(p) == (1, 1, 1, im, jm, 1) else k, p) for k, p in b["bc"]]
    split = cases.split_i(single, 2)
    assert sum(k == BC_TOTALPRESSURE_IN for b in split["blocks"] for k, _ in b["bc"]) == 2
    o1 = oracle.Oracle(single)
    o1.initialize(single["pv0"])
    o2 = oracle.Oracle(split)
    o2.initialize(split["pv0"])
    r1 = o1.residual(0)["res"]
    r2 = np.concatenate([o2.residual(0)["res"], o2.residual(1)["res"]], axis=2)
    # away from the split's own halo seam: cells next to the inlet (k = 0) included
    ia = split["blocks"][0]["imax"] - 1
    core = np.ones(r1.shape[2], dtype=bool)
    core[ia - 2:ia + 2] = False
    core[:2] = core[-2:] = False
    scale = np.maximum(np.abs(r1).max(axis=(0, 1, 2)), 1e-300)
    err = np.abs(r1[:-2, 2:-2, core] - r2[:-2, 2:-2, core]).max(axis=(0, 1, 2)) / scale
    assert err.max() < 1e-10, err


def test_golden_fixtures(oracle):
    """The oracle reproduces its committed golden vectors (regression pin)."""
    g = np.load(os.path.join(GOLDEN, "eos_points.npz"))
    dv, tv = oracle.eos(g["p"], g["t"], g["y1"], g["y2"], prop=True)
    assert np.array_equal(dv, g["dv"]) or np.abs(dv - g["dv"]).max() <= 1e-15 * np.abs(g["dv"]).max()
    assert np.allclose(tv, g["tv"], rtol=1e-14, atol=0)
    for name in ("plain_small", "cavitating"):
        f = np.load(os.path.join(GOLDEN, f"residual_{name}.npz"))
        kw = {"scale": int(f["scale"])}
        c = cases.make(name, **kw)
        o = oracle.Oracle(c)
        o.initialize(c["pv0"])
        r = o.residual(0)["res"]
        s = np.abs(f["res"]).max()
        assert np.abs(r - f["res"]).max() <= 1e-12 * s
        o.iterate(1, 1)
        st = o.get_state(0)
        assert np.abs(st["pv"] - f["pv1"]).max() <= 1e-10 * np.abs(f["pv1"]).max()
