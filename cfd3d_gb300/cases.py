"""Seeded synthetic cases standing in for the five benchmark configurations.

The reference ships no grids or datasets (its runs read user-supplied CGNS files), so
every case here is generated: node coordinates, BC patches in CGNS PointRange form,
1-to-1 connections, the solver configuration and the initial primitive state.
Names follow the configurations they stand for:

  plain_small      single block 64x32x32 cells, IAPWS liquid water, Roe, TVD minmod, Euler
  cavitating       single block 128x64x64, water/vapour, AUSM+-up, MLP, Merkle, laminar
  batched          24 uneven blocks (32^3 .. 96x64x48), 1-to-1 point-matched interfaces, SST
  adjoint          64^3 cavitating SST block from a perturbed converged-like state
  large            384x192x192 stretched wall-bounded SST cavitating block, BDF2 dual time

Every generator accepts a `scale` divisor so tests can run the same physics on small
grids.
"""
import math

import numpy as np

from .abi import BC_FARFIELD, BC_SYMMETRY, BC_WALL, sizes

PREF = 101325.0


def pww_iapws(t):
    """IF97 saturation pressure (the reference's h2o_pww, src/eos_module.f90:2266-2279)."""
    tt = min(max(t, 273.15), 647.096)
    theta = tt - 0.23855557567849 / (tt - 0.65017534844798e3)
    a = theta ** 2 + 0.11670521452767e4 * theta - 0.72421316703206e6
    b = -0.17073846940092e2 * theta ** 2 + 0.12020824702470e5 * theta - 0.32325550322333e7
    c = 0.14915108613530e2 * theta ** 2 - 0.48232657361591e4 * theta + 0.40511340542057e6
    return 1.0e6 * (2.0 * c / (-b + math.sqrt(b * b - 4.0 * a * c))) ** 4


def box_nodes(ni, nj, nk, lx, ly, lz, shear=0.0, seed=0, ystretch=None):
    """Node coordinates (nk+1, nj+1, ni+1, 3) of a sheared / stretched box.

    `shear` displaces interior nodes by shear * L * sin-products with seeded phases;
    `ystretch = (first_spacing, ratio)` clusters nodes geometrically towards y = 0."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, lx, ni + 1)
    if ystretch is None:
        y = np.linspace(0.0, ly, nj + 1)
    else:
        d0, r = ystretch
        dy = d0 * r ** np.arange(nj)
        # geometric growth capped at the uniform spacing of the remaining height
        y = np.zeros(nj + 1)
        for q in range(nj):
            rem = ly - y[q]
            cap = rem / (nj - q)
            y[q + 1] = y[q] + min(dy[q], cap)
        y *= ly / y[-1]
    z = np.linspace(0.0, lz, nk + 1)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    xyz = np.stack([X, Y, Z], axis=-1)
    if shear > 0.0:
        ph = rng.uniform(0.0, 2.0 * math.pi, size=(3, 3))
        sx, sy, sz = X / lx, Y / ly, Z / lz
        interior = np.zeros_like(X, dtype=bool)
        interior[1:-1, 1:-1, 1:-1] = True
        for d, L in enumerate((lx, ly, lz)):
            disp = shear * L * np.sin(2 * math.pi * sx + ph[d, 0]) * np.sin(2 * math.pi * sy + ph[d, 1]) * \
                np.sin(2 * math.pi * sz + ph[d, 2])
            if ystretch is not None and d == 1:
                disp *= 0.0
            xyz[..., d] = np.where(interior, xyz[..., d] + disp, xyz[..., d])
    return xyz


def face_patches(imax, jmax, kmax, kinds):
    """BC patches covering the six faces; kinds = dict face -> bc type (faces imin..kmax)."""
    full = {
        "imin": (1, 1, 1, 1, jmax, kmax), "imax": (imax, 1, 1, imax, jmax, kmax),
        "jmin": (1, 1, 1, imax, 1, kmax), "jmax": (1, jmax, 1, imax, jmax, kmax),
        "kmin": (1, 1, 1, imax, jmax, 1), "kmax": (1, 1, kmax, imax, jmax, kmax),
    }
    return [(kinds[f], full[f]) for f in ("imin", "imax", "jmin", "jmax", "kmin", "kmax") if f in kinds]


def _block(xyz, bc, con=None):
    nk, nj, ni, _ = xyz.shape
    return {"imax": ni, "jmax": nj, "kmax": nk, "xyz": xyz, "bc": bc, "con": con or []}


def _interior_centres(xyz):
    c = 0.125 * (xyz[:-1, :-1, :-1] + xyz[1:, :-1, :-1] + xyz[:-1, 1:, :-1] + xyz[:-1, :-1, 1:] +
                 xyz[1:, 1:, :-1] + xyz[1:, :-1, 1:] + xyz[:-1, 1:, 1:] + xyz[1:, 1:, 1:])
    return c  # (k, j, i, 3)


# ------------------------------------------------------------------------------------
def plain_small(scale=1, seed=0):
    """64x32x32 single-phase liquid, Roe + TVD minmod, Euler, steady LU-SGS."""
    ni, nj, nk = 64 // scale, 32 // scale, 32 // scale
    xyz = box_nodes(ni, nj, nk, 2.0, 1.0, 1.0, shear=0.02, seed=seed)
    bc = face_patches(ni + 1, nj + 1, nk + 1, {"imin": BC_FARFIELD, "imax": BC_FARFIELD, "jmin": BC_SYMMETRY,
                                               "jmax": BC_SYMMETRY, "kmin": BC_SYMMETRY, "kmax": BC_SYMMETRY})
    cfg = dict(iturb=-3, nscheme=1, nmuscl=1, nlim=1, timemethod=3, local=1, prec=1, cfl=5.0, fluid=2, ngas=1,
               ncav=0, pref=PREF, uref=10.0, tref=300.0, y1ref=0.0, y2ref=1e-7, l_chord=2.0, l_character=2.0,
               l_domain=2.0, dt_phy=1.0)
    blk = _block(xyz, bc)
    rng = np.random.default_rng(seed + 100)
    npv = sizes(cfg)[0]
    pv = np.zeros((nk, nj, ni, npv))
    pv[..., 1] = 10.0
    pv[..., 1:4] += rng.normal(0.0, 0.1, size=(nk, nj, ni, 3))
    pv[..., 4] = 300.0
    pv[..., 5] = 0.0
    pv[..., 6] = 1e-7
    return {"name": "plain_small", "cfg": cfg, "blocks": [blk], "pv0": [pv], "iterations": 100}


def vapour_mass_fraction(alpha, p, t, rho_l=996.5):
    """Mass fraction y1 of a vapour VOLUME fraction alpha (ideal-gas vapour density p/(R_v T))."""
    rho_v = p / (461.526 * t)
    return alpha * rho_v / (alpha * rho_v + (1.0 - alpha) * rho_l)


def _cavitating_state(blk, cfg, seed, u, sigma, turb=None, radius=0.1, length=1.0, alpha_max=0.5):
    """Water/vapour mixture at cavitation number sigma with a seeded spherical low-pressure
    region: p below p_sat inside, vapour VOLUME fraction alpha in [0, alpha_max] with a
    smooth (cosine) edge, converted to the mass fraction y1 the solver carries."""
    rng = np.random.default_rng(seed)
    npv = sizes(cfg)[0]
    xyz = blk["xyz"]
    cc = _interior_centres(xyz)
    nk, nj, ni = cc.shape[:3]
    pv = np.zeros((nk, nj, ni, npv))
    rho = 996.5
    psat = pww_iapws(cfg["tref"])
    pinf = psat + sigma * 0.5 * rho * u * u
    lo, hi = xyz.reshape(-1, 3).min(0), xyz.reshape(-1, 3).max(0)
    ctr = lo + (hi - lo) * np.array([0.3, 0.5, 0.5]) + rng.normal(0, 0.01, 3) * (hi - lo)
    r = np.linalg.norm(cc - ctr, axis=-1) / (radius * length)
    w = np.where(r < 1.0, 0.5 * (1.0 + np.cos(np.pi * np.minimum(r, 1.0))), 0.0)
    p = pinf + w * (0.8 * psat - pinf)
    pv[..., 0] = p - cfg["pref"]
    pv[..., 1] = u
    pv[..., 1:4] += rng.normal(0.0, 0.01 * u, size=(nk, nj, ni, 3))
    pv[..., 4] = cfg["tref"]
    alpha = alpha_max * w * rng.uniform(0.0, 1.0, size=r.shape)
    pv[..., 5] = vapour_mass_fraction(alpha, p, cfg["tref"])
    pv[..., 6] = 1e-7
    if turb is not None:
        k0, w0 = turb
        pv[..., 7] = k0
        pv[..., 8] = w0 * np.exp(rng.normal(0.0, 0.1, size=r.shape))
    return pv


def cavitating(scale=1, seed=1, nscheme=4, fix_cav_clamp=0):
    """128x64x64 water/vapour, AUSM-type flux, MLP, Merkle cavitation, laminar."""
    ni, nj, nk = 128 // scale, 64 // scale, 64 // scale
    xyz = box_nodes(ni, nj, nk, 2.0, 1.0, 1.0, shear=0.02, seed=seed)
    bc = face_patches(ni + 1, nj + 1, nk + 1, {"imin": BC_FARFIELD, "imax": BC_FARFIELD, "jmin": BC_SYMMETRY,
                                               "jmax": BC_SYMMETRY, "kmin": BC_SYMMETRY, "kmax": BC_SYMMETRY})
    u = 12.0
    psat = pww_iapws(300.0)
    pinf = psat + 0.8 * 0.5 * 996.5 * u * u
    cfg = dict(iturb=-2, nscheme=nscheme, nmuscl=2, nlim=8, timemethod=3, local=1, prec=1, cfl=2.0, fluid=2,
               ngas=1, ncav=1, c_v=100.0, c_c=100.0, pref=pinf, uref=u, tref=300.0, y1ref=0.0, y2ref=1e-7,
               l_chord=1.0, l_character=1.0, l_domain=2.0, dt_phy=1.0, fix_cav_clamp=fix_cav_clamp)
    blk = _block(xyz, bc)
    pv = _cavitating_state(blk, cfg, seed + 100, u, 0.8)
    return {"name": "cavitating", "cfg": cfg, "blocks": [blk], "pv0": [pv], "iterations": 500}


def _sst_cfg(u, pinf, length=1.0, extra=None):
    k0 = 1e-3 * u * u
    ell = 0.01 * length
    w0 = math.sqrt(k0) / (0.09 * ell)
    cfg = dict(iturb=0, ides=0, nscheme=4, nmuscl=2, nlim=8, timemethod=3, local=1, prec=1, cfl=2.0, fluid=2,
               ngas=1, ncav=1, c_v=100.0, c_c=100.0, pref=pinf, uref=u, tref=300.0, y1ref=0.0, y2ref=1e-7,
               l_chord=length, l_character=length, l_domain=2.0 * length, dt_phy=1.0, kinf=k0, oinf=w0)
    if extra:
        cfg.update(extra)
    return cfg, (k0, w0)


def batched(scale=1, seed=2, nblocks=24):
    """Uneven blocks from 32^3 to 96x64x48 cells in independent chains of point-matched
    blocks along x (identity transforms), same cavitating physics plus k-omega SST."""
    rng = np.random.default_rng(seed)
    u = 12.0
    psat = pww_iapws(300.0)
    pinf = psat + 0.8 * 0.5 * 996.5 * u * u
    cfg, turb = _sst_cfg(u, pinf)
    per_chain = 6
    nchains = max(1, nblocks // per_chain)
    blocks, pv0 = [], []
    for ch in range(nchains):
        nj = int(rng.integers(32, 65)) // scale
        nk = int(rng.integers(32, 49)) // scale
        nj, nk = max(nj, 4), max(nk, 4)
        nis = [max(int(rng.integers(32, 97)) // scale, 4) for _ in range(per_chain)]
        x0 = 0.0
        base = len(blocks)
        for q, ni in enumerate(nis):
            lx = ni / 64.0
            xyz = box_nodes(ni, nj, nk, lx, nj / 64.0, nk / 64.0, shear=0.0, seed=seed * 100 + len(blocks))
            xyz[..., 0] += x0
            x0 += lx
            kinds = {"jmin": BC_WALL, "jmax": BC_SYMMETRY, "kmin": BC_SYMMETRY, "kmax": BC_SYMMETRY}
            con = []
            I, J, K = ni + 1, nj + 1, nk + 1
            if q == 0:
                kinds["imin"] = BC_FARFIELD
            else:
                nip = nis[q - 1] + 1
                con.append({"donor": base + q - 1, "pnts": (1, 1, 1, 1, J, K), "pnts_donor": (nip, 1, 1, nip, J, K),
                            "transform": (1, 2, 3)})
            if q == per_chain - 1:
                kinds["imax"] = BC_FARFIELD
            else:
                con.append({"donor": base + q + 1, "pnts": (I, 1, 1, I, J, K), "pnts_donor": (1, 1, 1, 1, J, K),
                            "transform": (1, 2, 3)})
            bc = face_patches(I, J, K, kinds)
            blk = _block(xyz, bc, con)
            blocks.append(blk)
            pv0.append(_cavitating_state(blk, cfg, seed * 1000 + len(blocks), u, 0.8, turb=turb,
                                         radius=0.05, length=1.0))
    return {"name": "batched", "cfg": cfg, "blocks": blocks, "pv0": pv0, "iterations": 20}


def adjoint(scale=1, seed=3):
    """64^3 cavitating SST block from a converged-like state p0*(1+0.05*noise), y1 in [0,0.3]."""
    n = 64 // scale
    xyz = box_nodes(n, n, n, 1.0, 1.0, 1.0, shear=0.02, seed=seed)
    bc = face_patches(n + 1, n + 1, n + 1, {"imin": BC_FARFIELD, "imax": BC_FARFIELD, "jmin": BC_WALL,
                                            "jmax": BC_SYMMETRY, "kmin": BC_SYMMETRY, "kmax": BC_SYMMETRY})
    u = 12.0
    pinf = pww_iapws(300.0) + 0.8 * 0.5 * 996.5 * u * u
    cfg, turb = _sst_cfg(u, pinf)
    blk = _block(xyz, bc)
    rng = np.random.default_rng(seed + 100)
    npv = sizes(cfg)[0]
    pv = np.zeros((n, n, n, npv))
    pv[..., 0] = pinf * (1.0 + 0.05 * rng.normal(size=(n, n, n))) - cfg["pref"]
    pv[..., 1] = u + rng.normal(0.0, 0.1, size=(n, n, n))
    pv[..., 2:4] = rng.normal(0.0, 0.1, size=(n, n, n, 2))
    pv[..., 4] = 300.0
    pv[..., 5] = vapour_mass_fraction(rng.uniform(0.0, 0.3, size=(n, n, n)), pv[..., 0] + cfg["pref"], 300.0)
    pv[..., 6] = 1e-7
    pv[..., 7] = turb[0]
    pv[..., 8] = turb[1]
    return {"name": "adjoint", "cfg": cfg, "blocks": [blk], "pv0": [pv], "iterations": 1}


def large(scale=1, seed=4, nt_phy=20, ntmax=30):
    """384x192x192 stretched (wall spacing 1e-5 L, ratio 1.1) SST cavitating block with
    BDF2 dual time stepping; Re = 1e6 via L = 1 m.  Steady-form preconditioning (prec = 1):
    the unsteady form (prec = 2) floors the preconditioning speed at str = L / pi / dt_phy =
    477 m/s here, and from this synthetic start it diverges at CFL >= 0.5 (stable at CFL 0.1
    and below, or with dt_phy ten times larger), in the CPU restatement as in the engine."""
    ni, nj, nk = 384 // scale, 192 // scale, 192 // scale
    xyz = box_nodes(ni, nj, nk, 2.0, 1.0, 1.0, shear=0.0, seed=seed, ystretch=(1e-5 * scale, 1.1))
    bc = face_patches(ni + 1, nj + 1, nk + 1, {"imin": BC_FARFIELD, "imax": BC_FARFIELD, "jmin": BC_WALL,
                                               "jmax": BC_SYMMETRY, "kmin": BC_SYMMETRY, "kmax": BC_SYMMETRY})
    u = 15.0
    pinf = pww_iapws(300.0) + 0.8 * 0.5 * 996.5 * u * u
    dt_phy = 0.01 * 1.0 / u
    cfg, turb = _sst_cfg(u, pinf, extra=dict(nsteady=2, dt_phy=dt_phy, prec=1, npmax=nt_phy, ntmax=ntmax))
    blk = _block(xyz, bc)
    pv = _cavitating_state(blk, cfg, seed + 100, u, 0.8, turb=turb, radius=0.1)
    return {"name": "large", "cfg": cfg, "blocks": [blk], "pv0": [pv], "iterations": nt_phy * ntmax}


def split_i(case, nparts):
    """The single-block case cut along i into nparts point-matched blocks (1-to-1
    connections, identity transforms): the reference's decomposition of a block over
    MPI ranks, one block per rank (what its CPU build runs on several cores)."""
    assert len(case["blocks"]) == 1
    b = case["blocks"][0]
    imax = b["imax"]
    ncells = imax - 1
    nparts = max(1, min(nparts, ncells // 4))
    cuts = [round(q * ncells / nparts) for q in range(nparts + 1)]
    blocks, pv0 = [], []
    J, K = b["jmax"], b["kmax"]
    for q in range(nparts):
        c0, c1 = cuts[q], cuts[q + 1]          # cells c0..c1-1 (0-based), nodes c0+1..c1+1
        I = c1 - c0 + 1
        xyz = b["xyz"][:, :, c0:c1 + 1, :].copy()
        bc = []
        for kind, pn in b["bc"]:
            i1, j1, k1, i2, j2, k2 = pn
            if i1 == i2:   # an i-face patch: the first or the last part
                if i1 == 1 and q == 0:
                    bc.append((kind, (1, j1, k1, 1, j2, k2)))
                elif i1 == imax and q == nparts - 1:
                    bc.append((kind, (I, j1, k1, I, j2, k2)))
                continue
            lo, hi = max(i1, c0 + 1), min(i2, c1 + 1)
            if lo < hi:
                bc.append((kind, (lo - c0, j1, k1, hi - c0, j2, k2)))
        con = []
        if q > 0:
            nip = cuts[q] - cuts[q - 1] + 1
            con.append({"donor": q - 1, "pnts": (1, 1, 1, 1, J, K), "pnts_donor": (nip, 1, 1, nip, J, K),
                        "transform": (1, 2, 3)})
        if q < nparts - 1:
            con.append({"donor": q + 1, "pnts": (I, 1, 1, I, J, K), "pnts_donor": (1, 1, 1, 1, J, K),
                        "transform": (1, 2, 3)})
        blocks.append(_block(xyz, bc, con))
        pv0.append(case["pv0"][0][:, :, c0:c1, :].copy())
    out = dict(case)
    out["blocks"] = blocks
    out["pv0"] = pv0
    out["name"] = f"{case['name']} in {nparts} blocks along i"
    return out


CASES = {"plain_small": plain_small, "cavitating": cavitating, "batched": batched, "adjoint": adjoint,
         "large": large}


def make(name, **kw):
    return CASES[name](**kw)


def total_cells(case):
    return sum((b["imax"] - 1) * (b["jmax"] - 1) * (b["kmax"] - 1) for b in case["blocks"])
