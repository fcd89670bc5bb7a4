// adjoint_face.cu -- the face part of the discrete adjoint: per face, the vector-Jacobian
// product of its inviscid flux (src/flux_module.f90:198-641 with the reconstruction of
// src/muscl_module.f90:104-290) and its viscous flux (src/vsflux_module.f90:182-425) with
// respect to the face's stencil, the face cells' dv / tv and the free-stream speed.  The
// file comment of adjoint.cu describes the whole reverse pass.
#include "adjoint.cuh"

namespace cfd {

// ------------------------------------------------------------------ face adjoint
// seed layout of the inviscid pass
enum { S_PL = 0, S_PR = 9, S_RHOL = 18, S_HL, S_C2L, S_RHOR, S_HR, S_C2R, S_UREF = 24, S_SDST = 25, NS_INV = 43 };
// seed layout of the viscous pass
enum { V_GX = 0, V_GY = 6, V_GZ = 12, V_CC = 18, V_VIS = 24, V_CON, V_MUT, V_TCON, V_RHO, NS_VIS = 29 };

// Inviscid part of a face: lamF . dF/d(stencil pv, face-cell dv, uref).  Scatters into
// gpv / gdt and returns the uref gradient.
__device__ __noinline__ double adj_face_inviscid(const DevPtr& d, const Par& c, const AdjPtr& a, const double* nx,
                                                 long long g, long long gr, long long sn, long long s1, long long s2,
                                                 const double* lamF) {
  const long long n = d.ncell;
  const int npv = c.npv;
  const bool sensor = (c.nscheme == 2 || c.nscheme == 3);
  // ---- values: reconstruction, its clip decisions and the face EOS
  double pl[NPVM], pr[NPVM], c9[NPVM], c10[NPVM];
  int fl[NPVM], fr[NPVM];
  for (int v = 0; v < NPVM; ++v) { pl[v] = pr[v] = c9[v] = c10[v] = 0.0; fl[v] = fr[v] = 0; }
  for (int v = 0; v < npv; ++v) {
    if (c.nmuscl > 0) {
      double x[38];
      for (int l = 0; l < 38; ++l) x[l] = d.pv[v * n + stencil_cell(l, g, sn, s1, s2)];
      muscl_var<double>(c, x, pl[v], pr[v]);
      c9[v] = x[8]; c10[v] = x[9];
    } else {
      pl[v] = d.pv[v * n + g]; pr[v] = d.pv[v * n + gr];
    }
  }
  if (c.nmuscl > 0) clip_flags(c, c9, c10, pl, pr, fl, fr);
  double rl, hl, cl2, rr, hr, cr2;
  EosJac jl{}, jr{};
  if (c.nmuscl > 0) {
    jl = eos_jac(c.fluid, pl[0] + c.pref, pl[4], pl[5], pl[6]);
    jr = eos_jac(c.fluid, pr[0] + c.pref, pr[4], pr[5], pr[6]);
    rl = jl.rho; hl = jl.h; rr = jr.rho; hr = jr.h;
    cl2 = sensor ? jl.c2 : 0.0;   // the Roe and AUSM+-up fluxes do not read the face sound speeds
    cr2 = sensor ? jr.c2 : 0.0;
  } else {
    rl = d.dv[g]; hl = d.dv[n + g]; cl2 = d.dv[5 * n + g];
    rr = d.dv[gr]; hr = d.dv[n + gr]; cr2 = d.dv[5 * n + gr];
  }
  double sdv[18];
  for (int l = 0; l < 18; ++l) sdv[l] = sensor ? d.pv[stencil_cell(l, g, sn, s1, s2)] : 0.0;
  // Roe-average state and the derivatives of its sound speed in (p, T, y1, y2)
  FaceState Lv, Rv;
  for (int v = 0; v < NPVM; ++v) { Lv.pv[v] = pl[v]; Rv.pv[v] = pr[v]; }
  Lv.rho = rl; Lv.h = hl; Lv.c2 = cl2; Rv.rho = rr; Rv.h = hr; Rv.c2 = cr2;
  double rav[NPVM];
  for (int v = 0; v < NPVM; ++v) rav[v] = 0.0;
  roe_state<double>(npv, Lv, Rv, rav);
  const EosJac jc = eos_jac(c.fluid, rav[0] + c.pref, rav[4], rav[5], rav[6]);
  // ---- w = lamF . dF / d(seed), DC seeds per pass
  double w[NS_INV];
  for (int q = 0; q < NS_INV; ++q) w[q] = 0.0;
  const int nseed = sensor ? NS_INV : S_SDST;
  for (int k0 = 0; k0 < nseed; k0 += DC) {
    FaceStateT<DD> L, R;
    for (int v = 0; v < NPVM; ++v) { L.pv[v] = seed(pl[v], S_PL + v, k0); R.pv[v] = seed(pr[v], S_PR + v, k0); }
    L.rho = seed(rl, S_RHOL, k0); L.h = seed(hl, S_HL, k0); L.c2 = seed(cl2, S_C2L, k0);
    R.rho = seed(rr, S_RHOR, k0); R.h = seed(hr, S_HR, k0); R.c2 = seed(cr2, S_C2R, k0);
    DD ravg[NPVM];
    for (int v = 0; v < NPVM; ++v) ravg[v] = DD(0.0);
    roe_state<DD>(npv, L, R, ravg);
    const int am[4] = {0, 4, 5, 6};
    DD rc2(jc.c2);
    for (int m = 0; m < 4; ++m)
      for (int q = 0; q < DC; ++q) rc2.d[q] += jc.dc2[m] * ravg[am[m]].d[q];
    const DD uref = seed(c.uref, S_UREF, k0);
    DD sdst[18];
    for (int l = 0; l < 18; ++l) sdst[l] = seed(sdv[l], S_SDST + l, k0);
    DD fx[NPVM];
    inviscid_flux_core<DD>(c, nx, L, R, sdst, ravg, rc2, uref * uref, fx);
    for (int q = 0; q < DC && k0 + q < nseed; ++q) {
      double acc = 0.0;
      for (int v = 0; v < npv; ++v) acc += lamF[v] * fx[v].d[q];
      w[k0 + q] = acc;
    }
  }
  // ---- face densities / enthalpies / sound speeds: through the face EOS to the face
  //      states (reconstructed) or into the face cells' dv (first order)
  double gpl[NPVM], gpr[NPVM];
  for (int v = 0; v < NPVM; ++v) { gpl[v] = w[S_PL + v]; gpr[v] = w[S_PR + v]; }
  if (c.nmuscl > 0) {
    const int idx[4] = {0, 4, 5, 6};
    for (int m = 0; m < 4; ++m) {
      gpl[idx[m]] += w[S_RHOL] * jl.drho[m] + w[S_HL] * jl.dh[m] + w[S_C2L] * jl.dc2[m];
      gpr[idx[m]] += w[S_RHOR] * jr.drho[m] + w[S_HR] * jr.dh[m] + w[S_C2R] * jr.dc2[m];
    }
    // a clamped face state is a constant
    for (int v = 0; v < NPVM; ++v) {
      if (fl[v] == 2) gpl[v] = 0.0;
      if (fr[v] == 2) gpr[v] = 0.0;
    }
  } else {
    aadd(&a.gdt[GD_RHO * n + g], w[S_RHOL]); aadd(&a.gdt[GD_H * n + g], w[S_HL]); aadd(&a.gdt[GD_C2 * n + g], w[S_C2L]);
    aadd(&a.gdt[GD_RHO * n + gr], w[S_RHOR]); aadd(&a.gdt[GD_H * n + gr], w[S_HR]); aadd(&a.gdt[GD_C2 * n + gr], w[S_C2R]);
  }
  // ---- through the reconstruction, one variable at a time
  const int ncells = (c.nmuscl == 2) ? 38 : 6;
  for (int v = 0; v < npv; ++v) {
    if (gpl[v] == 0.0 && gpr[v] == 0.0) continue;
    if (c.nmuscl == 0) {
      aadd(&a.gpv[v * n + g], gpl[v]);
      aadd(&a.gpv[v * n + gr], gpr[v]);
      continue;
    }
    double gx[38];
    for (int l = 0; l < 38; ++l) gx[l] = 0.0;
    if (fl[v] == 1) gx[8] += gpl[v];
    if (fr[v] == 1) gx[9] += gpr[v];
    const bool lin = (fl[v] == 0 && gpl[v] != 0.0), rin = (fr[v] == 0 && gpr[v] != 0.0);
    if (lin || rin) {
      double xv[38];
      for (int l = 0; l < 38; ++l) xv[l] = d.pv[v * n + stencil_cell(l, g, sn, s1, s2)];
      for (int k0 = 0; k0 < ncells; k0 += DC) {
        DD x[38], xl, xr;
        for (int l = 0; l < 38; ++l) x[l] = DD(xv[l]);
        for (int q = 0; q < DC && k0 + q < ncells; ++q) {
          const int l = (c.nmuscl == 2) ? k0 + q : kMusclCells[k0 + q];
          x[l].d[q] = 1.0;
        }
        muscl_var<DD>(c, x, xl, xr);
        for (int q = 0; q < DC && k0 + q < ncells; ++q) {
          const int l = (c.nmuscl == 2) ? k0 + q : kMusclCells[k0 + q];
          if (lin) gx[l] += gpl[v] * xl.d[q];
          if (rin) gx[l] += gpr[v] * xr.d[q];
        }
      }
    }
    for (int l = 0; l < 38; ++l) aadd(&a.gpv[v * n + stencil_cell(l, g, sn, s1, s2)], gx[l]);
  }
  // pressure sensor stencil of Roe-M / AUSMPW+
  if (sensor)
    for (int l = 0; l < 18; ++l) aadd(&a.gpv[stencil_cell(l, g, sn, s1, s2)], w[S_SDST + l]);
  return w[S_UREF];
}

// Viscous part of a face: lamV . dV/d(stencil pv of u, v, w, T, k, omega; face-cell dv / tv)
__device__ __noinline__ void adj_face_viscous(const DevPtr& d, const Par& c, const AdjPtr& a, int dir, const double* nx,
                                              long long g, long long gr, long long sn, long long s1, long long s2,
                                              const double* lamV) {
  const long long n = d.ncell;
  const int npv = c.npv;
  const bool turb = (c.iturb == 0);
  const int ep = (dir == 0) ? GM_EX : (dir == 1 ? GM_TX : GM_CX);
  const int tp = (dir == 0) ? GM_TX : (dir == 1 ? GM_CX : GM_EX);
  double ev[3], tvv[3];
  for (int q = 0; q < 3; ++q) {
    const double* P = d.gm + (ep + q) * n;
    ev[q] = 0.25 * (P[g - s1] + P[g - s1 + sn] + P[g] + P[g + sn]);
    const double* T = d.gm + (tp + q) * n;
    tvv[q] = 0.25 * (T[g - s2] + T[g - s2 + sn] + T[g] + T[g + sn]);
  }
  const double vol = 2.0 / (d.gm[GM_GRD * n + g] + d.gm[GM_GRD * n + gr]);
  double tvl[3] = {0, 0, 0}, tvr[3] = {0, 0, 0};
  for (int q = 0; q < c.ntv; ++q) { tvl[q] = d.tv[q * n + g]; tvr[q] = d.tv[q * n + gr]; }
  const double vis = 0.5 * (tvl[0] + tvr[0]);
  const double con = 0.5 * (tvl[1] + tvr[1]);
  double emut = 0.0, tcon = 0.0, rho = 0.0, ydns = 0.0;
  const double cpl = d.dv[11 * n + g], cpr = d.dv[11 * n + gr];
  if (turb) {
    emut = 0.5 * (tvl[2] + tvr[2]);
    tcon = 0.5 * (tvl[2] * cpl + tvr[2] * cpr) / 0.9;
    rho = 0.5 * (d.dv[g] + d.dv[gr]);
    ydns = 0.5 * (d.gm[(GM_GRD + 4) * n + g] + d.gm[(GM_GRD + 4) * n + gr]);
  }
  const int vars[6] = {1, 2, 3, 4, 7, 8};
  const int nv = turb ? 6 : 4;
  double gxv[6], gyv[6], gzv[6], ccv[6];
  for (int q = 0; q < 6; ++q) gxv[q] = gyv[q] = gzv[q] = ccv[q] = 0.0;
  for (int q = 0; q < nv; ++q) {
    double x[18];
    for (int l = 0; l < 18; ++l) x[l] = d.pv[vars[q] * n + stencil_cell(l, g, sn, s1, s2)];
    face_gradient<double>(x, nx, ev, tvv, vol, gxv[q], gyv[q], gzv[q], ccv[q]);
  }
  double w[NS_VIS];
  for (int q = 0; q < NS_VIS; ++q) w[q] = 0.0;
  for (int k0 = 0; k0 < NS_VIS; k0 += DC) {
    DD gx[6], gy[6], gz[6], cc[6];
    for (int q = 0; q < 6; ++q) {
      gx[q] = seed(gxv[q], V_GX + q, k0); gy[q] = seed(gyv[q], V_GY + q, k0);
      gz[q] = seed(gzv[q], V_GZ + q, k0); cc[q] = seed(ccv[q], V_CC + q, k0);
    }
    DD fv[NPVM];
    vsflux_core<DD>(c, nx, gx, gy, gz, cc, seed(vis, V_VIS, k0), seed(con, V_CON, k0), seed(emut, V_MUT, k0),
                    seed(tcon, V_TCON, k0), seed(rho, V_RHO, k0), ydns, fv);
    for (int q = 0; q < DC && k0 + q < NS_VIS; ++q) {
      double acc = 0.0;
      for (int v = 0; v < npv; ++v) acc += lamV[v] * fv[v].d[q];
      w[k0 + q] = acc;
    }
  }
  // through the (linear) face gradients and averages to the stencil
  for (int q = 0; q < nv; ++q) {
    for (int l = 0; l < 18; ++l) {
      double cn, ce, ct, cc;
      grad_coeffs(l, cn, ce, ct, cc);
      const double dgx = (cn * nx[0] + ce * ev[0] + ct * tvv[0]) * vol;
      const double dgy = (cn * nx[1] + ce * ev[1] + ct * tvv[1]) * vol;
      const double dgz = (cn * nx[2] + ce * ev[2] + ct * tvv[2]) * vol;
      const double gs = w[V_GX + q] * dgx + w[V_GY + q] * dgy + w[V_GZ + q] * dgz + w[V_CC + q] * cc;
      aadd(&a.gpv[vars[q] * n + stencil_cell(l, g, sn, s1, s2)], gs);
    }
  }
  // face averages of the two cells' transport coefficients, specific heat and density
  const long long cl[2] = {g, gr};
  const double mut[2] = {tvl[2], tvr[2]}, cp[2] = {cpl, cpr};
  for (int s = 0; s < 2; ++s) {
    const long long q = cl[s];
    aadd(&a.gdt[GD_VIS * n + q], 0.5 * w[V_VIS]);
    aadd(&a.gdt[GD_CON * n + q], 0.5 * w[V_CON]);
    if (turb) {
      aadd(&a.gdt[GD_MUT * n + q], 0.5 * w[V_MUT] + w[V_TCON] * 0.5 * cp[s] / 0.9);
      aadd(&a.gdt[GD_CP * n + q], w[V_TCON] * 0.5 * mut[s] / 0.9);
      aadd(&a.gdt[GD_RHO * n + q], 0.5 * w[V_RHO]);
    }
  }
}

// One thread per face (the face numbering of k_face_flux).  Face g (between cells g and
// gr = g + sn) enters the residual of g as -F + V and of gr as +F - V.
__global__ void __launch_bounds__(64) k_adj_face(DevPtr d, Par c, AdjPtr a, int dir) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double wpar = 0.0;
  int b = 0;
  while (b + 1 < d.nblk && t >= d.blk[b + 1].face_off[dir]) ++b;
  const BlockGeom& B = d.blk[b];
  const long long loc = t - B.face_off[dir];
  int fi_, fj, fk;
  if (dir == 0) { fi_ = B.imax; fj = B.jmax - 1; fk = B.kmax - 1; }
  else if (dir == 1) { fi_ = B.imax - 1; fj = B.jmax; fk = B.kmax - 1; }
  else { fi_ = B.imax - 1; fj = B.jmax - 1; fk = B.kmax; }
  if (loc >= 0 && loc < (long long)fi_ * fj * fk) {
    const int i = (int)(loc % fi_) + (dir == 0 ? 1 : 2);
    const long long r = loc / fi_;
    const int j = (int)(r % fj) + (dir == 1 ? 1 : 2);
    const int k = (int)(r / fj) + (dir == 2 ? 1 : 2);
    const long long n = d.ncell;
    const long long si = 1, sj = B.ni, sk = (long long)B.ni * B.nj;
    const long long g = B.off + (i + 1) + sj * (j + 1) + sk * (k + 1);
    long long sn, s1, s2;
    if (dir == 0) { sn = si; s1 = sj; s2 = sk; }
    else if (dir == 1) { sn = sj; s1 = sk; s2 = si; }
    else { sn = sk; s1 = si; s2 = sj; }
    const long long gr = g + sn;
    double lamF[NPVM], lamV[NPVM];
    bool any = false;
    for (int v = 0; v < NPVM; ++v) {
      lamF[v] = (v < c.npv) ? a.lam[v * n + gr] - a.lam[v * n + g] : 0.0;
      lamV[v] = -lamF[v];
      any = any || (lamF[v] != 0.0);
    }
    if (any) {
      const int fplane = (dir == 0) ? GM_CX : (dir == 1 ? GM_EX : GM_TX);
      double nx[3];
      face_vec(d, fplane, g, nx);
      wpar = adj_face_inviscid(d, c, a, nx, g, gr, sn, s1, s2, lamF);
      if (c.iturb != -3) adj_face_viscous(d, c, a, dir, nx, g, gr, sn, s1, s2, lamV);
    }
  }
  // one atomic per warp for the free-stream-speed gradient
  for (int o = 16; o > 0; o >>= 1) wpar += __shfl_down_sync(0xffffffffu, wpar, o);
  if ((threadIdx.x & 31) == 0) aadd(&a.gpar[0], wpar);
}

void launch_adj_face(const Engine& E, const AdjPtr& a, cudaStream_t s) {
  const int T = 64;
  for (int dir = 0; dir < 3; ++dir)
    k_adj_face<<<(unsigned)((E.nface[dir] + T - 1) / T), T, 0, s>>>(E.d, E.par, a, dir);
}

}  // namespace cfd
