// flux.cu -- face fluxes of the FP64 form.
//
// One thread per face and direction: MUSCL/MLP reconstruction of the 38-cell stencil
// (src/muscl_module.f90:104-290), the face-state EOS, the inviscid flux
// (src/flux_module.f90:198-641) and the viscous flux (src/vsflux_module.f90:182-425),
// written to fi / fv at the index of the face's left cell (rhs_module.f90:282-538).
#include "engine.cuh"

namespace cfd {

// ------------------------------------------------------------------ face fluxes
template <int DIR>
__global__ void __launch_bounds__(128) k_face_flux(DevPtr d, Par c) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  // flat face numbering per direction: block-major, then (k, j, i) of the left cell
  int b = 0;
  while (b + 1 < d.nblk && t >= d.blk[b + 1].face_off[DIR]) ++b;
  const BlockGeom& B = d.blk[b];
  long long loc = t - B.face_off[DIR];
  int fi_, fj, fk;  // extents of the face set
  if (DIR == 0) { fi_ = B.imax; fj = B.jmax - 1; fk = B.kmax - 1; }
  else if (DIR == 1) { fi_ = B.imax - 1; fj = B.jmax; fk = B.kmax - 1; }
  else { fi_ = B.imax - 1; fj = B.jmax - 1; fk = B.kmax; }
  if (loc < 0 || loc >= (long long)fi_ * fj * fk) return;
  int i = (int)(loc % fi_) + (DIR == 0 ? 1 : 2);
  long long r = loc / fi_;
  int j = (int)(r % fj) + (DIR == 1 ? 1 : 2);
  int k = (int)(r / fj) + (DIR == 2 ? 1 : 2);
  const long long n = d.ncell;
  const long long si = 1, sj = B.ni, sk = (long long)B.ni * B.nj;
  const long long g = B.off + (i + 1) + sj * (j + 1) + sk * (k + 1);
  long long sn, s1, s2;
  if (DIR == 0) { sn = si; s1 = sj; s2 = sk; }
  else if (DIR == 1) { sn = sj; s1 = sk; s2 = si; }
  else { sn = sk; s1 = si; s2 = sj; }
  const int fplane = (DIR == 0) ? GM_CX : (DIR == 1 ? GM_EX : GM_TX);
  double nx[3];
  face_vec(d, fplane, g, nx);
  const int npv = c.npv;
  FaceState L, R;
  const long long gr = g + sn;
  if (c.nmuscl > 0) {
    double c9[NPVM], c10[NPVM];
    for (int v = 0; v < npv; ++v) {
      double x[38];
#pragma unroll
      for (int l = 0; l < 38; ++l) x[l] = d.pv[v * n + stencil_cell(l, g, sn, s1, s2)];
      muscl_var<double>(c, x, L.pv[v], R.pv[v]);
      c9[v] = x[8]; c10[v] = x[9];
    }
    muscl_clip<double>(c, c9, c10, L.pv, R.pv);
    if (c.nscheme == 2 || c.nscheme == 3) {
      // Roe-M and AUSMPW+ also read the face sound speeds
      double dl_[NDV], dr_[NDV];
      deteos_simple<false>(c.fluid, L.pv[0] + c.pref, L.pv[4], L.pv[5], L.pv[6], dl_, &d.sc->snd2_fallbacks);
      deteos_simple<false>(c.fluid, R.pv[0] + c.pref, R.pv[4], R.pv[5], R.pv[6], dr_, &d.sc->snd2_fallbacks);
      L.rho = dl_[0]; L.h = dl_[1]; L.c2 = dl_[5];
      R.rho = dr_[0]; R.h = dr_[1]; R.c2 = dr_[5];
    } else {
      eos_rho_h<false>(c.fluid, L.pv[0] + c.pref, L.pv[4], L.pv[5], L.pv[6], L.rho, L.h);
      eos_rho_h<false>(c.fluid, R.pv[0] + c.pref, R.pv[4], R.pv[5], R.pv[6], R.rho, R.h);
      L.c2 = R.c2 = 0.0;
    }
  } else {
    for (int v = 0; v < npv; ++v) { L.pv[v] = d.pv[v * n + g]; R.pv[v] = d.pv[v * n + gr]; }
    L.rho = d.dv[g]; L.h = d.dv[n + g]; L.c2 = d.dv[5 * n + g];
    R.rho = d.dv[gr]; R.h = d.dv[n + gr]; R.c2 = d.dv[5 * n + gr];
  }
  double sdst[18];
  if (c.nscheme == 2 || c.nscheme == 3) {
#pragma unroll
    for (int l = 0; l < 18; ++l) sdst[l] = d.pv[stencil_cell(l, g, sn, s1, s2)];
  }
  double fx[NPVM];
  inviscid_flux<false>(c, nx, L, R, sdst, fx, &d.sc->snd2_fallbacks);
  double* fi = d.fi + (long long)DIR * npv * n;
  for (int v = 0; v < npv; ++v) fi[v * n + g] = fx[v];
  if (c.iturb == -3) return;
  // ---- viscous flux (vsflux_laminar / vsflux_turbulent)
  const bool turb = (c.iturb == 0);
  const int ep = (DIR == 0) ? GM_EX : (DIR == 1 ? GM_TX : GM_CX);   // faces normal to t1
  const int tp = (DIR == 0) ? GM_TX : (DIR == 1 ? GM_CX : GM_EX);   // faces normal to t2
  double ev[3], tvv[3];
  for (int q = 0; q < 3; ++q) {
    const double* P = d.gm + (ep + q) * n;
    ev[q] = 0.25 * (P[g - s1] + P[g - s1 + sn] + P[g] + P[g + sn]);
    const double* T = d.gm + (tp + q) * n;
    tvv[q] = 0.25 * (T[g - s2] + T[g - s2 + sn] + T[g] + T[g + sn]);
  }
  double vol = 2.0 / (d.gm[GM_GRD * n + g] + d.gm[GM_GRD * n + gr]);
  double tvl[3] = {0, 0, 0}, tvr[3] = {0, 0, 0};
  for (int q = 0; q < c.ntv; ++q) { tvl[q] = d.tv[q * n + g]; tvr[q] = d.tv[q * n + gr]; }
  double vis = 0.5 * (tvl[0] + tvr[0]);
  double con = 0.5 * (tvl[1] + tvr[1]);
  double emut = 0.0, tcon = 0.0;
  if (turb) {
    emut = 0.5 * (tvl[2] + tvr[2]);
    tcon = 0.5 * (tvl[2] * d.dv[11 * n + g] + tvr[2] * d.dv[11 * n + gr]) / 0.9;
  }
  const int vars[6] = {1, 2, 3, 4, 7, 8};
  double gx[6], gy[6], gz[6], cc[6];
  const int nv = turb ? 6 : 4;
  for (int q = 0; q < nv; ++q) {
    const double* P = d.pv + vars[q] * n;
    double x[18];
#pragma unroll
    for (int l = 0; l < 18; ++l) x[l] = P[stencil_cell(l, g, sn, s1, s2)];
    double dn = x[9] - x[8];
    double de = 0.0625 * (-x[0] - x[1] + x[4] + x[5] + 2.0 * (-x[6] - x[7] + x[10] + x[11]) - x[12] - x[13] + x[16] + x[17]);
    double dt = 0.0625 * (-x[0] - x[1] + x[12] + x[13] + 2.0 * (-x[2] - x[3] + x[14] + x[15]) - x[4] - x[5] + x[16] + x[17]);
    gx[q] = (dn * nx[0] + de * ev[0] + dt * tvv[0]) * vol;
    gy[q] = (dn * nx[1] + de * ev[1] + dt * tvv[1]) * vol;
    gz[q] = (dn * nx[2] + de * ev[2] + dt * tvv[2]) * vol;
    cc[q] = 0.5 * (x[8] + x[9]);
  }
  const double c23 = 2.0 / 3.0;
  double mu = turb ? (vis + emut) : vis;
  double div = gx[0] + gy[1] + gz[2];
  double txx = mu * (2.0 * gx[0] - c23 * div), tyy = mu * (2.0 * gy[1] - c23 * div), tzz = mu * (2.0 * gz[2] - c23 * div);
  double txy = mu * (gy[0] + gx[1]), txz = mu * (gz[0] + gx[2]), tyz = mu * (gz[1] + gy[2]);
  double kc = turb ? (con + tcon) : con;
  double uc = cc[0], vc = cc[1], wc = cc[2];
  double fv[NPVM];
  fv[0] = 0.0;
  fv[1] = txx * nx[0] + txy * nx[1] + txz * nx[2];
  fv[2] = txy * nx[0] + tyy * nx[1] + tyz * nx[2];
  fv[3] = txz * nx[0] + tyz * nx[1] + tzz * nx[2];
  fv[4] = nx[0] * (uc * txx + vc * txy + wc * txz + kc * gx[3]) + nx[1] * (uc * txy + vc * tyy + wc * tyz + kc * gy[3]) +
          nx[2] * (uc * txz + vc * tyz + wc * tzz + kc * gz[3]);
  fv[5] = 0.0;
  fv[6] = 0.0;
  if (turb) {
    double pkw = gx[4] * gx[5] + gy[4] * gy[5] + gz[4] * gz[5];
    double rho = 0.5 * (d.dv[g] + d.dv[gr]);
    double ydns = 0.5 * (d.gm[(GM_GRD + 4) * n + g] + d.gm[(GM_GRD + 4) * n + gr]);
    double kf = cc[4], of = cc[5];
    double cdkw = fmax(1.712 * rho / of * pkw, 1.0e-10);
    double term1 = sqrt(kf) / (0.09 * of * ydns);
    double term2 = 500.0 * vis / rho / (of * ydns * ydns);
    double term3 = (3.424 * rho * kf) / (cdkw * ydns * ydns);
    double arg1 = fmin(fmax(term1, term2), term3);
    double a2 = arg1 * arg1;
    double bigf = tanh(a2 * a2);
    double tdk = bigf * 0.85 + (1.0 - bigf) * 1.0;
    double tdo = bigf * 0.5 + (1.0 - bigf) * 0.856;
    fv[7] = (vis + emut * tdk) * (gx[4] * nx[0] + gy[4] * nx[1] + gz[4] * nx[2]);
    fv[8] = (vis + emut * tdo) * (gx[5] * nx[0] + gy[5] * nx[1] + gz[5] * nx[2]);
  }
  double* fvp = d.fv + (long long)DIR * npv * n;
  for (int v = 0; v < npv; ++v) fvp[v * n + g] = fv[v];
}


void launch_face_flux(const Engine& E, cudaStream_t s) {
  const int T = 128;
  auto nb = [](long long n) { return (unsigned)((n + 127) / 128); };
  k_face_flux<0><<<nb(E.nface[0]), T, 0, s>>>(E.d, E.par);
  k_face_flux<1><<<nb(E.nface[1]), T, 0, s>>>(E.d, E.par);
  k_face_flux<2><<<nb(E.nface[2]), T, 0, s>>>(E.d, E.par);
}

}  // namespace cfd
