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
__global__ void __launch_bounds__(256) k_face_flux(DevPtr d, Par c) {
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
      deteos_simple<false>(c.fluid, L.pv[0] + c.pref, L.pv[4], L.pv[5], L.pv[6], dl_, &d.sc->snd2_fallbacks,
                           L.pv[5] != 0.0);
      deteos_simple<false>(c.fluid, R.pv[0] + c.pref, R.pv[4], R.pv[5], R.pv[6], dr_, &d.sc->snd2_fallbacks,
                           R.pv[5] != 0.0);
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
  if (c.rot) {
    // rothalpy_l / rothalpy_r (src/flux_module.f90:697-721): the face states' total enthalpy
    // less 0.5 |omega x r|^2 at the left and right cells' centroids; h enters the fluxes
    // only through it
    double rl[3], rr[3];
    for (int e = 0; e < 3; ++e) { rl[e] = d.gm[(GM_GRD + 1 + e) * n + g]; rr[e] = d.gm[(GM_GRD + 1 + e) * n + gr]; }
    L.h = L.h - rot_q(c, rl);
    R.h = R.h - rot_q(c, rr);
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
  const bool turb = (c.iturb >= -1);
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
    face_gradient<double>(x, nx, ev, tvv, vol, gx[q], gy[q], gz[q], cc[q]);
  }
  double rho = 0.0, ydns = 0.0;
  if (turb) {
    rho = 0.5 * (d.dv[g] + d.dv[gr]);
    ydns = 0.5 * (d.gm[(GM_GRD + 4) * n + g] + d.gm[(GM_GRD + 4) * n + gr]);
  }
  double fv[NPVM];
  vsflux_core<double>(c, nx, gx, gy, gz, cc, vis, con, emut, tcon, rho, ydns, fv);
  double* fvp = d.fv + (long long)DIR * npv * n;
  for (int v = 0; v < npv; ++v) fvp[v * n + g] = fv[v];
}


void launch_face_flux(const Engine& E, cudaStream_t s) {
  const int T = E.tpb_face;
  auto nb = [T](long long n) { return (unsigned)((n + T - 1) / T); };
  k_face_flux<0><<<nb(E.nface[0]), T, 0, s>>>(E.d, E.par);
  k_face_flux<1><<<nb(E.nface[1]), T, 0, s>>>(E.d, E.par);
  k_face_flux<2><<<nb(E.nface[2]), T, 0, s>>>(E.d, E.par);
}

}  // namespace cfd
