// flux_mixed.cu -- face fluxes of the mixed-precision form (CFD3D_MIXED).
//
// k_shadow writes the FP32 gauge shadow pvf = (p - pref, u, v, w, T - tref, y1, y2, k, omega)
// of every padded cell after the boundary program; k_face_flux_mx then reconstructs,
// evaluates and stores the face fluxes of one direction in FP32, one thread per face.  The
// face-state EOS runs through the df64 IF97 sums and an FP64 mixture; the fluxes are stored
// in fi32 / fv32 (half the bytes of the FP64 form) and accumulated in FP64 by k_rhs.
// Same faces, stencils and formulas as the FP64 form (flux.cu).
#include "engine.cuh"
#include "mixed.cuh"

namespace cfd {

__global__ void __launch_bounds__(256) k_shadow(DevPtr d, Par c) {
  const long long n = d.ncell;
  const long long total = n * c.npv;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += stride) {
    const int v = (int)(q / n);
    double x = d.pv[q];
    if (v == 4) x -= c.tref;
    d.pvf[q] = (float)x;
  }
}

template <int DIR>
__global__ void __launch_bounds__(128) k_face_flux_mx(DevPtr d, Par c) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int b = 0;
  while (b + 1 < d.nblk && t >= d.blk[b + 1].face_off[DIR]) ++b;
  const BlockGeom& B = d.blk[b];
  long long loc = t - B.face_off[DIR];
  int fi_, fj, fk;
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
  const long long gr = g + sn;
  const int fplane = (DIR == 0) ? GM_CX : (DIR == 1 ? GM_EX : GM_TX);
  float nx[3];
  for (int q = 0; q < 3; ++q) nx[q] = (float)d.gm[(fplane + q) * n + g];
  const int npv = c.npv;
  const float* P = d.pvf;
  FaceStateF L, R;
  if (c.nmuscl > 0) {
    float c9[NPVM], c10[NPVM];
    for (int v = 0; v < npv; ++v) {
      float x[38];
#pragma unroll
      for (int l = 0; l < 38; ++l) x[l] = P[v * n + stencil_cell(l, g, sn, s1, s2)];
      muscl_var<float>(c, x, L.pv[v], R.pv[v]);
      c9[v] = x[8]; c10[v] = x[9];
    }
    muscl_clip<float>(c, c9, c10, L.pv, R.pv);
    const double pl = c.pref + (double)L.pv[0], tl = c.tref + (double)L.pv[4];
    const double pr = c.pref + (double)R.pv[0], tr = c.tref + (double)R.pv[4];
    if (c.nscheme == 2 || c.nscheme == 3) {
      double dl_[NDV], dr_[NDV];
      deteos_simple<true>(c.fluid, pl, tl, L.pv[5], L.pv[6], dl_, &d.sc->snd2_fallbacks);
      deteos_simple<true>(c.fluid, pr, tr, R.pv[5], R.pv[6], dr_, &d.sc->snd2_fallbacks);
      L.rho = (float)dl_[0]; L.h = (float)dl_[1]; L.c2 = (float)dl_[5];
      R.rho = (float)dr_[0]; R.h = (float)dr_[1]; R.c2 = (float)dr_[5];
    } else {
      double rl, hl, rr, hr;
      eos_rho_h<true>(c.fluid, pl, tl, L.pv[5], L.pv[6], rl, hl);
      eos_rho_h<true>(c.fluid, pr, tr, R.pv[5], R.pv[6], rr, hr);
      L.rho = (float)rl; L.h = (float)hl; R.rho = (float)rr; R.h = (float)hr;
      L.c2 = R.c2 = 0.0f;
    }
  } else {
    for (int v = 0; v < npv; ++v) { L.pv[v] = P[v * n + g]; R.pv[v] = P[v * n + gr]; }
    L.rho = (float)d.dv[g]; L.h = (float)d.dv[n + g]; L.c2 = (float)d.dv[5 * n + g];
    R.rho = (float)d.dv[gr]; R.h = (float)d.dv[n + gr]; R.c2 = (float)d.dv[5 * n + gr];
  }
  float sdst[18];
  if (c.nscheme == 2 || c.nscheme == 3) {
#pragma unroll
    for (int l = 0; l < 18; ++l) sdst[l] = P[stencil_cell(l, g, sn, s1, s2)];
  }
  // Roe-average state; its sound speed comes from the FP64 mixture EOS
  // (src/flux_module.f90:237,319,461,588)
  float ravg[NPVM];
  {
    float srl = sqrtf(L.rho), srr = sqrtf(R.rho);
    float rd = 1.0f / (srl + srr);
    ravg[0] = 0.5f * (L.pv[0] + R.pv[0]);
    ravg[4] = 0.5f * (L.pv[4] + R.pv[4]);
    for (int q = 1; q <= 3; ++q) ravg[q] = (srl * L.pv[q] + srr * R.pv[q]) * rd;
    for (int q = 5; q < npv; ++q) ravg[q] = (srl * L.pv[q] + srr * R.pv[q]) * rd;
  }
  float rc2 = 0.0f;
  if (nx[0] != 0.0f || nx[1] != 0.0f || nx[2] != 0.0f) {
    double rdv[NDV];
    deteos_simple<true>(c.fluid, c.pref + (double)ravg[0], c.tref + (double)ravg[4], ravg[5], ravg[6], rdv,
                        &d.sc->snd2_fallbacks);
    rc2 = (float)rdv[5];
  }
  float fx[NPVM];
  inviscid_flux_mx(c, nx, L, R, sdst, rc2, ravg, fx);
  float* fo = d.fi32 + (long long)DIR * npv * n;
  for (int v = 0; v < npv; ++v) fo[v * n + g] = fx[v];
  if (c.iturb == -3) return;
  // ---- viscous flux (vsflux_laminar / vsflux_turbulent, src/vsflux_module.f90:182-425)
  const bool turb = (c.iturb == 0);
  const int ep = (DIR == 0) ? GM_EX : (DIR == 1 ? GM_TX : GM_CX);
  const int tp = (DIR == 0) ? GM_TX : (DIR == 1 ? GM_CX : GM_EX);
  float ev[3], tvv[3];
  for (int q = 0; q < 3; ++q) {
    const double* E1 = d.gm + (ep + q) * n;
    ev[q] = (float)(0.25 * (E1[g - s1] + E1[g - s1 + sn] + E1[g] + E1[g + sn]));
    const double* T1 = d.gm + (tp + q) * n;
    tvv[q] = (float)(0.25 * (T1[g - s2] + T1[g - s2 + sn] + T1[g] + T1[g + sn]));
  }
  float vol = (float)(2.0 / (d.gm[GM_GRD * n + g] + d.gm[GM_GRD * n + gr]));
  float tvl[3] = {0, 0, 0}, tvr[3] = {0, 0, 0};
  for (int q = 0; q < c.ntv; ++q) { tvl[q] = (float)d.tv[q * n + g]; tvr[q] = (float)d.tv[q * n + gr]; }
  float vis = 0.5f * (tvl[0] + tvr[0]);
  float con = 0.5f * (tvl[1] + tvr[1]);
  float emut = 0.0f, tcon = 0.0f;
  if (turb) {
    emut = 0.5f * (tvl[2] + tvr[2]);
    tcon = 0.5f * (tvl[2] * (float)d.dv[11 * n + g] + tvr[2] * (float)d.dv[11 * n + gr]) / 0.9f;
  }
  const int vars[6] = {1, 2, 3, 4, 7, 8};
  float gx[6], gy[6], gz[6], cc[6];
  const int nv = turb ? 6 : 4;
  for (int q = 0; q < nv; ++q) {
    const float* X = P + vars[q] * n;
    float x[18];
#pragma unroll
    for (int l = 0; l < 18; ++l) x[l] = X[stencil_cell(l, g, sn, s1, s2)];
    float dn = x[9] - x[8];
    float de = 0.0625f * (-x[0] - x[1] + x[4] + x[5] + 2.0f * (-x[6] - x[7] + x[10] + x[11]) - x[12] - x[13] + x[16] + x[17]);
    float dt = 0.0625f * (-x[0] - x[1] + x[12] + x[13] + 2.0f * (-x[2] - x[3] + x[14] + x[15]) - x[4] - x[5] + x[16] + x[17]);
    gx[q] = (dn * nx[0] + de * ev[0] + dt * tvv[0]) * vol;
    gy[q] = (dn * nx[1] + de * ev[1] + dt * tvv[1]) * vol;
    gz[q] = (dn * nx[2] + de * ev[2] + dt * tvv[2]) * vol;
    cc[q] = 0.5f * (x[8] + x[9]);
  }
  const float c23 = 2.0f / 3.0f;
  float mu = turb ? (vis + emut) : vis;
  float div = gx[0] + gy[1] + gz[2];
  float txx = mu * (2.0f * gx[0] - c23 * div), tyy = mu * (2.0f * gy[1] - c23 * div), tzz = mu * (2.0f * gz[2] - c23 * div);
  float txy = mu * (gy[0] + gx[1]), txz = mu * (gz[0] + gx[2]), tyz = mu * (gz[1] + gy[2]);
  float kc = turb ? (con + tcon) : con;
  float uc = cc[0], vc = cc[1], wc = cc[2];
  float fv[NPVM];
  fv[0] = 0.0f;
  fv[1] = txx * nx[0] + txy * nx[1] + txz * nx[2];
  fv[2] = txy * nx[0] + tyy * nx[1] + tyz * nx[2];
  fv[3] = txz * nx[0] + tyz * nx[1] + tzz * nx[2];
  fv[4] = nx[0] * (uc * txx + vc * txy + wc * txz + kc * gx[3]) + nx[1] * (uc * txy + vc * tyy + wc * tyz + kc * gy[3]) +
          nx[2] * (uc * txz + vc * tyz + wc * tzz + kc * gz[3]);
  fv[5] = 0.0f;
  fv[6] = 0.0f;
  if (turb) {
    float pkw = gx[4] * gx[5] + gy[4] * gy[5] + gz[4] * gz[5];
    float rho = (float)(0.5 * (d.dv[g] + d.dv[gr]));
    float ydns = (float)(0.5 * (d.gm[(GM_GRD + 4) * n + g] + d.gm[(GM_GRD + 4) * n + gr]));
    float kf = cc[4], of = cc[5];
    float cdkw = fmaxf(1.712f * rho / of * pkw, 1.0e-10f);
    float term1 = sqrtf(kf) / (0.09f * of * ydns);
    float term2 = 500.0f * vis / rho / (of * ydns * ydns);
    float term3 = (3.424f * rho * kf) / (cdkw * ydns * ydns);
    float arg1 = fminf(fmaxf(term1, term2), term3);
    float a2 = arg1 * arg1;
    float bigf = tanhf(a2 * a2);
    float tdk = bigf * 0.85f + (1.0f - bigf) * 1.0f;
    float tdo = bigf * 0.5f + (1.0f - bigf) * 0.856f;
    fv[7] = (vis + emut * tdk) * (gx[4] * nx[0] + gy[4] * nx[1] + gz[4] * nx[2]);
    fv[8] = (vis + emut * tdo) * (gx[5] * nx[0] + gy[5] * nx[1] + gz[5] * nx[2]);
  }
  float* fvo = d.fv32 + (long long)DIR * npv * n;
  for (int v = 0; v < npv; ++v) fvo[v * n + g] = fv[v];
}

void launch_face_flux_mixed(const Engine& E, cudaStream_t s) {
  const int T = 128;
  auto nb = [](long long n) { return (unsigned)((n + 127) / 128); };
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  k_shadow<<<std::max(nsm, 1) * 8, 256, 0, s>>>(E.d, E.par);
  k_face_flux_mx<0><<<nb(E.nface[0]), T, 0, s>>>(E.d, E.par);
  k_face_flux_mx<1><<<nb(E.nface[1]), T, 0, s>>>(E.d, E.par);
  k_face_flux_mx<2><<<nb(E.nface[2]), T, 0, s>>>(E.d, E.par);
}

}  // namespace cfd
