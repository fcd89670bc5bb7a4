// mixed.cuh -- FP32 face arithmetic of the mixed-precision form (CFD3D_MIXED).
//
// Precision map of the mixed form (the FP64 form keeps everything in FP64):
//   reconstruction, limiters, inviscid and viscous flux arithmetic, stored fluxes  FP32
//   IF97 Gibbs sums of liquid and vapour                                         df64
//   saturation pressure, mixture density / enthalpy / sound speed                FP64
//   residual accumulation, LU-SGS diagonal block and sweeps, state update         FP64
// The FP32 arithmetic runs on a gauge shadow of the state, (p - pref, u, v, w, T - tref,
// y1, y2, k, omega), so that rounding is relative to the variations, not to pref or tref.
// Stored momentum fluxes leave out the uniform pref * n * dl part of the pressure flux;
// the residual kernel adds it back in FP64 (it is a pure geometric term).  AUSM-type fluxes
// carry pref * (P+ + P- - 1), evaluated from the odd parts P -/+ 1/2 so that it keeps its
// relative accuracy at low Mach numbers.
#pragma once
#include "physics.cuh"

namespace cfd {

// FP32 face state: gauge primitive variables (p - pref, u, v, w, T - tref, y1, y2, k, omega)
struct FaceStateF { float pv[NPVM]; float rho, h, c2; };

__device__ __forceinline__ float sdst_ratio_min_f(const float* s) {
  float v = fminf(s[8] / s[9], s[9] / s[8]);
  v = fminf(v, fminf(s[10] / s[8], s[8] / s[10]));
  v = fminf(v, fminf(s[8] / s[6], s[6] / s[8]));
  v = fminf(v, fminf(s[8] / s[2], s[2] / s[8]));
  v = fminf(v, fminf(s[8] / s[14], s[14] / s[8]));
  v = fminf(v, fminf(s[9] / s[11], s[11] / s[9]));
  v = fminf(v, fminf(s[9] / s[7], s[7] / s[9]));
  v = fminf(v, fminf(s[3] / s[9], s[9] / s[3]));
  v = fminf(v, fminf(s[9] / s[15], s[15] / s[9]));
  return v;
}

// inviscid face flux in FP32 with gauge pressures (src/flux_module.f90:198-641).  rc2 is
// the sound speed of the Roe-average state (FP64 mixture EOS) and ravg that state; the
// returned momentum flux excludes the geometric pref * n * dl term
__device__ __forceinline__ void inviscid_flux_mx(const Par& c, const float* n, const FaceStateF& L, const FaceStateF& Rs,
                                                 const float* sdst_g, float rc2, const float* ravg, float* fx) {
  const int npv = c.npv;
  float dl = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  if (dl == 0.0f) {
    for (int k = 0; k < npv; ++k) fx[k] = 0.0f;
    return;
  }
  float nx = n[0] / dl, ny = n[1] / dl, nz = n[2] / dl;
  const float* pl = L.pv;
  const float* pr = Rs.pv;
  float uull = nx * pl[1] + ny * pl[2] + nz * pl[3];
  float uurr = nx * pr[1] + ny * pr[2] + nz * pr[3];
  float srl = sqrtf(L.rho), srr = sqrtf(Rs.rho);
  float ravg_d = 1.0f / (srl + srr);
  float hl = L.h + 0.5f * (pl[1] * pl[1] + pl[2] * pl[2] + pl[3] * pl[3]);
  float hr = Rs.h + 0.5f * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]);
  float rrho = sqrtf(L.rho * Rs.rho);
  const float nn[3] = {nx, ny, nz};
  if (c.nscheme == 1 || c.nscheme == 2) {
    float ravg_ht = (srl * hl + srr * hr) * ravg_d;
    float u2 = ravg[1] * ravg[1] + ravg[2] * ravg[2] + ravg[3] * ravg[3];
    float uuu = nx * ravg[1] + ny * ravg[2] + nz * ravg[3];
    if (c.nscheme == 1) {
      float sndp2 = sndp2_of<float>(c, rc2, u2);
      float q = sndp2 / rc2;
      float uup = 0.5f * (1.0f + q) * uuu;
      float ddd = 0.5f * sqrtf((1.0f - q) * (1.0f - q) * uuu * uuu + 4.0f * sndp2);
      float c_star = 0.5f * (fabsf(uup + ddd) + fabsf(uup - ddd));
      float m_star = 0.5f * (fabsf(uup + ddd) - fabsf(uup - ddd)) / ddd;
      float du = m_star * (uurr - uull) + (c_star - q * fabsf(uuu) - 0.5f * (1.0f - q) * uuu * m_star) * (pr[0] - pl[0]) / rrho / sndp2;
      float dp = m_star * (pr[0] - pl[0]) + (c_star - fabsf(uuu) + 0.5f * (1.0f - q) * uuu * m_star) * rrho * (uurr - uull);
      float au = fabsf(uuu);
      fx[0] = 0.5f * (L.rho * uull + Rs.rho * uurr - (au * (Rs.rho - L.rho) + du * rrho)) * dl;
      for (int q3 = 0; q3 < 3; ++q3) {
        float df = au * (Rs.rho * pr[1 + q3] - L.rho * pl[1 + q3]) + du * rrho * ravg[1 + q3] + dp * nn[q3];
        fx[1 + q3] = 0.5f * (L.rho * uull * pl[1 + q3] + nn[q3] * pl[0] + Rs.rho * uurr * pr[1 + q3] + nn[q3] * pr[0] - df) * dl;
      }
      float df4 = au * (Rs.rho * hr - pr[0] - L.rho * hl + pl[0]) + du * rrho * ravg_ht + dp * uuu;
      fx[4] = 0.5f * (L.rho * uull * hl + Rs.rho * uurr * hr - df4) * dl;
      for (int k = 5; k < npv; ++k) {
        float df = au * (Rs.rho * pr[k] - L.rho * pl[k]) + du * rrho * ravg[k];
        fx[k] = 0.5f * (L.rho * uull * pl[k] + Rs.rho * uurr * pr[k] - df) * dl;
      }
      return;
    }
    float am2rmid_du = sndp2_du_of<float>(c, rc2, u2) / rc2;
    float am2rmid = sndp2_of<float>(c, rc2, u2) / rc2;
    float fmid = sqrtf(am2rmid) * (2.0f - sqrtf(am2rmid));
    float fmid_du = sqrtf(am2rmid_du) * (2.0f - sqrtf(am2rmid_du));
    float amid = sqrtf(rc2);
    float b1 = fmaxf(fmaxf(0.0f, uuu + amid), uurr + amid);
    float b2 = fminf(fminf(0.0f, uuu - amid), uull - amid);
    float b1_du = fmaxf(fmaxf(0.0f, uuu + fmid_du * amid), uurr + fmid_du * amid);
    float b2_du = fminf(fminf(0.0f, uuu - fmid_du * amid), uull - fmid_du * amid);
    float m_tilde = copysignf(1.0f, uuu) * fminf(fabsf(uuu) / amid, 1.0f);
    float m_tilde_du = copysignf(1.0f, uuu) * fminf(fabsf(uuu) / (fmid_du * amid), 1.0f);
    float sd[18];
    float add0 = 0.1f * fminf(L.rho * L.c2, Rs.rho * Rs.c2);
    for (int k = 0; k < 18; ++k) sd[k] = sdst_g[k] + (float)c.pref + add0;
    float ff = 1.0f - sdst_ratio_min_f(sd);
    ff = (uuu != 0.0f) ? powf(fabsf(uuu) / amid, ff) : 1.0f;
    float gg = 1.0f - fminf(sd[8] / sd[9], sd[9] / sd[8]);
    gg = (uuu != 0.0f) ? powf(fabsf(uuu) / amid, gg) : 1.0f;
    float add = 1.0f + fabsf(m_tilde), aaa = 1.0f + fabsf(m_tilde_du);
    float dq[NPVM], fl[NPVM], fr[NPVM], bdq[NPVM];
    dq[0] = Rs.rho - L.rho;
    for (int k = 1; k <= 3; ++k) dq[k] = Rs.rho * pr[k] - L.rho * pl[k];
    dq[4] = Rs.rho * hr - L.rho * hl;
    for (int k = 5; k < npv; ++k) dq[k] = Rs.rho * pr[k] - L.rho * pl[k];
    fl[0] = L.rho * uull; fr[0] = Rs.rho * uurr;
    for (int q3 = 0; q3 < 3; ++q3) {
      fl[1 + q3] = L.rho * uull * pl[1 + q3] + nn[q3] * pl[0];
      fr[1 + q3] = Rs.rho * uurr * pr[1 + q3] + nn[q3] * pr[0];
    }
    fl[4] = L.rho * uull * hl; fr[4] = Rs.rho * uurr * hr;
    for (int k = 5; k < npv; ++k) { fl[k] = L.rho * uull * pl[k]; fr[k] = Rs.rho * uurr * pr[k]; }
    bdq[0] = dq[0] - ff * (pr[0] - pl[0]) / rc2 / fmid;
    for (int k = 1; k <= 3; ++k) bdq[k] = bdq[0] * ravg[k] + rrho * (pr[k] - pl[k]);
    bdq[4] = bdq[0] * ravg_ht + rrho * (hr - hl);
    for (int k = 5; k < npv; ++k) bdq[k] = bdq[0] * ravg[k] + rrho * (pr[k] - pl[k]);
    for (int k = 0; k < npv; ++k) fx[k] = (b1 * fl[k] - b2 * fr[k] + b1 * b2 * (dq[k] - gg * bdq[k] / add)) / (b1 - b2) * dl;
    for (int q3 = 0; q3 < 3; ++q3)
      fx[1 + q3] = fx[1 + q3] + gg * b1_du * b2_du * rrho * (uurr - uull) * nn[q3] / aaa / (b1_du - b2_du) * dl;
    return;
  }
  // AUSM family
  float amid = sqrtf(rc2);
  float zmr = uurr / amid, zml = uull / amid;
  float fmid, fmid1, am2mid;
  if (c.nscheme == 3) {
    am2mid = ravg[1] * ravg[1] + ravg[2] * ravg[2] + ravg[3] * ravg[3];
    float a1 = sndp2_du_of<float>(c, rc2, am2mid) / rc2;
    float a0 = sndp2_of<float>(c, rc2, am2mid) / rc2;
    fmid = sqrtf(a0) * (2.0f - sqrtf(a0));
    fmid1 = sqrtf(a1) * (2.0f - sqrtf(a1));
  } else {
    float un = nx * ravg[1] + ny * ravg[2] + nz * ravg[3];
    am2mid = un * un;
    float a0 = sndp2_of<float>(c, rc2, am2mid) / rc2;
    fmid = sqrtf(a0) * (2.0f - sqrtf(a0));
    fmid1 = fmid;
  }
  float alpha = 3.0f / 16.0f * (-4.0f + 5.0f * fmid1 * fmid1);
  alpha = fmaxf(fminf(alpha, 3.0f / 16.0f), -3.0f / 4.0f);
  const float beta = 0.125f;
  // split Mach numbers and pressure weights.  In FP32 the sums M+(ML) + M-(MR) and
  // P+(ML) + P-(MR) - 1 cancel (M+ ~ 3/8 + ML/2, M- ~ -3/8 + MR/2 at low Mach), so they are
  // formed from their odd parts: dpl = P+(ML) - 1/2, dpr = P-(MR) - 1/2, and for subsonic
  // ML, MR  M+ + M- = (ML + MR)/2 + (ML - MR)(ML + MR)(1/4 - 2 beta + beta (ML^2 + MR^2)).
  float zmmr, pmr, zmpl, ppl, dpl, dpr;
  const bool subl = fabsf(zml) < 1.0f, subr = fabsf(zmr) < 1.0f;
  if (!subr) {
    zmmr = 0.5f * (zmr - fabsf(zmr));
    pmr = 0.5f * (1.0f - zmr / fabsf(zmr));
    dpr = pmr - 0.5f;
  } else {
    float s2 = (zmr * zmr - 1.0f) * (zmr * zmr - 1.0f);
    zmmr = -(0.25f * (zmr - 1.0f) * (zmr - 1.0f)) - beta * s2;
    dpr = -0.25f * zmr * (3.0f - zmr * zmr) - alpha * zmr * s2;
    pmr = 0.5f + dpr;
  }
  if (!subl) {
    zmpl = 0.5f * (zml + fabsf(zml));
    ppl = 0.5f * (1.0f + zml / fabsf(zml));
    dpl = ppl - 0.5f;
  } else {
    float s2 = (zml * zml - 1.0f) * (zml * zml - 1.0f);
    zmpl = 0.25f * (zml + 1.0f) * (zml + 1.0f) + beta * s2;
    dpl = 0.25f * zml * (3.0f - zml * zml) + alpha * zml * s2;
    ppl = 0.5f + dpl;
  }
  const float zsum = (subl && subr)
      ? 0.5f * (zml + zmr) + (zml - zmr) * (zml + zmr) * ((0.25f - 2.0f * beta) + beta * (zml * zml + zmr * zmr))
      : zmpl + zmmr;
  // gauge interface pressure: P+ pl + P- pr + pref (P+ + P- - 1) - dissipation
  float pdev = (float)(c.pref * ((double)dpl + (double)dpr));
  float zmpl1, zmmr1, pmid;
  if (c.nscheme == 3) {
    float zmid = zsum;
    pmid = ppl * pl[0] + pmr * pr[0] + pdev - 2.0f * ppl * pmr * rrho * fmid1 * amid * (uurr - uull);
    float sd[18];
    float add0 = 0.1f * fminf(L.rho * L.c2, Rs.rho * Rs.c2);
    for (int k = 0; k < 18; ++k) sd[k] = sdst_g[k] + (float)c.pref + add0;
    float m1 = fminf(sd[8] / sd[9], sd[9] / sd[8]);
    float ww1 = 1.0f - m1 * m1 * m1;
    float m2 = sdst_ratio_min_f(sd);
    float ww = fmaxf(ww1, 1.0f - m2 * m2);
    float pmt = rrho * rc2;
    float wq = (1.0f - ww) / fmid;
    float pwl = ((float)((double)pl[0] + c.pref) / pmt) * wq;
    float pwr = ((float)((double)pr[0] + c.pref) / pmt) * wq;
    float dpw = ((pr[0] - pl[0]) / pmt) * wq;   // pwr - pwl from the gauge difference
    if (zmid >= 0.0f) {
      float sc = rrho / L.rho;
      pwl *= sc; pwr *= sc; dpw *= sc;
      // zmpl + zmmr ((1 - ww)(1 + pwr) - pwl), with zmpl + zmmr taken from zsum
      zmpl1 = zsum + zmmr * (dpw - ww * (1.0f + pwr));
      zmmr1 = zmmr * ww * (1.0f + pwr);
    } else {
      float sc = rrho / Rs.rho;
      pwl *= sc; pwr *= sc; dpw *= sc;
      zmpl1 = zmpl * ww * (1.0f + pwl);
      zmmr1 = zsum + zmpl * (-dpw - ww * (1.0f + pwl));
    }
  } else {
    const float kp = 0.25f;
    float zmid = zsum - kp * fmaxf(1.0f - am2mid / rc2, 0.0f) * (pr[0] - pl[0]) / rrho / rc2 / fmid;
    pmid = ppl * pl[0] + pmr * pr[0] + pdev - 2.0f * ppl * pmr * rrho * fmid * amid * (uurr - uull);
    if (zmid > 0.0f) { zmpl1 = zmid; zmmr1 = 0.0f; } else { zmmr1 = zmid; zmpl1 = 0.0f; }
  }
  float ml = zmpl1 * amid * L.rho, mr = zmmr1 * amid * Rs.rho;
  fx[0] = (ml + mr) * dl;
  fx[1] = (ml * pl[1] + mr * pr[1] + pmid * nx) * dl;
  fx[2] = (ml * pl[2] + mr * pr[2] + pmid * ny) * dl;
  fx[3] = (ml * pl[3] + mr * pr[3] + pmid * nz) * dl;
  fx[4] = (ml * hl + mr * hr) * dl;
  for (int k = 5; k < npv; ++k) fx[k] = (ml * pl[k] + mr * pr[k]) * dl;
}

}  // namespace cfd
