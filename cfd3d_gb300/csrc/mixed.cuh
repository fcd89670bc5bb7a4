// mixed.cuh -- device functions of the mixed-precision form (CFD3D_MIXED).
//
// Precision map of the mixed form (the FP64 form keeps everything in FP64):
//   reconstruction and limiters                                         FP32
//   flux dissipation, split Mach / pressure corrections, viscous fluxes  FP32
//   Roe-average sound speed (IF97 + mixture)                             FP32
//   face-state density and enthalpy: IF97 Gibbs sums                     df64
//                                    saturation test, mixture            FP64
//   leading-order (central / upwind-transport) flux terms                FP64
//   residual accumulation, LU-SGS operator, state update and its EOS     FP64 (IF97 in df64)
//
// Three devices keep FP32 rounding relative to the flow's variations rather than to its
// absolute level:
//  * the state is reconstructed from a gauge shadow pvf = (p - pref, u - U, v - V, w - W,
//    T - tref, y1, y2, k, omega), U = (U, V, W) the free-stream velocity;
//  * face densities and enthalpies travel as rho - rho_ref, h - h_ref and their jumps are
//    formed from the FP64 values;
//  * a face stores F - Phi.n dl, its flux minus the flux of the uniform free stream through
//    the same face.  Every scheme returns Phi.n dl for a uniform state, and Phi.n is linear
//    in n, so the residual adds - Phi . sum(n dl) back in FP64 (zero up to the metrics'
//    closure error).
#pragma once
#include "physics.cuh"

namespace cfd {

// ------------------------------------------------------------------ FP32 sound speed
// Mixture sound speed at (p, T, y1, y2) with every step in FP32: the Roe-average state's
// c^2, which only scales dissipation and Mach splitting (src/flux_module.f90:237,319,461,588).
__device__ __forceinline__ float eos_c2_f(int fluid, float p, float t, float y1, float y2, unsigned long long* fb) {
  Phase<float> l, v, g;
  if (fluid == 1) {
    stiffened<float>(p, t, l);
    ideal_gas<float>(p, t, v);
  } else {
    iapws_l<float, true>(p, t, l);
    // without vapour every vapour term below carries the factor y1 = 0: skip its sums
    if (y1 != 0.0f) iapws_v_meta<float, true>(p, t, p > h2o_pww<float>(t), v);
    else { v.rho = 1.0f; v.h = 0.0f; v.drdp = 0.0f; v.drdt = 0.0f; v.dhdp = 0.0f; v.dhdt = 1.0f; }
  }
  ideal_gas<float>(p, t, g);
  float yl = 1.0f - y1 - y2;
  float il = 1.0f / l.rho, iv = 1.0f / v.rho, ig = 1.0f / g.rho;
  float rho = 1.0f / (yl * il + y1 * iv + y2 * ig);
  float r2 = rho * rho;
  float d6 = r2 * (yl * il * il * l.drdp + y1 * iv * iv * v.drdp + y2 * ig * ig * g.drdp);
  float d7 = r2 * (yl * il * il * l.drdt + y1 * iv * iv * v.drdt + y2 * ig * ig * g.drdt);
  float d10 = yl * l.dhdp + y1 * v.dhdp + y2 * g.dhdp;
  float d11 = yl * l.dhdt + y1 * v.dhdt + y2 * g.dhdt;
  float c2 = rho * d11 / (rho * d6 * d11 + d7 * (1.0f - rho * d10));
  if (c2 <= 0.0f) {  // the reference's "alternative calculation for snd2"
    if (fb) atomicAdd(fb, 1ull);
    float cl = (l.rho * l.drdp * l.dhdt + l.drdt * (1.0f - l.rho * l.dhdp)) / (l.rho * l.dhdt);
    float cv = (v.rho * v.drdp * v.dhdt + v.drdt * (1.0f - v.rho * v.dhdp)) / (v.rho * v.dhdt);
    float cg = (g.rho * g.drdp * g.dhdt + g.drdt * (1.0f - g.rho * g.dhdp)) / (g.rho * g.dhdt);
    c2 = 1.0f / (r2 * (yl * cl * il * il + y1 * cv * iv * iv + y2 * cg * ig * ig));
  }
  return c2;
}

// ------------------------------------------------------------------ SST source
// sst_source (physics.cuh) in FP32, for the mixed form: its terms are a part of the k and
// omega residuals and of their implicit coefficients, which an FP32 evaluation gives to
// about 1e-6 relative.  Same formulas and order.
__device__ __forceinline__ SstOut<float> sst_source_f(const float (*gr)[3], float kk, float oo, float rho, float mu,
                                                      float mut, float y5, float vol, int ides = 0,
                                                      double hmax = 0.0) {
  const float c23 = 2.0f / 3.0f, c59 = 5.0f / 9.0f;
  SstOut<float> o;
  float dudx = gr[0][0], dudy = gr[0][1], dudz = gr[0][2];
  float dvdx = gr[1][0], dvdy = gr[1][1], dvdz = gr[1][2];
  float dwdx = gr[2][0], dwdy = gr[2][1], dwdz = gr[2][2];
  o.strain = 2.0f * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + sq(dudy + dvdx) + sq(dudz + dwdx) + sq(dvdz + dwdy);
  o.div = dudx + dvdy + dwdz;
  float prod = mut * (o.strain - c23 * o.div * o.div) - c23 * rho * kk * o.div;
  o.prod = fminf(prod, 0.9f * rho * kk * oo);
  o.pkw = gr[3][0] * gr[4][0] + gr[3][1] * gr[4][1] + gr[3][2] * gr[4][2];
  float cdkw = fmaxf(1.712f * rho / oo * o.pkw, 1.0e-10f);
  float term1 = sqrtf(kk) / (0.09f * oo * y5);
  float term2 = 500.0f * mu / rho / (oo * y5 * y5);
  float term3 = (3.424f * rho * kk) / (cdkw * y5 * y5);
  float arg1 = fminf(fmaxf(term1, term2), term3);
  float a2 = arg1 * arg1;
  o.bigf = tanhf(a2 * a2);
  o.talpha = o.bigf * c59 + (1.0f - o.bigf) * 0.44f;
  o.tbeta = o.bigf * 0.075f + (1.0f - o.bigf) * 0.0828f;
  float tl = sqrtf(kk) / 9.0f / oo * 100.0f;
  if (ides != 0) {
    const float vort = sq(dudy - dvdx) + sq(dudz - dwdx) + sq(dvdz - dwdy);
    tl = sst_length_f(ides, kk, oo, o.bigf, o.strain, vort, hmax, (double)y5, mu, mut);
  }
  o.dest = rho * kk * sqrtf(kk) / tl;
  o.r7 = (o.prod - o.dest) * vol;
  o.r8 = (o.talpha * rho * (1.0f / mut) * o.prod - o.tbeta * rho * oo * oo + 1.712f * (1.0f - o.bigf) * rho * (1.0f / oo) * o.pkw) * vol;
  return o;
}

// ------------------------------------------------------------------ reconstruction clips
// muscl_clip for the FP32 reconstruction.  Where the MLP factor is exactly 2 the
// reconstructed y1 (or y2) equals a neighbour's value, typically exactly 0 at the edge of a
// vapour region; FP64 evaluates it to 0 while FP32 rounds to +-1e-9 |y|.  A value that is
// negative only by that rounding is taken as the bound itself (0), so the mixed form makes
// the same clip decision as the FP64 form instead of resetting the state to the cell value.
__device__ __forceinline__ float clip_lo0(float x, float cell) {
  const float tol = 1.0e-5f * fabsf(cell);
  return (x < 0.0f && x >= -tol) ? 0.0f : x;
}
__device__ __forceinline__ void muscl_clip_mx(const Par& c, const float* c9, const float* c10, float* xl, float* xr) {
  for (int k = 5; k <= 6; ++k) { xl[k] = clip_lo0(xl[k], c9[k]); xr[k] = clip_lo0(xr[k], c10[k]); }
  muscl_clip<float>(c, c9, c10, xl, xr);
}

// ------------------------------------------------------------------ face states
// A reconstructed face state as the flux kernel sees it: gauge primitives in FP32 and the
// FP64 quantities the leading-order flux terms need.
struct FaceMx {
  float g[NPVM];      // gauge primitives (p', u', v', w', T', y1, y2, k, omega)
  df64 rho, h;        // mixture density and static enthalpy (df64, ~1e-14)
  df64 u[3];          // full velocity (df64: U + u', exact)
  float c2;           // face sound speed (Roe-M and AUSMPW+ pressure sensor only)
};

__device__ __forceinline__ float tof(df64 a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ df64 dfp(const float* p2) { return df64(p2[0], p2[1]); }
__device__ __forceinline__ df64 dff(float a) { return df64(a, 0.0f); }

// per-face record written by the reconstruction kernel: for each side
// g[0..npv-1], rho - rho_ref, h - h_ref, c2
constexpr int FREC_SIDE = NPVM + 3;

// ------------------------------------------------------------------ inviscid flux
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

// Inviscid face flux of the mixed form (src/flux_module.f90:198-641), returned as
// F - Phi.nv (FP64 values to be stored in FP32).  nv is the unnormalised face vector,
// sdst the gauge pressures of the 18 stencil cells (schemes 2 and 3), rc2 the FP32
// sound speed of the Roe-average state, ravg_u its full velocity and ravg_s its
// primitives (scalars k >= 5 used).
__device__ __forceinline__ void inviscid_flux_mx(const Par& c, const df64* nv, const FaceMx& L, const FaceMx& R,
                                                 const float* sdst, float rc2, const float* ravg_u,
                                                 const float* ravg_s, float* fx) {
  const int npv = c.npv;
  // The leading-order terms are df64 (float-float on the FP32 pipes, ~1e-14) on the
  // unnormalised face vector nv (|nv| = dl): the normal velocities unl = nv . u are the
  // fluxes' transport velocities times dl, so no square root or division is needed; the
  // FP32 terms use the unit normal and are scaled by the FP32 length dlf.  The result is
  // the face flux minus the free-stream flux Phi . nv, rounded once to FP32.
  const float nvf[3] = {nv[0].hi, nv[1].hi, nv[2].hi};
  const float dlf = sqrtf(nvf[0] * nvf[0] + nvf[1] * nvf[1] + nvf[2] * nvf[2]);
  if (dlf == 0.0f) {
#pragma unroll
    for (int k = 0; k < NPVM; ++k) if (k < npv) fx[k] = 0.0f;
    return;
  }
  df64 fd[NPVM];
  const float idlf = 1.0f / dlf;
  const float nf[3] = {nvf[0] * idlf, nvf[1] * idlf, nvf[2] * idlf};
  const float* pl = L.g;
  const float* pr = R.g;
  // df64 leading-order quantities
  const df64 unl = nv[0] * L.u[0] + nv[1] * L.u[1] + nv[2] * L.u[2];
  const df64 unr = nv[0] * R.u[0] + nv[1] * R.u[1] + nv[2] * R.u[2];
  const df64 half(0.5f, 0.0f);
  const df64 HL = L.h + half * (L.u[0] * L.u[0] + L.u[1] * L.u[1] + L.u[2] * L.u[2]);
  const df64 HR = R.h + half * (R.u[0] * R.u[0] + R.u[1] * R.u[1] + R.u[2] * R.u[2]);
  // FP32 copies (unit-normal velocities) and accurate jumps
  const float uull = tof(unl) * idlf, uurr = tof(unr) * idlf;
  const float rl = tof(L.rho), rr = tof(R.rho);
  const float drho = tof(R.rho - L.rho);
  const float dH = tof(HR - HL);
  const float dun = tof(unr - unl) * idlf;
  const float ulf[3] = {tof(L.u[0]), tof(L.u[1]), tof(L.u[2])};
  const float hlf = tof(HL);
  float du3[3];
  for (int q = 0; q < 3; ++q) du3[q] = pr[1 + q] - pl[1 + q];   // gauge differences are the velocity jumps
  const float dp = pr[0] - pl[0];
  const float rrho = sqrtf(rl * rr);
  // free-stream flux through the face, Phi . nv = (m . nv) s, subtracted from every
  // scheme's result (m = rho_ref U, s = (1, U, H_ref, y_ref, k_ref, omega_ref))
  const df64 mn = dfp(c.m2[0]) * nv[0] + dfp(c.m2[1]) * nv[1] + dfp(c.m2[2]) * nv[2];

  if (c.nscheme == 1 || c.nscheme == 2) {
    const float u2 = ravg_u[0] * ravg_u[0] + ravg_u[1] * ravg_u[1] + ravg_u[2] * ravg_u[2];
    const float uuu = nf[0] * ravg_u[0] + nf[1] * ravg_u[1] + nf[2] * ravg_u[2];
    const float srl = sqrtf(rl), srr = sqrtf(rr);
    const float ravg_ht = (srl * tof(HL) + srr * tof(HR)) / (srl + srr);
    if (c.nscheme == 1) {
      // Roe: central part in FP64, dissipation in FP32
      float sndp2 = sndp2_of<float>(c, rc2, u2);
      float q = sndp2 / rc2;
      float uup = 0.5f * (1.0f + q) * uuu;
      float ddd = 0.5f * sqrtf((1.0f - q) * (1.0f - q) * uuu * uuu + 4.0f * sndp2);
      float c_star = 0.5f * (fabsf(uup + ddd) + fabsf(uup - ddd));
      float m_star = 0.5f * (fabsf(uup + ddd) - fabsf(uup - ddd)) / ddd;
      float du = m_star * dun + (c_star - q * fabsf(uuu) - 0.5f * (1.0f - q) * uuu * m_star) * dp / rrho / sndp2;
      float dpp = m_star * dp + (c_star - fabsf(uuu) + 0.5f * (1.0f - q) * uuu * m_star) * rrho * dun;
      float au = fabsf(uuu);
      // mass fluxes times dl
      const df64 mL = L.rho * unl, mR = R.rho * unr;
      fd[0] = half * (mL + mR - dff(dlf * (au * drho + du * rrho)));
      for (int q3 = 0; q3 < 3; ++q3) {
        // rho_R u_R - rho_L u_L = rho_R (u_R - u_L) + (rho_R - rho_L) u_L
        float df = au * (rr * du3[q3] + drho * ulf[q3]) + du * rrho * ravg_u[q3] + dpp * nf[q3];
        fd[1 + q3] = half * (mL * L.u[q3] + mR * R.u[q3] + nv[q3] * (dff(pl[0]) + dff(pr[0])) - dff(dlf * df));
      }
      float df4 = au * (rr * dH + drho * hlf - dp) + du * rrho * ravg_ht + dpp * uuu;
      fd[4] = half * (mL * HL + mR * HR - dff(dlf * df4));
#pragma unroll
      for (int k = 5; k < NPVM; ++k) if (k < npv) {
        float df = au * (rr * (pr[k] - pl[k]) + drho * pl[k]) + du * rrho * ravg_s[k];
        fd[k] = half * (mL * dff(pl[k]) + mR * dff(pr[k]) - dff(dlf * df));
      }
#pragma unroll
      for (int k = 0; k < NPVM; ++k) if (k < npv) fx[k] = tof(fd[k] - mn * dfp(c.sc2[k]));
      return;
    }
    // Roe-M
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
    float add0 = 0.1f * fminf(rl * L.c2, rr * R.c2);
    for (int k = 0; k < 18; ++k) sd[k] = sdst[k] + (float)c.pref + add0;
    float ff = 1.0f - sdst_ratio_min_f(sd);
    ff = (uuu != 0.0f) ? powf(fabsf(uuu) / amid, ff) : 1.0f;
    float gg = 1.0f - fminf(sd[8] / sd[9], sd[9] / sd[8]);
    gg = (uuu != 0.0f) ? powf(fabsf(uuu) / amid, gg) : 1.0f;
    float add = 1.0f + fabsf(m_tilde), aaa = 1.0f + fabsf(m_tilde_du);
    // jumps of the conservative variables, and of (1, u, H, y..) for bdq
    float dq[NPVM], bdq[NPVM];
    dq[0] = drho;
    for (int k = 1; k <= 3; ++k) dq[k] = rr * du3[k - 1] + drho * ulf[k - 1];
    dq[4] = rr * dH + drho * hlf;
#pragma unroll
    for (int k = 5; k < NPVM; ++k) if (k < npv) dq[k] = rr * (pr[k] - pl[k]) + drho * pl[k];
    bdq[0] = dq[0] - ff * dp / rc2 / fmid;
    for (int k = 1; k <= 3; ++k) bdq[k] = bdq[0] * ravg_u[k - 1] + rrho * du3[k - 1];
    bdq[4] = bdq[0] * ravg_ht + rrho * dH;
#pragma unroll
    for (int k = 5; k < NPVM; ++k) if (k < npv) bdq[k] = bdq[0] * ravg_s[k] + rrho * (pr[k] - pl[k]);
    // central part (b1 F_L - b2 F_R) / (b1 - b2) in FP64
    // the weights b1 / (b1 - b2), b2 / (b1 - b2) in df64 from FP32 wave speeds (their
    // difference is exact in df64); fluxes times dl
    const df64 iB = dff(1.0f) / two_sum(b1, -b2);
    const df64 w1 = dff(b1) * iB, w2 = dff(b2) * iB;
    const df64 mL = L.rho * unl, mR = R.rho * unr;
    df64 fl[NPVM], fr[NPVM];
    fl[0] = mL; fr[0] = mR;
    for (int q3 = 0; q3 < 3; ++q3) {
      fl[1 + q3] = mL * L.u[q3] + nv[q3] * dff(pl[0]);
      fr[1 + q3] = mR * R.u[q3] + nv[q3] * dff(pr[0]);
    }
    fl[4] = mL * HL; fr[4] = mR * HR;
#pragma unroll
    for (int k = 5; k < NPVM; ++k) if (k < npv) { fl[k] = mL * dff(pl[k]); fr[k] = mR * dff(pr[k]); }
    const float wdiss = dlf * b1 * b2 / (b1 - b2);
#pragma unroll
    for (int k = 0; k < NPVM; ++k)
      if (k < npv) fd[k] = w1 * fl[k] - w2 * fr[k] + dff(wdiss * (dq[k] - gg * bdq[k] / add));
    for (int q3 = 0; q3 < 3; ++q3)
      fd[1 + q3] += dff(dlf * gg * b1_du * b2_du * rrho * dun * nf[q3] / aaa / (b1_du - b2_du));
#pragma unroll
    for (int k = 0; k < NPVM; ++k) if (k < npv) fx[k] = tof(fd[k] - mn * dfp(c.sc2[k]));
    return;
  }
  // AUSM family: the interface velocity amid * M_1/2 = (u_L + u_R)/2 + small terms is
  // assembled in FP64 from its leading part and FP32 corrections
  const float amid = sqrtf(rc2);
  const float zmr = uurr / amid, zml = uull / amid;
  float fmid, fmid1, am2mid;
  if (c.nscheme == 3) {
    am2mid = ravg_u[0] * ravg_u[0] + ravg_u[1] * ravg_u[1] + ravg_u[2] * ravg_u[2];
    float a1 = sndp2_du_of<float>(c, rc2, am2mid) / rc2;
    float a0 = sndp2_of<float>(c, rc2, am2mid) / rc2;
    fmid = sqrtf(a0) * (2.0f - sqrtf(a0));
    fmid1 = sqrtf(a1) * (2.0f - sqrtf(a1));
  } else {
    float un = nf[0] * ravg_u[0] + nf[1] * ravg_u[1] + nf[2] * ravg_u[2];
    am2mid = un * un;
    float a0 = sndp2_of<float>(c, rc2, am2mid) / rc2;
    fmid = sqrtf(a0) * (2.0f - sqrtf(a0));
    fmid1 = fmid;
  }
  float alpha = 3.0f / 16.0f * (-4.0f + 5.0f * fmid1 * fmid1);
  alpha = fmaxf(fminf(alpha, 3.0f / 16.0f), -3.0f / 4.0f);
  const float beta = 0.125f;
  // split Mach numbers M+(ML), M-(MR) and pressure weights; dpl = P+(ML) - 1/2,
  // dpr = P-(MR) - 1/2 (the odd parts, no cancellation at low Mach)
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
  // amid * (M+ + M-) = (u_L + u_R)/2 + amid * E for subsonic ML, MR, with
  // E = (ML - MR)(ML + MR)(1/4 - 2 beta + beta (ML^2 + MR^2))
  // (times dl: vsum is the interface velocity times the face length)
  df64 vsum;
  if (subl && subr)
    vsum = half * (unl + unr) + dff(dlf * amid * ((zml - zmr) * (zml + zmr) * ((0.25f - 2.0f * beta) + beta * (zml * zml + zmr * zmr))));
  else
    vsum = dff(dlf * amid * (zmpl + zmmr));
  // gauge interface pressure: P+ p'L + P- p'R + pref (P+ + P- - 1) - dissipation
  const float pdev = (float)(c.pref * ((double)dpl + (double)dpr));
  df64 ml, mr;
  float pmid;
  if (c.nscheme == 3) {
    pmid = ppl * pl[0] + pmr * pr[0] + pdev - 2.0f * ppl * pmr * rrho * fmid1 * amid * dun;
    float sd[18];
    float add0 = 0.1f * fminf(rl * L.c2, rr * R.c2);
    for (int k = 0; k < 18; ++k) sd[k] = sdst[k] + (float)c.pref + add0;
    float m1 = fminf(sd[8] / sd[9], sd[9] / sd[8]);
    float ww1 = 1.0f - m1 * m1 * m1;
    float m2 = sdst_ratio_min_f(sd);
    float ww = fmaxf(ww1, 1.0f - m2 * m2);
    float pmt = rrho * rc2;
    float wq = (1.0f - ww) / fmid;
    float pwl = ((float)((double)pl[0] + c.pref) / pmt) * wq;
    float pwr = ((float)((double)pr[0] + c.pref) / pmt) * wq;
    float dpw = (dp / pmt) * wq;   // pwr - pwl from the gauge difference
    if (vsum.hi >= 0.0f) {
      // both weights scaled by the left density, as the reference does
      float sc = rrho / rl;
      pwl *= sc; pwr *= sc; dpw *= sc;
      // M+_1 = (M+ + M-) + M- ((pwr - pwl) - ww (1 + pwr)), M-_1 = M- ww (1 + pwr)
      ml = L.rho * (vsum + dff(dlf * amid * zmmr * (dpw - ww * (1.0f + pwr))));
      mr = R.rho * dff(dlf * amid * zmmr * ww * (1.0f + pwr));
    } else {
      float sc = rrho / rr;
      pwl *= sc; pwr *= sc; dpw *= sc;
      ml = L.rho * dff(dlf * amid * zmpl * ww * (1.0f + pwl));
      mr = R.rho * (vsum + dff(dlf * amid * zmpl * (-dpw - ww * (1.0f + pwl))));
    }
  } else {
    const float kp = 0.25f;
    const df64 vmid = vsum - dff(dlf * amid * kp * fmaxf(1.0f - am2mid / rc2, 0.0f) * dp / rrho / rc2 / fmid);
    pmid = ppl * pl[0] + pmr * pr[0] + pdev - 2.0f * ppl * pmr * rrho * fmid * amid * dun;
    if (vmid.hi > 0.0f) { ml = L.rho * vmid; mr = dff(0.0f); } else { mr = R.rho * vmid; ml = dff(0.0f); }
  }
  // ml, mr are mass fluxes times dl; the pressure acts on the face vector itself
  fd[0] = ml + mr;
  for (int q3 = 0; q3 < 3; ++q3) fd[1 + q3] = ml * L.u[q3] + mr * R.u[q3] + dff(pmid) * nv[q3];
  fd[4] = ml * HL + mr * HR;
#pragma unroll
  for (int k = 5; k < NPVM; ++k) if (k < npv) fd[k] = ml * dff(pl[k]) + mr * dff(pr[k]);
#pragma unroll
  for (int k = 0; k < NPVM; ++k) if (k < npv) fx[k] = tof(fd[k] - mn * dfp(c.sc2[k]));
}

}  // namespace cfd
