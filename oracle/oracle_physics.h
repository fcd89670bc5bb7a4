/*
 * oracle_physics.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Pointwise physics of the CPU oracle: a line-by-line FP64 restatement of the
 * reference's EOS, reconstruction, flux, viscous, source, Jacobian and diagonal
 * operators (kwonhwi1/3dcode, the src/ Fortran files).  Nothing in the product includes this
 * file; the tests use it to verify the GPU path and bench.py's CPU baseline arm times it.
 *
 * parity unpinned: the reference is Fortran + MPI + CGNS and cannot be built in this
 * environment, and it ships no tests or golden vectors; this restatement is the
 * parity reference, validated by self-consistency properties (tests/test_oracle.py).
 *
 * Evaluation order follows the Fortran source (left-to-right products, no fused
 * multiply-add: build with -ffp-contract=off).  Integer powers with a variable
 * exponent use binary exponentiation (the order gfortran's __builtin_powi runtime
 * uses); the IF97 routines multiply by four literals that the reference writes
 * without a kind suffix, i.e. single-precision constants (src/eos_module.f90:1367,
 * 1370, 1371, 1457), reproduced here as float literals widened to double.
 */
#ifndef ORACLE_PHYSICS_H
#define ORACLE_PHYSICS_H

#include <cmath>
#include <algorithm>

namespace orc {

static inline double sq(double x) { return x * x; }
static inline double cube(double x) { return x * x * x; }
static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }
static inline double dmax3(double a, double b, double c) { return dmax(dmax(a, b), c); }
static inline double dmin3(double a, double b, double c) { return dmin(dmin(a, b), c); }
static inline double dsign(double a, double b) { return std::copysign(std::fabs(a), b); }

/* real**integer with a variable exponent: binary exponentiation, reciprocal last. */
static inline double powi(double x, int m) {
  unsigned n = m < 0 ? 0u - (unsigned)m : (unsigned)m;
  double y = (n % 2u) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2u) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

#include "oracle_iapws_tables.inc"

struct Eos2 { double rho, h, drdp, drdt, dhdp, dhdt; };
struct Prop2 { double vis, cond; };

/* ---------------- saturation curve, surface tension (src/eos_module.f90:2266-2439) */
static inline double h2o_pww(double t) {
  double tt = dmin(dmax(t, 273.15), 647.096);
  double theta = tt - 0.23855557567849 / (tt - 0.65017534844798e3);
  double a = theta * theta + 0.11670521452767e4 * theta - 0.72421316703206e6;
  double b = -(0.17073846940092e2 * (theta * theta)) + 0.12020824702470e5 * theta - 0.32325550322333e7;
  double c = 0.14915108613530e2 * (theta * theta) - 0.48232657361591e4 * theta + 0.40511340542057e6;
  double q = 2.0 * c / (-b + std::sqrt(b * b - 4.0 * a * c));
  double q2 = q * q;
  return 1.0e6 * (q2 * q2);
}
static inline double h2o_tww(double p) {
  double beta = std::pow(p / 1.0e6, 0.25);
  double e = beta * beta - 0.17073846940092e2 * beta + 0.14915108613530e2;
  double f = 0.11670521452767e4 * (beta * beta) + 0.12020824702470e5 * beta - 0.48232657361591e4;
  double g = -(0.72421316703206e6 * (beta * beta)) - 0.32325550322333e7 * beta + 0.40511340542057e6;
  double d = 2.0 * g / (-f - std::sqrt(f * f - 4.0 * e * g));
  double s = 0.65017534844798e3 + d;
  return 0.5 * (0.65017534844798e3 + d - std::sqrt(s * s - 4.0 * (-0.23855557567849 + 0.65017534844798e3 * d)));
}
static inline double h2o_sigma(double t) {
  return 0.0881130429998226 + 0.0000616475914044782 * t - 4.4860167748009e-7 * (t * t) +
         2.53682468718936e-10 * powi(t, 3) - 2.62005668908913e-13 * powi(t, 4) +
         2.97878955533757e-16 * powi(t, 5);
}

/* ---------------- ideal gas / stiffened water (src/eos_module.f90:1236-1329) */
static inline void ideal(double p, double t, Eos2& e) {
  const double r1 = 0.00348383500557;
  double tau = 1.0 / t;
  e.rho = p * r1 * tau;
  e.h = 1004.64 * t;
  e.drdp = r1 * tau;
  e.drdt = -(p * r1 * (tau * tau));
  e.dhdp = 0.0;
  e.dhdt = 1004.64;
}
static inline void ideal_prop(double t, Prop2& pr) {
  pr.vis = 1.716e-5 * std::pow(t / 273.11, 1.5) * 383.67 / (t + 110.56);
  pr.cond = 1395.333333 * pr.vis;
}
static inline void stiffened(double p, double t, Eos2& e) {
  const double r1 = 0.00037160906726;
  double tau = 1.0 / t;
  e.rho = (p + 8.5e8) * r1 * tau;
  e.h = 4186.0 * t - 917822.36;
  e.drdp = r1 * tau;
  e.drdt = -((p + 8.5e8) * r1 * (tau * tau));
  e.dhdp = 0.0;
  e.dhdt = 4186.0;
}
static inline void stiffened_prop(double t, Prop2& pr) {
  double temp = dmax(273.0, t);
  double r = 273.0 / temp;
  pr.vis = 1.788e-3 * std::exp(-1.704 - 5.306 * 273.0 / temp + 7.003 * (r * r));
  pr.cond = 4598.0 * pr.vis;
}

/* ---------------- IF97 region 1 (src/eos_module.f90:1331-1374) */
static inline void iapws97_l(double p, double t, Eos2& e) {
  double pi = p * 0.00000006049607;
  double tau = 1386.0 / t;
  double pi1 = 1.0 / (7.1 - pi);
  double tau1 = 1.0 / (tau - 1.222);
  double gt = 0, gp = 0, gpp = 0, gtt = 0, gpt = 0;
  for (int k = 0; k < 34; ++k) {
    const int I = R1_IJN[k].i, J = R1_IJN[k].j;
    double g = R1_IJN[k].n * powi(7.1 - pi, I) * powi(tau - 1.222, J);
    double g1 = (double)J * g * tau1;
    double g2 = -((double)I * g * pi1);
    double g3 = -((double)(I - 1) * g2 * pi1);
    double g4 = (double)(J - 1) * g1 * tau1;
    double g5 = (double)J * g2 * tau1;
    gt += g1; gp += g2; gpp += g3; gtt += g4; gpt += g5;
  }
  double gp1 = 1.0 / gp;
  e.rho = (double)25.841246054191803727f * tau * gp1;
  e.h = 639675.036 * gt;
  e.drdp = -(gpp * 1.5632937721834122e-6 * tau * (gp1 * gp1));
  e.drdt = -(e.rho * 7.215007215007215e-4 * tau) + (double)0.01864447767257706f * gpt * cube(tau) * (gp1 * gp1);
  e.dhdp = (double)0.03869782431941923775f * gpt;
  e.dhdt = -(461.526 * (tau * tau) * gtt);
}

/* ---------------- IF97 region 2 + metastable vapour (src/eos_module.f90:1376-1461) */
static inline void iapws97_v(double p, double t, Eos2& e) {
  double pww = h2o_pww(t);
  double pi = p * 1e-6;
  double tau = 540.0 / t;
  double pi1 = 1.0e6 / p;
  double tau1 = 1.0 / tau;
  double tau2 = 1.0 / (tau - 0.5);
  double g0t = 0, g0p = pi1, g0pp = -(pi1 * pi1), g0tt = 0, g0pt = 0;
  double grt = 0, grp = 0, grpp = 0, grtt = 0, grpt = 0;
  const bool meta = p > pww;
  const int nres = meta ? 13 : 43;
  for (int k = 0; k < nres; ++k) {
    if (k < 9) {
      int J = meta ? R2M_IDEAL_JN[k].j : R2_IDEAL_JN[k].j;
      double n = meta ? R2M_IDEAL_JN[k].n : R2_IDEAL_JN[k].n;
      double g0 = n * powi(tau, J);
      double g01 = (double)J * g0 * tau1;
      double g02 = (double)(J - 1) * g01 * tau1;
      g0t += g01; g0tt += g02;
    }
    int I = meta ? R2M_RES_IJN[k].i : R2_RES_IJN[k].i;
    int J = meta ? R2M_RES_IJN[k].j : R2_RES_IJN[k].j;
    double n = meta ? R2M_RES_IJN[k].n : R2_RES_IJN[k].n;
    double gr = n * powi(pi, I) * powi(tau - 0.5, J);
    double gr1 = (double)J * gr * tau2;
    double gr2 = (double)I * gr * pi1;
    double gr3 = (double)(I - 1) * gr2 * pi1;
    double gr4 = (double)(J - 1) * gr1 * tau2;
    double gr5 = (double)J * gr2 * tau2;
    grt += gr1; grp += gr2; grpp += gr3; grtt += gr4; grpt += gr5;
  }
  double gp1 = 1.0 / (g0p + grp);
  e.rho = 4.01245401527075799 * tau * gp1;
  e.h = 249224.04 * (g0t + grt);
  e.drdp = -((g0pp + grpp) * 4.01245401527075799e-6 * tau * (gp1 * gp1));
  e.drdt = -(e.rho * (double)0.00185185185185185185f * tau) +
           (double)0.0074304703986495518f * (g0pt + grpt) * cube(tau) * (gp1 * gp1);
  e.dhdp = 0.24922404 * (g0pt + grpt);
  e.dhdt = -(461.526 * (tau * tau) * (g0tt + grtt));
}

/* ---------------- IAPWS transport part of *_prop (src/eos_module.f90:1507-1537) */
static inline void iapws_transport(double t, double rho, Prop2& pr) {
  double tt = t * 0.00154495032985;
  double rr = dmax(1.0e-3, dmin(1332.4, rho)) * 0.00314699949333;
  double tt1 = 647.27 / t;
  double mu0 = std::sqrt(tt) / (VIS_H[0] + VIS_H[1] * tt1 + VIS_H[2] * (tt1 * tt1) + VIS_H[3] * cube(tt1));
  double mu1 = 0.0;
  for (int i = 0; i <= 5; ++i)
    for (int j = 0; j <= 6; ++j) mu1 = mu1 + VIS_HH[i][j] * powi(tt1 - 1.0, i) * powi(rr - 1.0, j);
  mu1 = std::exp(rr * mu1);
  pr.vis = 55.071e-6 * mu0 * mu1 * 1.0;
  double lam0 = std::sqrt(tt) / (CON_L[0] + CON_L[1] * tt1 + CON_L[2] * (tt1 * tt1) + CON_L[3] * cube(tt1));
  double lam1 = 0.0;
  for (int i = 0; i <= 4; ++i)
    for (int j = 0; j <= 5; ++j) lam1 = lam1 + CON_LL[i][j] * powi(tt1 - 1.0, i) * powi(rr - 1.0, j);
  lam1 = std::exp(rr * lam1);
  pr.cond = 0.4945 * (lam0 * lam1 + 0.0);
}

/* fluid selector: 1 = stiffened water + ideal vapour, 2 = IAPWS-97; gas: ideal. */
struct EosSel { int fluid, ngas; };

static inline void eos_phase_l(const EosSel& s, double p, double t, Eos2& e) {
  if (s.fluid == 1) stiffened(p, t, e); else iapws97_l(p, t, e);
}
static inline void eos_phase_v(const EosSel& s, double p, double t, Eos2& e) {
  if (s.fluid == 1) ideal(p, t, e); else iapws97_v(p, t, e);
}

/* counter of the reference's "alternative calculation for snd2" branch */
extern long g_snd2_fallbacks;

/* mixture (src/eos_module.f90:1064-1118 / 1176-1234); tv may be nullptr */
static inline void mixture(const Eos2& l, const Eos2& v, const Eos2& g, double y1, double y2, double* dv) {
  dv[2] = l.rho; dv[3] = v.rho; dv[4] = g.rho;
  double irhol = 1.0 / dv[2], irhov = 1.0 / dv[3], irhog = 1.0 / dv[4];
  double yl = 1.0 - y1 - y2;
  double irho = yl * irhol + y1 * irhov + y2 * irhog;
  dv[0] = 1.0 / irho;
  dv[1] = yl * l.h + y1 * v.h + y2 * g.h;
  double r2 = dv[0] * dv[0];
  dv[6] = r2 * (yl * (irhol * irhol) * l.drdp + y1 * (irhov * irhov) * v.drdp + y2 * (irhog * irhog) * g.drdp);
  dv[7] = r2 * (yl * (irhol * irhol) * l.drdt + y1 * (irhov * irhov) * v.drdt + y2 * (irhog * irhog) * g.drdt);
  dv[8] = r2 * (irhol - irhov);
  dv[9] = r2 * (irhol - irhog);
  dv[10] = yl * l.dhdp + y1 * v.dhdp + y2 * g.dhdp;
  dv[11] = yl * l.dhdt + y1 * v.dhdt + y2 * g.dhdt;
  dv[12] = v.h - l.h;
  dv[13] = g.h - l.h;
  dv[5] = dv[0] * dv[11] / (dv[0] * dv[6] * dv[11] + dv[7] * (1.0 - dv[0] * dv[10]));
  if (dv[5] <= 0.0) {
    ++g_snd2_fallbacks;
    double ic2l = (dv[2] * l.drdp * l.dhdt + l.drdt * (1.0 - dv[2] * l.dhdp)) / (dv[2] * l.dhdt);
    double ic2v = (dv[3] * v.drdp * v.dhdt + v.drdt * (1.0 - dv[3] * v.dhdp)) / (dv[3] * v.dhdt);
    double ic2g = (dv[4] * g.drdp * g.dhdt + g.drdt * (1.0 - dv[4] * g.dhdp)) / (dv[4] * g.dhdt);
    dv[5] = 1.0 / (r2 * (yl * ic2l * (irhol * irhol) + y1 * ic2v * (irhov * irhov) + y2 * ic2g * (irhog * irhog)));
  }
  dv[14] = v.drdp; dv[15] = v.drdt; dv[16] = l.drdp; dv[17] = l.drdt;
}

/* eos%deteos_simple: dv(18) */
static inline void deteos_simple(const EosSel& s, double p, double t, double y1, double y2, double* dv) {
  Eos2 l, v, g;
  eos_phase_l(s, p, t, l);
  eos_phase_v(s, p, t, v);
  ideal(p, t, g);
  mixture(l, v, g, y1, y2, dv);
}

/* eos%deteos: deteos_prop (with_prop) or deteosonly; writes tv(1:2) only with props */
static inline void deteos(const EosSel& s, bool with_prop, double p, double t, double y1, double y2,
                          double* dv, double* tv) {
  if (!with_prop) { deteos_simple(s, p, t, y1, y2, dv); return; }
  Eos2 l, v, g;
  Prop2 lp, vp, gp;
  eos_phase_l(s, p, t, l);
  eos_phase_v(s, p, t, v);
  ideal(p, t, g);
  if (s.fluid == 1) { stiffened_prop(t, lp); ideal_prop(t, vp); }
  else { iapws_transport(t, l.rho, lp); iapws_transport(t, v.rho, vp); }
  ideal_prop(t, gp);
  mixture(l, v, g, y1, y2, dv);
  double yl = 1.0 - y1 - y2;
  double irhol = 1.0 / dv[2], irhov = 1.0 / dv[3], irhog = 1.0 / dv[4];
  tv[0] = dv[0] * (lp.vis * yl * irhol + vp.vis * y1 * irhov + gp.vis * y2 * irhog);
  tv[1] = dv[0] * (lp.cond * yl * irhol + vp.cond * y1 * irhov + gp.cond * y2 * irhog);
}

}  // namespace orc
#endif
