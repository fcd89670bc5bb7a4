/*
 * oracle_schemes.h -- TEST INFRASTRUCTURE ONLY (CPU oracle; see oracle_physics.h).
 *
 * Restatement of the reference's reconstruction (src/muscl_module.f90), inviscid
 * fluxes (src/flux_module.f90), viscous fluxes (src/vsflux_module.f90), cavitation
 * sources (src/cav_module.f90), SST source / eddy viscosity
 * (src/turbsource_module.f90, src/eddy_module.f90), dual-time source
 * (src/unsteady_module.f90), diagonal operator (src/lhs_module.f90) and split
 * Jacobians (src/jacobian_module.f90).  Arrays are 0-based: x[l][n] is the
 * reference's x(l+1, n+1).
 */
#ifndef ORACLE_SCHEMES_H
#define ORACLE_SCHEMES_H

#include <vector>
#include "oracle_physics.h"

namespace orc {

enum { NPV_MAX = 9, NDV = 18, STENCIL = 38 };

/* derived configuration (t_config after construct + setref) */
struct Cfg {
  int npv, ntv, nqq, ngrd;
  int nsteady, iturb, ides, nscheme, nmuscl, nlim, local, prec, fluid, ngas, ncav;
  double dt_phy, cfl, c_v, c_c, pref, uref, aoa, aos, tref, y1ref, y2ref;
  double l_chord, l_character, scale, l_domain, str, pi;
  double rhoref, visref, kref, oref, emutref;
  int fix_cav_clamp;
  int timemethod;  /* 1 explicit Euler, 2 RK3, 3 LU-SGS */
  int gravity;     /* 0 none, +-1..+-3 axis, 4 history */
  std::vector<double> grav_t, grav_a;   /* the history: times, accelerations (3 per row) */
  int csf;         /* 1: the surface-tension source rhs%csf */
  int rotation;    /* 0 none, +-1..+-3: the rotating frame about +-x, +-y, +-z */
  double omega[3]; /* its angular velocity (src/config_module.f90:126-141) */
  double tp_pt, tp_tt, tp_ht;   /* total-pressure inlet: its totals and h(p_t, T_t) */
  bool with_prop;  /* t_eos_prop (iturb >= -2) vs t_eosonly (Euler) */
  EosSel eos;
};

/* The rotating frame.  The grid velocity omega x r of the boundary routines (gridvel,
   src/bc_module.f90:2496-2498 and the others), and the term that turns the total enthalpy
   into the rothalpy, 0.5 |omega x r|^2 written as rothalpy_l / rothalpy_r / the lhs's and the
   jacobian's rothalpy do (src/flux_module.f90:697-721, lhs_module.f90:573-584,
   jacobian_module.f90:486-495), r the cell centroid grd(2:4).  Zero without rotation. */
static inline void grid_vel(const Cfg& c, const double* r, double* gv) {
  gv[0] = c.omega[1] * r[2] - c.omega[2] * r[1];
  gv[1] = c.omega[2] * r[0] - c.omega[0] * r[2];
  gv[2] = c.omega[0] * r[1] - c.omega[1] * r[0];
}
static inline double rot_q(const Cfg& c, const double* r) {
  if (!c.rotation) return 0.0;
  const double* w = c.omega;
  return 0.5 * (w[0] * w[0] * (r[1] * r[1] + r[2] * r[2]) + w[1] * w[1] * (r[0] * r[0] + r[2] * r[2]) +
                w[2] * w[2] * (r[0] * r[0] + r[1] * r[1]) -
                2.0 * (w[0] * w[1] * r[0] * r[1] + w[1] * w[2] * r[1] * r[2] + w[2] * w[0] * r[2] * r[0]));
}

/* preconditioning speed (flux/lhs/jacobian/timestep/bc all share the same forms) */
static inline double sndp2_of(const Cfg& c, double snd2, double u2) {
  switch (c.prec) {
    case 0: return snd2;
    case 1: return dmin(snd2, dmax(u2, c.uref * c.uref));
    default: return dmin(snd2, dmax3(u2, c.uref * c.uref, c.str * c.str));
  }
}
/* flux%getsndp2_du: prec 2 uses the steady form (src/flux_module.f90:133-136) */
static inline double sndp2_du_of(const Cfg& c, double snd2, double u2) {
  if (c.prec == 0) return snd2;
  return dmin(snd2, dmax(u2, c.uref * c.uref));
}

/* ================= MUSCL / MLP (src/muscl_module.f90:104-413) ================= */
struct Lim { double r[2], r1[2], r2[2], alp[2]; };

static inline double limiter(int nlim, const Lim& m, int n) {
  const double r = m.r[n], alp = m.alp[n];
  double c;
  switch (nlim) {
    case 0: return 1.0;
    case 1: return dmax(0.0, dmin(1.0, r));
    case 2: return dmax3(0.0, dmin(1.0, alp * r), dmin(alp, r));
    case 3: c = (r + std::fabs(r)) / (1.0 + std::fabs(r)); return dmax(0.0, dmin3(alp, alp * r, c));
    case 4: c = (1.0 + r) / 2.0; return dmax(0.0, dmin3(alp, alp * r, c));
    case 5: c = (r * r + r) / (1.0 + r * r); return dmax3(0.0, dmin(c * r, 1.0), dmin(r, c));
    case 6: c = dmin(1.5, alp); return dmax3(0.0, dmin(c * r, 1.0), dmin(r, c));
    case 7: c = (1.0 + 2.0 * r) / 3.0; return dmax(0.0, dmin3(alp, alp * r, c));
    case 8: c = (-2.0 * m.r1[n] + 11.0 + 24.0 * r - 3.0 * m.r2[n]) / 30.0; return dmax(0.0, dmin3(alp, alp * r, c));
    case 9: return (1.0 + 2.0 * r) / 3.0;
    default: return (-2.0 * m.r1[n] + 11.0 + 24.0 * r - 3.0 * m.r2[n]) / 30.0;
  }
}

static inline double minl(const double (*x)[NPV_MAX], int k, std::initializer_list<int> ids) {
  double v = 0; bool first = true;
  for (int l : ids) { double q = x[l - 1][k]; if (first) { v = q; first = false; } else v = dmin(v, q); }
  return v;
}
static inline double maxl(const double (*x)[NPV_MAX], int k, std::initializer_list<int> ids) {
  double v = 0; bool first = true;
  for (int l : ids) { double q = x[l - 1][k]; if (first) { v = q; first = false; } else v = dmax(v, q); }
  return v;
}

static inline void muscl_postclip(const Cfg& c, const double (*x)[NPV_MAX], double* xl, double* xr) {
  xl[0] = dmax(-c.pref + 1.0e1, xl[0]);
  xr[0] = dmax(-c.pref + 1.0e1, xr[0]);
  if (xl[5] < 0.0 || xl[5] > 1.0) xl[5] = x[8][5];
  if (xr[5] < 0.0 || xr[5] > 1.0) xr[5] = x[9][5];
  if (xl[6] < 0.0 || xl[6] > 1.0) xl[6] = x[8][6];
  if (xr[6] < 0.0 || xr[6] > 1.0) xr[6] = x[9][6];
  if (xl[5] + xl[6] > 1.0) { xl[5] = x[8][5]; xl[6] = x[8][6]; }
  if (xr[5] + xr[6] > 1.0) { xr[5] = x[9][5]; xr[6] = x[9][6]; }
  if (c.npv > 7) {
    if (xl[7] < 0.0 && x[8][7] > 0.0) xl[7] = x[8][7];
    if (xr[7] < 0.0 && x[9][7] > 0.0) xr[7] = x[9][7];
    if (xl[8] < 0.0 && x[8][8] > 0.0) xl[8] = x[8][8];
    if (xr[8] < 0.0 && x[9][8] > 0.0) xr[8] = x[9][8];
  }
}

/* tvd (nmuscl = 1) and mlp (nmuscl = 2) */
static inline void muscl(const Cfg& c, const double (*x)[NPV_MAX], double* xl, double* xr) {
  const double eps = 1.0e-30, eps2 = 1.0e-3;
  for (int k = 0; k < c.npv; ++k) {
    Lim m;
    double dq = x[9][k] - x[8][k];
    double dqm = x[8][k] - x[22][k];
    double dqm1 = x[22][k] - x[36][k];
    double dqp = x[31][k] - x[9][k];
    double dqp1 = x[37][k] - x[31][k];
    double dqmm = 1.0 / (dqm + eps);
    m.r[0] = dq * dqmm; m.r1[0] = dqm1 * dqmm; m.r2[0] = dqp * dqmm;
    double dqpp = 1.0 / (dqp + eps);
    m.r[1] = dq * dqpp; m.r1[1] = dqp1 * dqpp; m.r2[1] = dqm * dqpp;
    if (c.nmuscl == 1) {
      m.alp[0] = 2.0; m.alp[1] = 2.0;
    } else {
      double rxy_l = std::fabs((x[10][k] - x[6][k]) / (x[9][k] - x[22][k] + eps));
      double rxz_l = std::fabs((x[14][k] - x[2][k]) / (x[9][k] - x[22][k] + eps));
      double rxy_r = std::fabs((x[11][k] - x[7][k]) / (x[31][k] - x[8][k] + eps));
      double rxz_r = std::fabs((x[15][k] - x[3][k]) / (x[31][k] - x[8][k] + eps));
      double qmin, qmax;
      if (rxy_l < eps2 && rxz_l < eps2) {
        qmin = minl(x, k, {1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18,19,20,21,22,23,24,25,26,27});
        qmax = maxl(x, k, {1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18,19,20,21,22,23,24,25,26,27});
      } else if (x[9][k] - x[22][k] > 0.0) {
        qmax = maxl(x, k, {1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18});
        qmin = minl(x, k, {1,11,3,13,5,15,7,17,9,19,20,21,22,23,24,25,26,27});
      } else {
        qmin = minl(x, k, {1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18});
        qmax = maxl(x, k, {1,11,3,13,5,15,7,17,9,19,20,21,22,23,24,25,26,27});
      }
      double qml = dmin(std::fabs(qmax - x[8][k]), std::fabs(qmin - x[8][k]));
      if (rxy_r < eps2 && rxz_r < eps2) {
        qmin = minl(x, k, {1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18,28,29,30,31,32,33,34,35,36});
        qmax = maxl(x, k, {1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18,28,29,30,31,32,33,34,35,36});
      } else if (x[31][k] - x[8][k] > 0.0) {
        qmax = maxl(x, k, {10,2,12,4,14,6,16,8,18,28,29,30,31,32,33,34,35,36});
        qmin = minl(x, k, {1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18});
      } else {
        qmin = minl(x, k, {10,2,12,4,14,6,16,8,18,28,29,30,31,32,33,34,35,36});
        qmax = maxl(x, k, {1,2,3,4,5,6,7,8,9,10,11,12,13,14,15,16,17,18});
      }
      double qmr = dmin(std::fabs(qmax - x[9][k]), std::fabs(qmin - x[9][k]));
      if (std::fabs(dq) <= eps) {
        m.alp[0] = 2.0 * dmax(1.0, m.r[0]) / (std::fabs(dq) + eps) / (1.0 + rxy_l + rxz_l) * qml;
        m.alp[1] = 2.0 * dmax(1.0, dqp / eps) * std::fabs(dqpp) / (1.0 + rxy_r + rxz_r) * qmr;
      } else {
        m.alp[0] = 2.0 * dmax(1.0, m.r[0]) / (std::fabs(dq) + eps) / (1.0 + rxy_l + rxz_l) * qml;
        m.alp[1] = 2.0 * dmax(1.0, 1.0 / m.r[1]) * std::fabs(dqpp) / (1.0 + rxy_r + rxz_r) * qmr;
      }
      m.alp[0] = dmax(1.0, dmin(2.0, m.alp[0]));
      m.alp[1] = dmax(1.0, dmin(2.0, m.alp[1]));
    }
    xl[k] = x[8][k] + 0.5 * limiter(c.nlim, m, 0) * dqm;
    xr[k] = x[9][k] - 0.5 * limiter(c.nlim, m, 1) * dqp;
  }
  muscl_postclip(c, x, xl, xr);
}

/* ================= inviscid fluxes (src/flux_module.f90:198-721) ================= */
struct FaceIn {
  const double* nx;              /* unnormalised face area vector */
  const double *pvl, *pvr, *dvl, *dvr;
  const double* sdst;            /* pressure of stencil cells 1..18 */
  double rotl, rotr;             /* rot_q of the left and right cells (0 without rotation) */
};

/* enthalpy_l / enthalpy_r, or rothalpy_l / rothalpy_r in a rotating frame */
static inline double enth_l(const FaceIn& f) { return f.dvl[1] + 0.5 * (sq(f.pvl[1]) + sq(f.pvl[2]) + sq(f.pvl[3])) - f.rotl; }
static inline double enth_r(const FaceIn& f) { return f.dvr[1] + 0.5 * (sq(f.pvr[1]) + sq(f.pvr[2]) + sq(f.pvr[3])) - f.rotr; }

static inline double sdst_ratio_min(const double* s) {
  /* min over the 18 pressure ratios of the AUSMPW+ / Roe-M shock sensor */
  double v = dmin(s[8] / s[9], s[9] / s[8]);
  v = dmin(v, s[10] / s[8]); v = dmin(v, s[8] / s[10]);
  v = dmin(v, s[8] / s[6]); v = dmin(v, s[6] / s[8]);
  v = dmin(v, s[8] / s[2]); v = dmin(v, s[2] / s[8]);
  v = dmin(v, s[8] / s[14]); v = dmin(v, s[14] / s[8]);
  v = dmin(v, s[9] / s[11]); v = dmin(v, s[11] / s[9]);
  v = dmin(v, s[9] / s[7]); v = dmin(v, s[7] / s[9]);
  v = dmin(v, s[3] / s[9]); v = dmin(v, s[9] / s[3]);
  v = dmin(v, s[9] / s[15]); v = dmin(v, s[15] / s[9]);
  return v;
}

/* shared Roe-average prologue; returns false for a degenerate face */
struct RoeAvg { double nx, ny, nz, dl, uull, uurr, ravg[NPV_MAX], ravg_ht, rdv[NDV]; };

static inline bool roe_avg(const Cfg& c, const FaceIn& f, RoeAvg& a, bool need_ht) {
  a.dl = std::sqrt(sq(f.nx[0]) + sq(f.nx[1]) + sq(f.nx[2]));
  if (a.dl == 0.0) return false;
  a.nx = f.nx[0] / a.dl; a.ny = f.nx[1] / a.dl; a.nz = f.nx[2] / a.dl;
  a.uull = a.nx * f.pvl[1] + a.ny * f.pvl[2] + a.nz * f.pvl[3];
  a.uurr = a.nx * f.pvr[1] + a.ny * f.pvr[2] + a.nz * f.pvr[3];
  double ravg_d = 1.0 / (std::sqrt(f.dvl[0]) + std::sqrt(f.dvr[0]));
  a.ravg[0] = 0.5 * (f.pvl[0] + f.pvr[0]);
  a.ravg[4] = 0.5 * (f.pvl[4] + f.pvr[4]);
  for (int k = 1; k <= 3; ++k) a.ravg[k] = (std::sqrt(f.dvl[0]) * f.pvl[k] + std::sqrt(f.dvr[0]) * f.pvr[k]) * ravg_d;
  for (int k = 5; k < c.npv; ++k) a.ravg[k] = (std::sqrt(f.dvl[0]) * f.pvl[k] + std::sqrt(f.dvr[0]) * f.pvr[k]) * ravg_d;
  if (need_ht) a.ravg_ht = (std::sqrt(f.dvl[0]) * enth_l(f) + std::sqrt(f.dvr[0]) * enth_r(f)) * ravg_d;
  deteos_simple(c.eos, a.ravg[0] + c.pref, a.ravg[4], a.ravg[5], a.ravg[6], a.rdv);
  return true;
}

static inline void flux_roe(const Cfg& c, const FaceIn& f, double* fx) {
  RoeAvg a;
  if (!roe_avg(c, f, a, true)) { for (int k = 0; k < c.npv; ++k) fx[k] = 0.0; return; }
  const double nx = a.nx, ny = a.ny, nz = a.nz, dl = a.dl;
  double u2 = sq(a.ravg[1]) + sq(a.ravg[2]) + sq(a.ravg[3]);
  double* rdv = a.rdv;
  rdv[0] = std::sqrt(f.dvl[0] * f.dvr[0]);
  double uuu = nx * a.ravg[1] + ny * a.ravg[2] + nz * a.ravg[3];
  double sndp2 = sndp2_of(c, rdv[5], u2);
  double uup = 0.5 * (1.0 + sndp2 / rdv[5]) * uuu;
  double ddd = 0.5 * std::sqrt(sq(1.0 - sndp2 / rdv[5]) * sq(uuu) + 4.0 * sndp2);
  double c_star = 0.5 * (std::fabs(uup + ddd) + std::fabs(uup - ddd));
  double m_star = 0.5 * (std::fabs(uup + ddd) - std::fabs(uup - ddd)) / ddd;
  double du = m_star * (a.uurr - a.uull) +
              (c_star - sndp2 / rdv[5] * std::fabs(uuu) - 0.5 * (1.0 - sndp2 / rdv[5]) * uuu * m_star) *
                  (f.pvr[0] - f.pvl[0]) / rdv[0] / sndp2;
  double dp = m_star * (f.pvr[0] - f.pvl[0]) +
              (c_star - std::fabs(uuu) + 0.5 * (1.0 - sndp2 / rdv[5]) * uuu * m_star) * rdv[0] * (a.uurr - a.uull);
  double hl = enth_l(f), hr = enth_r(f);
  double df[NPV_MAX];
  double au = std::fabs(uuu);
  df[0] = au * (f.dvr[0] - f.dvl[0]) + du * rdv[0];
  df[1] = au * (f.dvr[0] * f.pvr[1] - f.dvl[0] * f.pvl[1]) + du * rdv[0] * a.ravg[1] + dp * nx;
  df[2] = au * (f.dvr[0] * f.pvr[2] - f.dvl[0] * f.pvl[2]) + du * rdv[0] * a.ravg[2] + dp * ny;
  df[3] = au * (f.dvr[0] * f.pvr[3] - f.dvl[0] * f.pvl[3]) + du * rdv[0] * a.ravg[3] + dp * nz;
  df[4] = au * (f.dvr[0] * hr - f.pvr[0] - f.dvl[0] * hl + f.pvl[0]) + du * rdv[0] * a.ravg_ht + dp * uuu;
  for (int k = 5; k < c.npv; ++k) df[k] = au * (f.dvr[0] * f.pvr[k] - f.dvl[0] * f.pvl[k]) + du * rdv[0] * a.ravg[k];
  fx[0] = 0.5 * (f.dvl[0] * a.uull + f.dvr[0] * a.uurr - df[0]) * dl;
  fx[1] = 0.5 * (f.dvl[0] * a.uull * f.pvl[1] + nx * (f.pvl[0] + c.pref) + f.dvr[0] * a.uurr * f.pvr[1] + nx * (f.pvr[0] + c.pref) - df[1]) * dl;
  fx[2] = 0.5 * (f.dvl[0] * a.uull * f.pvl[2] + ny * (f.pvl[0] + c.pref) + f.dvr[0] * a.uurr * f.pvr[2] + ny * (f.pvr[0] + c.pref) - df[2]) * dl;
  fx[3] = 0.5 * (f.dvl[0] * a.uull * f.pvl[3] + nz * (f.pvl[0] + c.pref) + f.dvr[0] * a.uurr * f.pvr[3] + nz * (f.pvr[0] + c.pref) - df[3]) * dl;
  fx[4] = 0.5 * (f.dvl[0] * a.uull * hl + f.dvr[0] * a.uurr * hr - df[4]) * dl;
  for (int k = 5; k < c.npv; ++k) fx[k] = 0.5 * (f.dvl[0] * a.uull * f.pvl[k] + f.dvr[0] * a.uurr * f.pvr[k] - df[k]) * dl;
}

static inline void flux_roem(const Cfg& c, const FaceIn& f, double* fx) {
  RoeAvg a;
  if (!roe_avg(c, f, a, true)) { for (int k = 0; k < c.npv; ++k) fx[k] = 0.0; return; }
  const double nx = a.nx, ny = a.ny, nz = a.nz, dl = a.dl;
  double u2 = sq(a.ravg[1]) + sq(a.ravg[2]) + sq(a.ravg[3]);
  double* rdv = a.rdv;
  rdv[0] = std::sqrt(f.dvl[0] * f.dvr[0]);
  double uuu = nx * a.ravg[1] + ny * a.ravg[2] + nz * a.ravg[3];
  double am2rmid_du = sndp2_du_of(c, rdv[5], u2) / rdv[5];
  double am2rmid = sndp2_of(c, rdv[5], u2) / rdv[5];
  double fmid = std::sqrt(am2rmid) * (2.0 - std::sqrt(am2rmid));
  double fmid_du = std::sqrt(am2rmid_du) * (2.0 - std::sqrt(am2rmid_du));
  (void)fmid;
  double amid = std::sqrt(rdv[5]);
  double b1 = dmax3(0.0, uuu + amid, a.uurr + amid);
  double b2 = dmin3(0.0, uuu - amid, a.uull - amid);
  double b1_du = dmax3(0.0, uuu + fmid_du * amid, a.uurr + fmid_du * amid);
  double b2_du = dmin3(0.0, uuu - fmid_du * amid, a.uull - fmid_du * amid);
  double m_tilde = dsign(1.0, uuu) * dmin(std::fabs(uuu) / amid, 1.0);
  double m_tilde_du = dsign(1.0, uuu) * dmin(std::fabs(uuu) / (fmid_du * amid), 1.0);
  double hl = enth_l(f), hr = enth_r(f);
  double dqp[NPV_MAX], dq[NPV_MAX], fl[NPV_MAX], fr[NPV_MAX], bdq[NPV_MAX];
  for (int k = 0; k < c.npv; ++k) dqp[k] = f.pvr[k] - f.pvl[k];
  dq[0] = f.dvr[0] - f.dvl[0];
  for (int k = 1; k <= 3; ++k) dq[k] = f.dvr[0] * f.pvr[k] - f.dvl[0] * f.pvl[k];
  dq[4] = f.dvr[0] * hr - f.dvl[0] * hl;
  for (int k = 5; k < c.npv; ++k) dq[k] = f.dvr[0] * f.pvr[k] - f.dvl[0] * f.pvl[k];
  fl[0] = f.dvl[0] * a.uull;
  fl[1] = f.dvl[0] * a.uull * f.pvl[1] + nx * (f.pvl[0] + c.pref);
  fl[2] = f.dvl[0] * a.uull * f.pvl[2] + ny * (f.pvl[0] + c.pref);
  fl[3] = f.dvl[0] * a.uull * f.pvl[3] + nz * (f.pvl[0] + c.pref);
  fl[4] = f.dvl[0] * a.uull * hl;
  for (int k = 5; k < c.npv; ++k) fl[k] = f.dvl[0] * a.uull * f.pvl[k];
  fr[0] = f.dvr[0] * a.uurr;
  fr[1] = f.dvr[0] * a.uurr * f.pvr[1] + nx * (f.pvr[0] + c.pref);
  fr[2] = f.dvr[0] * a.uurr * f.pvr[2] + ny * (f.pvr[0] + c.pref);
  fr[3] = f.dvr[0] * a.uurr * f.pvr[3] + nz * (f.pvr[0] + c.pref);
  fr[4] = f.dvr[0] * a.uurr * hr;
  for (int k = 5; k < c.npv; ++k) fr[k] = f.dvr[0] * a.uurr * f.pvr[k];
  double sdst[18];
  for (int k = 0; k < 18; ++k) sdst[k] = f.sdst[k] + c.pref + 0.1 * dmin(f.dvl[0] * f.dvl[5], f.dvr[0] * f.dvr[5]);
  double ff = 1.0 - sdst_ratio_min(sdst);
  ff = (uuu != 0.0) ? std::pow(std::fabs(uuu) / amid, ff) : 1.0;
  double gg = 1.0 - dmin(sdst[8] / sdst[9], sdst[9] / sdst[8]);
  gg = (uuu != 0.0) ? std::pow(std::fabs(uuu) / amid, gg) : 1.0;
  double add = 1.0 + std::fabs(m_tilde);
  double aaa = 1.0 + std::fabs(m_tilde_du);
  double fmid2 = std::sqrt(am2rmid) * (2.0 - std::sqrt(am2rmid));
  bdq[0] = dq[0] - ff * dqp[0] / rdv[5] / fmid2;
  bdq[1] = bdq[0] * a.ravg[1] + rdv[0] * dqp[1];
  bdq[2] = bdq[0] * a.ravg[2] + rdv[0] * dqp[2];
  bdq[3] = bdq[0] * a.ravg[3] + rdv[0] * dqp[3];
  bdq[4] = bdq[0] * a.ravg_ht + rdv[0] * (hr - hl);
  for (int k = 5; k < c.npv; ++k) bdq[k] = bdq[0] * a.ravg[k] + rdv[0] * dqp[k];
  for (int k = 0; k < c.npv; ++k) fx[k] = (b1 * fl[k] - b2 * fr[k] + b1 * b2 * (dq[k] - gg * bdq[k] / add)) / (b1 - b2) * dl;
  fx[1] = fx[1] + gg * b1_du * b2_du * rdv[0] * (a.uurr - a.uull) * nx / aaa / (b1_du - b2_du) * dl;
  fx[2] = fx[2] + gg * b1_du * b2_du * rdv[0] * (a.uurr - a.uull) * ny / aaa / (b1_du - b2_du) * dl;
  fx[3] = fx[3] + gg * b1_du * b2_du * rdv[0] * (a.uurr - a.uull) * nz / aaa / (b1_du - b2_du) * dl;
}

/* AUSM split Mach / pressure polynomials, shared by AUSMPW+ and AUSM+-up */
static inline void ausm_split(double zml, double zmr, double alpha, double& zmpl, double& ppl,
                              double& zmmr, double& pmr) {
  const double beta = 0.125;
  if (std::fabs(zmr) >= 1.0) {
    zmmr = 0.5 * (zmr - std::fabs(zmr));
    pmr = 0.5 * (1.0 - zmr / std::fabs(zmr));
  } else {
    zmmr = -(0.25 * sq(zmr - 1.0)) - beta * sq(sq(zmr) - 1.0);
    pmr = 0.25 * sq(zmr - 1.0) * (2.0 + zmr) - alpha * zmr * sq(sq(zmr) - 1.0);
  }
  if (std::fabs(zml) >= 1.0) {
    zmpl = 0.5 * (zml + std::fabs(zml));
    ppl = 0.5 * (1.0 + zml / std::fabs(zml));
  } else {
    zmpl = 0.25 * sq(zml + 1.0) + beta * sq(sq(zml) - 1.0);
    ppl = 0.25 * sq(zml + 1.0) * (2.0 - zml) + alpha * zml * sq(sq(zml) - 1.0);
  }
}

static inline void ausm_out(const Cfg& c, const FaceIn& f, const RoeAvg& a, double zmpl1, double zmmr1,
                            double amid, double pmid, double* fx) {
  const double dl = a.dl;
  double hl = enth_l(f), hr = enth_r(f);
  fx[0] = (zmpl1 * amid * f.dvl[0] + zmmr1 * amid * f.dvr[0]) * dl;
  fx[1] = (zmpl1 * amid * f.dvl[0] * f.pvl[1] + zmmr1 * amid * f.dvr[0] * f.pvr[1] + pmid * a.nx) * dl;
  fx[2] = (zmpl1 * amid * f.dvl[0] * f.pvl[2] + zmmr1 * amid * f.dvr[0] * f.pvr[2] + pmid * a.ny) * dl;
  fx[3] = (zmpl1 * amid * f.dvl[0] * f.pvl[3] + zmmr1 * amid * f.dvr[0] * f.pvr[3] + pmid * a.nz) * dl;
  fx[4] = (zmpl1 * amid * f.dvl[0] * hl + zmmr1 * amid * f.dvr[0] * hr) * dl;
  for (int k = 5; k < c.npv; ++k) fx[k] = (zmpl1 * amid * f.dvl[0] * f.pvl[k] + zmmr1 * amid * f.dvr[0] * f.pvr[k]) * dl;
}

static inline void flux_ausmpwp(const Cfg& c, const FaceIn& f, double* fx) {
  RoeAvg a;
  if (!roe_avg(c, f, a, false)) { for (int k = 0; k < c.npv; ++k) fx[k] = 0.0; return; }
  double* rdv = a.rdv;
  rdv[0] = std::sqrt(f.dvl[0] * f.dvr[0]);
  double amid = std::sqrt(rdv[5]);
  double zmr = a.uurr / amid, zml = a.uull / amid;
  double am2mid = sq(a.ravg[1]) + sq(a.ravg[2]) + sq(a.ravg[3]);
  double am2rmid1 = sndp2_du_of(c, rdv[5], am2mid) / rdv[5];
  double am2rmid = sndp2_of(c, rdv[5], am2mid) / rdv[5];
  double fmid = std::sqrt(am2rmid) * (2.0 - std::sqrt(am2rmid));
  double fmid1 = std::sqrt(am2rmid1) * (2.0 - std::sqrt(am2rmid1));
  double alpha = 3.0 / 16.0 * (-4.0 + 5.0 * sq(fmid1));
  alpha = dmax(dmin(alpha, 3.0 / 16.0), -3.0 / 4.0);
  double zmpl, ppl, zmmr, pmr;
  ausm_split(zml, zmr, alpha, zmpl, ppl, zmmr, pmr);
  double zmid = zmpl + zmmr;
  const double ku = 1.0;
  double pmid = ppl * (f.pvl[0] + c.pref) + pmr * (f.pvr[0] + c.pref) - 2.0 * ku * ppl * pmr * rdv[0] * fmid1 * amid * (a.uurr - a.uull);
  double sdst[18];
  for (int k = 0; k < 18; ++k) sdst[k] = f.sdst[k] + c.pref + 0.1 * dmin(f.dvl[0] * f.dvl[5], f.dvr[0] * f.dvr[5]);
  double ww1 = 1.0 - cube(dmin(sdst[8] / sdst[9], sdst[9] / sdst[8]));
  double ww2 = 1.0 - sq(sdst_ratio_min(sdst));
  double ww = dmax(ww1, ww2);
  double pmt = rdv[0] * rdv[5];
  double pwl = ((f.pvl[0] + c.pref + rdv[0] * rdv[5]) / pmt - 1.0) * (1.0 - ww) / fmid;
  double pwr = ((f.pvr[0] + c.pref + rdv[0] * rdv[5]) / pmt - 1.0) * (1.0 - ww) / fmid;
  double zmpl1, zmmr1;
  if (zmid >= 0.0) {
    pwl = pwl * rdv[0] / f.dvl[0];
    pwr = pwr * rdv[0] / f.dvl[0];   /* the reference scales both by dvl(1) */
    zmpl1 = zmpl + zmmr * ((1.0 - ww) * (1.0 + pwr) - pwl);
    zmmr1 = zmmr * ww * (1.0 + pwr);
  } else {
    pwl = pwl * rdv[0] / f.dvr[0];
    pwr = pwr * rdv[0] / f.dvr[0];
    zmpl1 = zmpl * ww * (1.0 + pwl);
    zmmr1 = zmmr + zmpl * ((1.0 - ww) * (1.0 + pwl) - pwr);
  }
  ausm_out(c, f, a, zmpl1, zmmr1, amid, pmid, fx);
}

static inline void flux_ausmpup(const Cfg& c, const FaceIn& f, double* fx) {
  RoeAvg a;
  if (!roe_avg(c, f, a, false)) { for (int k = 0; k < c.npv; ++k) fx[k] = 0.0; return; }
  double* rdv = a.rdv;
  rdv[0] = std::sqrt(f.dvl[0] * f.dvr[0]);
  double amid = std::sqrt(rdv[5]);
  double zmr = a.uurr / amid, zml = a.uull / amid;
  double am2mid = sq(a.nx * a.ravg[1] + a.ny * a.ravg[2] + a.nz * a.ravg[3]);
  double am2rmid = sndp2_of(c, rdv[5], am2mid) / rdv[5];
  double fmid = std::sqrt(am2rmid) * (2.0 - std::sqrt(am2rmid));
  double alpha = 3.0 / 16.0 * (-4.0 + 5.0 * sq(fmid));
  alpha = dmax(dmin(alpha, 3.0 / 16.0), -3.0 / 4.0);
  double zmpl, ppl, zmmr, pmr;
  ausm_split(zml, zmr, alpha, zmpl, ppl, zmmr, pmr);
  const double kp = 0.25, ku = 1.0;
  double zmid = zmpl + zmmr - kp * dmax(1.0 - am2mid / rdv[5], 0.0) * (f.pvr[0] - f.pvl[0]) / rdv[0] / rdv[5] / fmid;
  double pmid = ppl * (f.pvl[0] + c.pref) + pmr * (f.pvr[0] + c.pref) - 2.0 * ku * ppl * pmr * rdv[0] * fmid * amid * (a.uurr - a.uull);
  double zmpl1, zmmr1;
  if (zmid > 0.0) { zmpl1 = zmid; zmmr1 = 0.0; } else { zmmr1 = zmid; zmpl1 = 0.0; }
  ausm_out(c, f, a, zmpl1, zmmr1, amid, pmid, fx);
}

static inline void calflux(const Cfg& c, const FaceIn& f, double* fx) {
  switch (c.nscheme) {
    case 1: flux_roe(c, f, fx); break;
    case 2: flux_roem(c, f, fx); break;
    case 3: flux_ausmpwp(c, f, fx); break;
    default: flux_ausmpup(c, f, fx); break;
  }
}

/* ================= viscous fluxes (src/vsflux_module.f90:182-425) ================= */
struct VsIn {
  const double *nx, *ex1, *ex2, *ex3, *ex4, *tx1, *tx2, *tx3, *tx4;
  const double *grdl, *grdr, *dvl, *dvr, *tvl, *tvr;
  const double (*pv)[NPV_MAX];   /* stencil x(1:18, :) */
};

static inline double tder_e(const double (*p)[NPV_MAX], int v) {
  return 0.0625 * (-p[0][v] - p[1][v] + p[4][v] + p[5][v] + 2.0 * (-p[6][v] - p[7][v] + p[10][v] + p[11][v]) -
                   p[12][v] - p[13][v] + p[16][v] + p[17][v]);
}
static inline double tder_t(const double (*p)[NPV_MAX], int v) {
  return 0.0625 * (-p[0][v] - p[1][v] + p[12][v] + p[13][v] + 2.0 * (-p[2][v] - p[3][v] + p[14][v] + p[15][v]) -
                   p[4][v] - p[5][v] + p[16][v] + p[17][v]);
}

static inline void vsflux(const Cfg& c, const VsIn& s, double* fx) {
  const bool turb = (c.iturb >= -1);
  double ex = 0.25 * (s.ex1[0] + s.ex2[0] + s.ex3[0] + s.ex4[0]);
  double ey = 0.25 * (s.ex1[1] + s.ex2[1] + s.ex3[1] + s.ex4[1]);
  double ez = 0.25 * (s.ex1[2] + s.ex2[2] + s.ex3[2] + s.ex4[2]);
  double tx = 0.25 * (s.tx1[0] + s.tx2[0] + s.tx3[0] + s.tx4[0]);
  double ty = 0.25 * (s.tx1[1] + s.tx2[1] + s.tx3[1] + s.tx4[1]);
  double tz = 0.25 * (s.tx1[2] + s.tx2[2] + s.tx3[2] + s.tx4[2]);
  double vol = 2.0 / (s.grdl[0] + s.grdr[0]);
  double vis = 0.5 * (s.tvl[0] + s.tvr[0]);
  double con = 0.5 * (s.tvl[1] + s.tvr[1]);
  double emut = 0, tcon = 0;
  if (turb) {
    emut = 0.5 * (s.tvl[2] + s.tvr[2]);
    tcon = 0.5 * (s.tvl[2] * s.dvl[11] + s.tvr[2] * s.dvr[11]) / 0.9;
  }
  const double (*p)[NPV_MAX] = s.pv;
  double uc = 0.5 * (p[8][1] + p[9][1]);
  double vc = 0.5 * (p[8][2] + p[9][2]);
  double wc = 0.5 * (p[8][3] + p[9][3]);
  const double* n = s.nx;
  /* gradients of u,v,w,T (and k,omega) */
  const int vars[6] = {1, 2, 3, 4, 7, 8};
  double gx[6], gy[6], gz[6];
  int nv = turb ? 6 : 4;
  for (int q = 0; q < nv; ++q) {
    int v = vars[q];
    double dn = p[9][v] - p[8][v];
    double de = tder_e(p, v);
    double dt = tder_t(p, v);
    gx[q] = (dn * n[0] + de * ex + dt * tx) * vol;
    gy[q] = (dn * n[1] + de * ey + dt * ty) * vol;
    gz[q] = (dn * n[2] + de * ez + dt * tz) * vol;
  }
  double dudx = gx[0], dvdx = gx[1], dwdx = gx[2], dtdx = gx[3];
  double dudy = gy[0], dvdy = gy[1], dwdy = gy[2], dtdy = gy[3];
  double dudz = gz[0], dvdz = gz[1], dwdz = gz[2], dtdz = gz[3];
  const double c23 = 2.0 / 3.0;
  double mu = turb ? (vis + emut) : vis;
  double tauxx = mu * (2.0 * dudx - c23 * (dudx + dvdy + dwdz));
  double tauyy = mu * (2.0 * dvdy - c23 * (dudx + dvdy + dwdz));
  double tauzz = mu * (2.0 * dwdz - c23 * (dudx + dvdy + dwdz));
  double tauxy = mu * (dudy + dvdx);
  double tauxz = mu * (dudz + dwdx);
  double tauyz = mu * (dvdz + dwdy);
  double kc = turb ? (con + tcon) : con;
  fx[0] = 0.0;
  fx[1] = tauxx * n[0] + tauxy * n[1] + tauxz * n[2];
  fx[2] = tauxy * n[0] + tauyy * n[1] + tauyz * n[2];
  fx[3] = tauxz * n[0] + tauyz * n[1] + tauzz * n[2];
  fx[4] = n[0] * (uc * tauxx + vc * tauxy + wc * tauxz + kc * dtdx) +
          n[1] * (uc * tauxy + vc * tauyy + wc * tauyz + kc * dtdy) +
          n[2] * (uc * tauxz + vc * tauyz + wc * tauzz + kc * dtdz);
  fx[5] = 0.0;
  fx[6] = 0.0;
  if (turb) {
    double dkdx = gx[4], dkdy = gy[4], dkdz = gz[4], dodx = gx[5], dody = gy[5], dodz = gz[5];
    /* SST blending F1 on the face (kwsst, src/vsflux_module.f90:400-425) */
    double pkw = dkdx * dodx + dkdy * dody + dkdz * dodz;
    double rho = 0.5 * (s.dvl[0] + s.dvr[0]);
    double ydns = 0.5 * (s.grdl[4] + s.grdr[4]);
    double visf = 0.5 * (s.tvl[0] + s.tvr[0]);
    double k = 0.5 * (p[8][7] + p[9][7]);
    double o = 0.5 * (p[8][8] + p[9][8]);
    double term0 = 1.712 * rho / o * pkw;
    double cdkw = dmax(term0, 1.0e-10);
    double term1 = std::sqrt(k) / (0.09 * o * ydns);
    double term2 = 500.0 * visf / rho / (o * sq(ydns));
    double term3 = (3.424 * rho * k) / (cdkw * sq(ydns));
    double arg2 = dmax(term1, term2);
    double arg1 = dmin(arg2, term3);
    double bigf = std::tanh(sq(sq(arg1)));
    /* tdk1, tdk2, tdo1, tdo2 of vsflux%construct (:62-90): SST 0.85, 1, 0.5, 0.856; k-epsilon
       0, 1, 0, 1/1.3 with calbigf = 0 (:427-435) */
    double tdk = bigf * 0.85 + (1.0 - bigf) * 1.0;
    double tdo = bigf * 0.5 + (1.0 - bigf) * 0.856;
    if (c.iturb == -1) { bigf = 0.0; tdk = bigf * 0.0 + (1.0 - bigf) * 1.0; tdo = bigf * 0.0 + (1.0 - bigf) * (1.0 / 1.3); }
    fx[7] = (vis + emut * tdk) * (dkdx * n[0] + dkdy * n[1] + dkdz * n[2]);
    fx[8] = (vis + emut * tdo) * (dodx * n[0] + dody * n[1] + dodz * n[2]);
  }
}

/* ================= cavitation sources (src/cav_module.f90:136-357) ================= */
struct CavOut { double r_c, r_v, icav[4]; };

static inline void cav_finish(CavOut& o) {
  const double phi = 1.0;
  double lam = dsign(1.0, o.icav[2]);
  double f = phi * (1.0 - 0.5 * (1.0 - lam)) - 0.5 * (1.0 - lam);
  for (int q = 0; q < 4; ++q) o.icav[q] = o.icav[q] * f;
}

/* pv2 = pv of the cell, dv its dv(18), vol = grd(1) */
static inline CavOut cavsource(const Cfg& c, const double* pv2, const double* dv, double vol) {
  CavOut o = {0.0, 0.0, {0.0, 0.0, 0.0, 0.0}};
  const double t_crit = 647.096;
  if (pv2[4] >= t_crit) return o;
  const double dp_ref = 2.0 / (c.rhoref * sq(c.uref));
  const double t_ref = c.uref / c.l_chord;
  const double P = pv2[0] + c.pref;
  /* the reference clamps with pv(2,5) (temperature) and pv(2,6); fix_cav_clamp uses y1, y2 */
  const double clamp_c = c.fix_cav_clamp ? pv2[5] : pv2[4];
  const double clamp_v = c.fix_cav_clamp ? (1.0 - pv2[5] - pv2[6]) : (1.0 - pv2[4] - pv2[5]);
  double r_c, r_v;
  switch (c.ncav) {
    case 1: {  /* Merkle */
      double pww = h2o_pww(pv2[4]);
      double rho1 = 1.0 / dv[0];
      r_c = c.c_c * dv[0] * pv2[5] * dmax(pv2[0] + c.pref - pww, 0.0) * dp_ref * t_ref;
      r_v = c.c_v * dv[0] * (1.0 - pv2[5] - pv2[6]) * dmax(pww - pv2[0] - c.pref, 0.0) * dp_ref * t_ref;
      r_c = dmin(r_c, dv[0] * clamp_c);
      r_v = dmin(r_v, dv[0] * clamp_v);
      o.r_c = r_c * vol; o.r_v = r_v * vol;
      if (r_c != 0.0) {
        o.icav[0] = -(r_c * dv[6] * rho1) - c.c_c * dv[0] * pv2[5] * dp_ref * t_ref;
        o.icav[1] = -(r_c * dv[7] * rho1);
        o.icav[2] = -(r_c * dv[8] * rho1) - c.c_c * dv[0] * dmax(pv2[0] + c.pref - pww, 0.0) * dp_ref * t_ref;
        o.icav[3] = -(r_c * dv[9] * rho1);
      }
      if (r_v != 0.0) {
        o.icav[0] = r_v * dv[6] * rho1 - c.c_v * dv[0] * (1.0 - pv2[5] - pv2[6]) * dp_ref * t_ref;
        o.icav[1] = r_v * dv[7] * rho1;
        o.icav[2] = r_v * dv[8] * rho1 - c.c_v * dv[0] * dmax(pww - pv2[0] - c.pref, 0.0) * dp_ref * t_ref;
        o.icav[3] = r_v * dv[9] * rho1 - c.c_v * dv[0] * dmax(pww - pv2[0] - c.pref, 0.0) * dp_ref * t_ref;
      }
      break;
    }
    case 2: {  /* Kunz */
      double pww = h2o_pww(pv2[4]);
      double rho1 = 1.0 / dv[0];
      double av = dv[0] * pv2[5] / dv[3];
      double ag = dv[0] * pv2[6] / dv[4];
      double al = 1.0 - av - ag;
      r_c = c.c_c * dv[3] * av * sq(al + ag) * t_ref;
      r_v = c.c_v * dv[0] * (1.0 - pv2[5] - pv2[6]) * dmax(pww - pv2[0] - c.pref, 0.0) * dp_ref * t_ref;
      r_c = dmin(r_c, dv[0] * clamp_c);
      r_v = dmin(r_v, dv[0] * clamp_v);
      o.r_c = r_c * vol; o.r_v = r_v * vol;
      double av1 = 1.0 - 4.0 * av + 3.0 * sq(av);
      o.icav[0] = -(c.c_c * t_ref * (dv[6] * pv2[5] * av1 + 2.0 * sq(av) * dv[14] * (al + ag)));
      o.icav[1] = -(c.c_c * t_ref * (dv[7] * pv2[5] * av1 + 2.0 * sq(av) * dv[15] * (al + ag)));
      o.icav[2] = -(c.c_c * t_ref * (dv[8] * pv2[5] + dv[0]) * av1);
      o.icav[3] = -(c.c_c * t_ref * dv[9] * pv2[5] * av1);
      if (r_v != 0.0) {
        o.icav[0] = r_v * dv[6] * rho1 - c.c_v * dv[0] * (1.0 - pv2[5] - pv2[6]) * dp_ref * t_ref;
        o.icav[1] = r_v * dv[7] * rho1;
        o.icav[2] = r_v * dv[8] * rho1 - c.c_v * dv[0] * dmax(pww - pv2[0] - c.pref, 0.0) * dp_ref * t_ref;
        o.icav[3] = r_v * dv[9] * rho1 - c.c_v * dv[0] * dmax(pww - pv2[0] - c.pref, 0.0) * dp_ref * t_ref;
      }
      break;
    }
    case 3: {  /* Singhal */
      double pww = h2o_pww(pv2[4]);
      double sigma = h2o_sigma(pv2[4]);
      double rho1 = 1.0 / dv[2], rho2 = 1.0 / dv[3];
      double cc = c.c_c * c.uref / sigma * dv[2] * dv[3];
      double cv = c.c_v * c.uref / sigma * dv[2] * dv[3];
      r_c = cc * std::sqrt(2.0 / 3.0 * dmax(P - pww, 0.0) * rho1) * pv2[5];
      r_v = cv * std::sqrt(2.0 / 3.0 * dmax(pww - pv2[0] - c.pref, 0.0) * rho1) * (1.0 - pv2[5] - pv2[6]);
      r_c = dmin(r_c, dv[0] * clamp_c);
      r_v = dmin(r_v, dv[0] * clamp_v);
      o.r_c = r_c * vol; o.r_v = r_v * vol;
      if (r_c != 0.0) {
        o.icav[0] = -(r_c * (dv[14] * rho2 + 0.5 * dv[16] * rho1)) -
                    0.5 * cc * std::sqrt(2.0 / 3.0 * rho1) * pv2[5] * std::pow(P - pww, -0.5);
        o.icav[1] = -(r_c * (dv[15] * rho2 + 0.5 * dv[17] * rho1));
        o.icav[2] = -(cc * std::sqrt(2.0 / 3.0 * dmax(P - pww, 0.0) * rho1));
        o.icav[3] = 0.0;
      }
      if (r_v != 0.0) {
        o.icav[0] = r_v * (dv[14] * rho2 + 0.5 * dv[16] * rho1) -
                    0.5 * cv * std::sqrt(2.0 / 3.0 * rho1) * (1.0 - pv2[5] - pv2[6]) * std::pow(pww - pv2[0] - c.pref, -0.5);
        o.icav[1] = r_v * (dv[15] * rho2 + 0.5 * dv[17] * rho1);
        o.icav[2] = -(cv * std::sqrt(2.0 / 3.0 * dmax(pww - pv2[0] - c.pref, 0.0) * rho1));
        o.icav[3] = -(cv * std::sqrt(2.0 / 3.0 * dmax(pww - pv2[0] - c.pref, 0.0) * rho1));
      }
      break;
    }
    case 4: {  /* Schnerr-Sauer */
      const double pi = 4.0 * std::atan(1.0), eta = 1.0e13;
      double pww = h2o_pww(pv2[4]);
      double rho1 = 1.0 / dv[0], rho3 = 1.0 / dv[2], rho4 = 1.0 / dv[3];
      double k0 = 3.0 * std::pow(4.0 * pi * eta / 3.0, 1.0 / 3.0) * std::sqrt(2.0 / 3.0);
      double yl = 1.0 - pv2[5] - pv2[6];
      r_c = c.c_c * k0 * dv[0] * std::pow(dv[3], 1.0 / 3.0) * std::pow(dv[2], -5.0 / 6.0) *
            std::pow(pv2[5], 2.0 / 3.0) * std::pow(yl, 4.0 / 3.0) * std::sqrt(dmax(P - pww, 0.0));
      r_v = c.c_v * k0 * dv[0] * std::pow(dv[3], 1.0 / 3.0) * std::pow(dv[2], -5.0 / 6.0) *
            std::pow(pv2[5] + pv2[6], 2.0 / 3.0) * std::pow(yl, 4.0 / 3.0) * std::sqrt(dmax(pww - pv2[0] - c.pref, 0.0));
      r_c = dmin(r_c, dv[0] * clamp_c);
      r_v = dmin(r_v, dv[0] * clamp_v);
      o.r_c = r_c * vol; o.r_v = r_v * vol;
      if (r_c != 0.0) {
        o.icav[0] = -(r_c * (dv[6] * rho1 + dv[14] * rho4 / 3.0 - 5.0 * dv[16] * rho3 / 6.0 + 0.5 / (P - pww)));
        o.icav[1] = -(r_c * (dv[7] * rho1 + dv[15] * rho4 / 3.0 - 5.0 * dv[17] * rho3 / 6.0));
        o.icav[2] = -(r_c * (dv[8] * rho1 + 2.0 / (3.0 * pv2[5]) - 4.0 / (3.0 * yl)));
        o.icav[3] = -(r_c * (dv[9] * rho1 - 4.0 / (3.0 * yl)));
      }
      if (r_v != 0.0) {
        o.icav[0] = r_v * (dv[6] * rho1 + dv[14] * rho4 / 3.0 - 5.0 * dv[16] * rho3 / 6.0 - 0.5 / (pww - pv2[0] - c.pref));
        o.icav[1] = r_v * (dv[7] * rho1 + dv[15] * rho4 / 3.0 - 5.0 * dv[17] * rho3 / 6.0);
        o.icav[2] = r_v * (dv[8] * rho1 + 2.0 / (3.0 * (pv2[5] + pv2[6])) - 4.0 / (3.0 * yl));
        o.icav[3] = r_v * (dv[9] * rho1 + 2.0 / (3.0 * (pv2[5] + pv2[6])) - 4.0 / (3.0 * yl));
      }
      break;
    }
    default: {  /* Lee */
      double tww = h2o_tww(pv2[0] + c.pref);
      double rho1 = 1.0 / dv[0];
      r_c = c.c_c * dv[0] * pv2[5] * dmax(tww - pv2[4], 0.0) / tww;
      r_v = c.c_v * dv[0] * (1.0 - pv2[5] - pv2[6]) * dmax(pv2[4] - tww, 0.0) / tww;
      r_c = dmin(r_c, dv[0] * clamp_c);
      r_v = dmin(r_v, dv[0] * clamp_v);
      o.r_c = r_c * vol; o.r_v = r_v * vol;
      if (r_c != 0.0) {
        o.icav[0] = -(r_c * dv[6] * rho1);
        o.icav[1] = -(r_c * dv[7] * rho1) + c.c_c * dv[0] * pv2[5] / tww;
        o.icav[2] = -(r_c * dv[8] * rho1) - c.c_c * dv[0] * dmax(tww - pv2[4], 0.0) / tww;
        o.icav[3] = -(r_c * dv[9] * rho1);
      }
      if (r_v != 0.0) {
        o.icav[0] = r_v * dv[6] * rho1;
        o.icav[1] = r_v * dv[7] * rho1 + c.c_v * dv[0] * (1.0 - pv2[5] - pv2[6]) / tww;
        o.icav[2] = r_v * dv[8] * rho1 - c.c_v * dv[0] * dmax(pv2[4] - tww, 0.0) / tww;
        o.icav[3] = r_v * dv[9] * rho1 - c.c_v * dv[0] * dmax(pv2[4] - tww, 0.0) / tww;
      }
      break;
    }
  }
  cav_finish(o);
  return o;
}

/* ================= cell-centred velocity gradients (turbsource / eddy) ================= */
struct Grad7 { double d[5][3]; };  /* u,v,w,k,o x (x,y,z) */

/* x[0..6] = pv at (i-1),(i),(i+1),(j-1),(j+1),(k-1),(k+1); faces cx1,cx2,ex1,ex2,tx1,tx2 */
static inline void cell_grad(const double (*x)[NPV_MAX], const double* cx1, const double* cx2,
                             const double* ex1, const double* ex2, const double* tx1, const double* tx2,
                             double vol_in, int var, double* g) {
  double v1 = 0.5 * (x[0][var] + x[1][var]);
  double v2 = 0.5 * (x[2][var] + x[1][var]);
  double v3 = 0.5 * (x[3][var] + x[1][var]);
  double v4 = 0.5 * (x[4][var] + x[1][var]);
  double v5 = 0.5 * (x[5][var] + x[1][var]);
  double v6 = 0.5 * (x[6][var] + x[1][var]);
  double vol = 1.0 / vol_in;
  for (int d = 0; d < 3; ++d)
    g[d] = (v2 * cx2[d] + v4 * ex2[d] + v6 * tx2[d] - v1 * cx1[d] - v3 * ex1[d] - v5 * tx1[d]) * vol;
}

struct TurbOut { double source[2], itt[4], omega_cut; };

/* x**10 as a Fortran compiler expands it (cube() is x**3) */
static inline double pow10i(double x) { const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4; return x8 * x2; }

/* calturblength: the turbulent length scale of the k destruction, by ides -- no_des, sst_des,
 * sst_ddes, sst_iddes, sst_s_iddes (src/turbsource_module.f90:406-576) */
static inline double turb_length(int ides, double k, double o, double bigf, double strain_sq, double vorticity_sq,
                                 const double* cx1, const double* cx2, const double* ex1, const double* ex2,
                                 const double* tx1, const double* tx2, const double* grd, const double* tv) {
  const double tl_rans = std::sqrt(k) / 9.0 / o * 100.0;
  if (ides == 0) return tl_rans;
  const double vol = grd[0];
  double gs[3];
  const double* f[3][2] = {{cx1, cx2}, {ex1, ex2}, {tx1, tx2}};
  for (int d = 0; d < 3; ++d)
    gs[d] = vol / (0.5 * (std::sqrt(sq(f[d][0][0]) + sq(f[d][0][1]) + sq(f[d][0][2])) +
                          std::sqrt(sq(f[d][1][0]) + sq(f[d][1][1]) + sq(f[d][1][2]))));
  const double hmax = dmax3(gs[0], gs[1], gs[2]);
  if (ides == 1) return dmin(tl_rans, 0.61 * hmax);
  const double cdes = 0.78 * bigf + 0.61 * (1.0 - bigf);
  const double den = sq(0.41) * sq(grd[4]) * std::sqrt(0.5 * (strain_sq + vorticity_sq));
  if (ides == 2) {
    const double tl_les = cdes * hmax;
    const double rd = (tv[0] + tv[2]) / den;
    const double fd = 1.0 - std::tanh(cube(20.0 * rd));
    return tl_rans - fd * dmax(0.0, tl_rans - tl_les);
  }
  const double tl_les = cdes * dmin(0.15 * dmax(grd[4], hmax), hmax);
  const double alpha = 0.25 - grd[4] / hmax;
  const double fb = dmin(2.0 * std::exp(-9.0 * sq(alpha)), 1.0);
  const double rdt = tv[2] / den;
  const double fdt = 1.0 - std::tanh(cube(20.0 * rdt));
  const double fd = dmax(1.0 - fdt, fb);
  if (ides == 4) return fd * tl_rans + (1.0 - fd) * tl_les;
  const double rdl = tv[0] / den;
  const double fl = std::tanh(pow10i(25.0 * rdl));
  const double ft = std::tanh(cube(3.4969 * rdt));
  const double fe2 = 1.0 - dmax(ft, fl);
  const double fe1 = (alpha >= 0.0) ? 2.0 * std::exp(-11.09 * sq(alpha)) : 2.0 * std::exp(-9.0 * sq(alpha));
  const double fe = fe2 * dmax(fe1 - 1.0, 0.0);
  return fd * (1.0 + fe) * tl_rans + (1.0 - fd) * tl_les;
}

/* kwsst source (src/turbsource_module.f90:269-383) with the length scale of ides */
static inline TurbOut kwsst_source(const double (*x)[NPV_MAX], const double* cx1, const double* cx2,
                                   const double* ex1, const double* ex2, const double* tx1, const double* tx2,
                                   const double* grd, const double* dv, const double* tv, int ides = 0) {
  TurbOut r;
  double gk[3], go[3], gu[3], gv[3], gw[3];
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 7, gk);
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 8, go);
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 1, gu);
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 2, gv);
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 3, gw);
  double dudx = gu[0], dudy = gu[1], dudz = gu[2];
  double dvdx = gv[0], dvdy = gv[1], dvdz = gv[2];
  double dwdx = gw[0], dwdy = gw[1], dwdz = gw[2];
  const double c23 = 2.0 / 3.0, c59 = 5.0 / 9.0, phi = 1.0;
  const double k = x[1][7], o = x[1][8];
  double strain_sq = 2.0 * (sq(dudx) + sq(dvdy) + sq(dwdz)) + sq(dudy + dvdx) + sq(dudz + dwdx) + sq(dvdz + dwdy);
  double div = dudx + dvdy + dwdz;
  double prod = tv[2] * (strain_sq - c23 * sq(div)) - c23 * dv[0] * k * div;
  prod = dmin(prod, 0.9 * dv[0] * k * o);
  r.omega_cut = std::sqrt(strain_sq - c23 * sq(div));
  double pkw = gk[0] * go[0] + gk[1] * go[1] + gk[2] * go[2];
  /* calbigf (:385-404) */
  double term0 = 1.712 * dv[0] / o * pkw;
  double cdkw = dmax(term0, 1.0e-10);
  double term1 = std::sqrt(k) / (0.09 * o * grd[4]);
  double term2 = 500.0 * tv[0] / dv[0] / (o * sq(grd[4]));
  double term3 = (3.424 * dv[0] * k) / (cdkw * sq(grd[4]));
  double bigf = std::tanh(sq(sq(dmin(dmax(term1, term2), term3))));
  double talpha = bigf * c59 + (1.0 - bigf) * 0.44;
  double tbeta = bigf * 0.075 + (1.0 - bigf) * 0.0828;
  double ki = 1.0 / k, oi = 1.0 / o, ei = 1.0 / tv[2];
  const double vorticity_sq = sq(dudy - dvdx) + sq(dudz - dwdx) + sq(dvdz - dwdy);
  double tl = turb_length(ides, k, o, bigf, strain_sq, vorticity_sq, cx1, cx2, ex1, ex2, tx1, tx2, grd, tv);
  double dest = dv[0] * std::pow(k, 1.5) / tl;
  r.source[0] = (prod - dest) * grd[0];
  r.source[1] = (talpha * dv[0] * ei * prod - tbeta * dv[0] * sq(o) + 1.712 * (1.0 - bigf) * dv[0] * oi * pkw) * grd[0];
  double dpdk = prod * ki;
  double dpdo = -((prod + c23 * dv[0] * k * div) * oi);
  r.itt[0] = dpdk - dest * ki;
  r.itt[1] = dpdo - dest * oi;
  r.itt[2] = 0.0;
  r.itt[3] = talpha * dv[0] * ei * dpdo + talpha * dv[0] * ei * prod * oi - 2.0 * tbeta * dv[0] * o -
             1.712 * (1.0 - bigf) * dv[0] * sq(oi) * pkw;
  double t = r.itt[0] + r.itt[3];
  double d = r.itt[0] * r.itt[3] - r.itt[1] * r.itt[2];
  double lam1 = 0.5 * t + std::sqrt(dmax(0.25 * sq(t) - d, 0.0));
  double lam2 = 0.5 * t - std::sqrt(dmax(0.25 * sq(t) - d, 0.0));
  lam1 = dsign(1.0, lam1);
  lam2 = dsign(1.0, lam2);
  double f1 = phi * (1.0 - 0.5 * (1.0 - lam1)) - 0.5 * (1.0 - lam1);
  double f2 = phi * (1.0 - 0.5 * (1.0 - lam2)) - 0.5 * (1.0 - lam2);
  r.itt[0] *= f1; r.itt[1] *= f1;
  r.itt[2] *= f2; r.itt[3] *= f2;
  return r;
}

/* t_kepsilon kepsilon (src/turbsource_module.f90:170-267) */
static inline TurbOut kepsilon_source(const double (*x)[NPV_MAX], const double* cx1, const double* cx2,
                                      const double* ex1, const double* ex2, const double* tx1, const double* tx2,
                                      const double* grd, const double* dv, const double* tv) {
  TurbOut r;
  const double c23 = 2.0 / 3.0, phi = 1.0;
  double gu[3], gv[3], gw[3], gk[3];
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 1, gu);
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 2, gv);
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 3, gw);
  /* the gradient of sqrt(k) from the square roots of the face averages */
  const double k1 = 0.5 * (x[0][7] + x[1][7]), k2 = 0.5 * (x[2][7] + x[1][7]), k3 = 0.5 * (x[3][7] + x[1][7]);
  const double k4 = 0.5 * (x[4][7] + x[1][7]), k5 = 0.5 * (x[5][7] + x[1][7]), k6 = 0.5 * (x[6][7] + x[1][7]);
  const double vol = 1.0 / grd[0];
  for (int d = 0; d < 3; ++d)
    gk[d] = (std::sqrt(k2) * cx2[d] + std::sqrt(k4) * ex2[d] + std::sqrt(k6) * tx2[d] - std::sqrt(k1) * cx1[d] -
             std::sqrt(k3) * ex1[d] - std::sqrt(k5) * tx1[d]) * vol;
  const double dudx = gu[0], dudy = gu[1], dudz = gu[2], dvdx = gv[0], dvdy = gv[1], dvdz = gv[2];
  const double dwdx = gw[0], dwdy = gw[1], dwdz = gw[2];
  const double k = x[1][7], e = x[1][8];
  const double kkyy = sq(gk[0]) + sq(gk[1]) + sq(gk[2]);
  double prod = tv[2] * (2.0 * (sq(dudx) + sq(dvdy) + sq(dwdz)) + sq(dudy + dvdx) + sq(dudz + dwdx) + sq(dvdz + dwdy) -
                         c23 * sq(dudx + dvdy + dwdz)) - c23 * dv[0] * k * (dudx + dvdy + dwdz);
  const double re_t = dv[0] * sq(k) / e / tv[0];
  const double fe1 = 1.0 - std::exp(-sq(re_t / 40.0));
  const double fe2 = 1.0 - 2.0 / 9.0 * std::exp(-sq(re_t / 6.0));
  prod = dmin(prod, 30.0 * dv[0] * e);
  const double ki = 1.0 / k, oi = 1.0 / e;
  r.omega_cut = 0.0;
  r.source[0] = (prod - dv[0] * e - 2.0 * tv[0] * kkyy) * grd[0];
  r.source[1] = (1.5 * fe1 * prod * e - 1.9 * fe2 * dv[0] * sq(e) + 2.9556 * tv[0] * e * kkyy) * ki * grd[0];
  const double dpdk = 2.0 * prod * ki + c23 * dv[0] * (dudx + dvdy + dwdz);
  const double dpdo = -((prod + c23 * dv[0] * k * (dudx + dvdy + dwdz)) * oi);
  r.itt[0] = dpdk;
  r.itt[1] = dpdo - dv[0];
  r.itt[2] = (1.9 * fe2 * dv[0] * sq(e) - 2.9556 * tv[0] * e * kkyy) * sq(ki);
  r.itt[3] = (1.5 * fe1 * dpdo * e + 1.5 * fe1 * prod - 3.8 * fe2 * dv[0] * e + 2.9556 * tv[0] * kkyy) * ki;
  const double t = r.itt[0] + r.itt[3], dd = r.itt[0] * r.itt[3] - r.itt[1] * r.itt[2];
  double lam1 = 0.5 * t + std::sqrt(dmax(0.25 * sq(t) - dd, 0.0));
  double lam2 = 0.5 * t - std::sqrt(dmax(0.25 * sq(t) - dd, 0.0));
  lam1 = dsign(1.0, lam1);
  lam2 = dsign(1.0, lam2);
  const double f1 = phi * (1.0 - 0.5 * (1.0 - lam1)) - 0.5 * (1.0 - lam1);
  const double f2 = phi * (1.0 - 0.5 * (1.0 - lam2)) - 0.5 * (1.0 - lam2);
  r.itt[0] *= f1; r.itt[1] *= f1;
  r.itt[2] *= f2; r.itt[3] *= f2;
  return r;
}

/* t_eddy_ke kepsilon (src/eddy_module.f90) */
static inline double kepsilon_eddy(const double* pv, const double* dv, const double* tv, const double* grd) {
  const double re_t = dv[0] * sq(pv[7]) / pv[8] / tv[0];
  const double re_e = dv[0] * std::pow(tv[0] / dv[0] * pv[8], 0.25) * grd[4] / tv[0];
  const double f_mu = (1.0 + 3.0 / std::pow(re_t, 3.0 / 4.0)) * (1.0 + 80.0 * std::exp(-re_e)) *
                      sq(1.0 - std::exp(-re_e / 43.0 - sq(re_e) / 330.0));
  return 0.09 * dv[0] * sq(pv[7]) / pv[8] * f_mu;
}

/* eddy%caleddy, SST (src/eddy_module.f90:135-187) */
static inline double kwsst_eddy(const double (*x)[NPV_MAX], const double* cx1, const double* cx2,
                                const double* ex1, const double* ex2, const double* tx1, const double* tx2,
                                const double* grd, const double* dv, const double* tv) {
  double gu[3], gv[3], gw[3];
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 1, gu);
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 2, gv);
  cell_grad(x, cx1, cx2, ex1, ex2, tx1, tx2, grd[0], 3, gw);
  const double k = x[1][7], o = x[1][8];
  double term1 = std::sqrt(k) / (0.09 * o * grd[4]);
  double term2 = 500.0 * tv[0] / dv[0] / (o * sq(grd[4]));
  double arg2 = dmax(2.0 * term1, term2);
  double bigf2 = std::tanh(sq(arg2));
  double sijsij = sq(gu[0]) + sq(gv[1]) + sq(gw[2]) + 0.5 * (sq(gu[1] + gv[0]) + sq(gu[2] + gw[0]) + sq(gv[2] + gw[1]));
  double sss = std::sqrt(2.0 * sijsij);
  double term6 = dmax(0.31 * o, sss * bigf2);
  return 0.31 * dv[0] * k / term6;
}

/* dual-time source (src/unsteady_module.f90:96-114) */
static inline void unsteady_source(const Cfg& c, const double* pv2, const double* dv, const double* qq1,
                                   const double* qq2, double vol, double* fx) {
  double b = (c.nsteady == 1) ? 1.0 : 1.5 * 0.5;
  fx[0] = dv[0];
  fx[1] = dv[0] * pv2[1];
  fx[2] = dv[0] * pv2[2];
  fx[3] = dv[0] * pv2[3];
  fx[4] = dv[0] * (dv[1] + 0.5 * (sq(pv2[1]) + sq(pv2[2]) + sq(pv2[3]))) - (pv2[0] + c.pref);
  for (int n = 5; n < c.npv; ++n) fx[n] = dv[0] * pv2[n];
  for (int n = 0; n < c.npv; ++n) {
    fx[n] = (double)c.nsteady * (b * fx[n] - qq1[n]) + 0.5 * ((double)c.nsteady - 1.0) * qq2[n];
    fx[n] = fx[n] * vol / c.dt_phy;
  }
}

/* ================= diagonal operator (src/lhs_module.f90:346-534) ================= */
static inline double eigenvis_of(const Cfg& c, const double* dv, const double* tv) {
  if (c.iturb == -3) return 0.0;
  if (c.iturb == -2)
    return dmax(dv[6] * tv[1] / (dv[7] + dv[11] * dv[6] * dv[0] - dv[10] * dv[7] * dv[0]), 4.0 / 3.0 * tv[0] / dv[0]);
  return dmax(dv[6] * (tv[1] + dv[11] * tv[2] / 0.9) / (dv[7] + dv[11] * dv[6] * dv[0] - dv[10] * dv[7] * dv[0]),
              4.0 / 3.0 * (tv[0] + tv[2]) / dv[0]);
}

struct LhsIn {
  const double *cx1, *cx2, *ex1, *ex2, *tx1, *tx2, *grd, *pv, *dv, *tv;
  double dt;
  const double* c;   /* icav(4) or zeros */
  const double* t;   /* itt(4) or zeros */
};

static inline double lhs_eigen(const Cfg& cf, const LhsIn& L) {
  const double cappa = 1.05;
  double uv2 = sq(L.pv[1]) + sq(L.pv[2]) + sq(L.pv[3]);
  double sndp2 = sndp2_of(cf, L.dv[5], uv2);
  const double* fa[3][2] = {{L.cx1, L.cx2}, {L.ex1, L.ex2}, {L.tx1, L.tx2}};
  double lamda = 0.0;
  for (int d = 0; d < 3; ++d) {
    double ox = 0.5 * (fa[d][0][0] + fa[d][1][0]);
    double oy = 0.5 * (fa[d][0][1] + fa[d][1][1]);
    double oz = 0.5 * (fa[d][0][2] + fa[d][1][2]);
    double ds = sq(ox) + sq(oy) + sq(oz);
    double u = ox * L.pv[1] + oy * L.pv[2] + oz * L.pv[3];
    double up = 0.5 * (1.0 + sndp2 / L.dv[5]) * u;
    double dd = 0.5 * std::sqrt(sq(u) * sq(1.0 - sndp2 / L.dv[5]) + 4.0 * sndp2 * ds);
    if (d == 0) lamda = cappa * (std::fabs(up) + dd);
    else lamda = lamda + cappa * (std::fabs(up) + dd);
  }
  return lamda;
}

static inline void lhs_getx(const Cfg& cf, const LhsIn& L, const double* res, double* x) {
  const double* pv = L.pv;
  const double* dv = L.dv;
  double ev = eigenvis_of(cf, dv, L.tv);
  if (cf.iturb != -3) {
    ev = ev * (0.25 * sq(L.cx1[0] + L.cx2[0]) + 0.25 * sq(L.cx1[1] + L.cx2[1]) + 0.25 * sq(L.cx1[2] + L.cx2[2]) +
               0.25 * sq(L.ex1[0] + L.ex2[0]) + 0.25 * sq(L.ex1[1] + L.ex2[1]) + 0.25 * sq(L.ex1[2] + L.ex2[2]) +
               0.25 * sq(L.tx1[0] + L.tx2[0]) + 0.25 * sq(L.tx1[1] + L.tx2[1]) + 0.25 * sq(L.tx1[2] + L.tx2[2]));
  }
  double bb = (cf.nsteady == 1) ? 1.0 : ((cf.nsteady == 2) ? 0.75 : 0.0);
  double a = 1.0 / (L.grd[0] / L.dt + lhs_eigen(cf, L));
  double unst = (cf.nsteady >= 1) ? (double)cf.nsteady * bb * L.grd[0] / cf.dt_phy : 0.0;
  double b = (unst + 2.0 * ev / L.grd[0]) * a;
  double c[4], t[4];
  for (int q = 0; q < 4; ++q) { c[q] = L.c[q] * L.grd[0] * a; t[q] = L.t[q] * L.grd[0] * a; }
  double b1 = 1.0 + b;
  double i_b1 = 1.0 / (b1 * dv[0]);
  double uv2 = sq(pv[1]) + sq(pv[2]) + sq(pv[3]);
  double sndp2 = sndp2_of(cf, dv[5], uv2);
  double ss = dv[0] * dv[11] * (1.0 / sndp2 + b / dv[5]);
  double rr = 1.0 / sndp2 - 1.0 / dv[5] + b1 * dv[6];
  double hst = dv[1] + 0.5 * (sq(pv[1]) + sq(pv[2]) + sq(pv[3])) - rot_q(cf, L.grd + 1) - uv2;
  double cross = dv[13] * dv[8] - dv[12] * dv[9];
  double cross1 = dv[12] * dv[7] - dv[11] * dv[8];
  double cross2 = dv[13] * dv[7] - dv[11] * dv[9];
  double dhdp1 = 1.0 - dv[10] * dv[0];
  double ssy1 = dv[12] * dv[0] * rr + b1 * dv[8] * dhdp1;
  double ssy2 = dv[13] * dv[0] * rr + b1 * dv[9] * dhdp1;
  double ssh = dv[0] * rr * hst - b1 * dhdp1 * dv[0];
  double aaa1 = dv[8] * hst + dv[12] * dv[0] - cross * pv[6];
  double aaa2 = dv[7] * hst + dv[11] * dv[0] - cross2 * pv[6];
  double uuu = res[1] * pv[1] + res[2] * pv[2] + res[3] * pv[3] - res[4];
  double coeff1 = res[0] * aaa1 + dv[8] * uuu + cross * res[6];
  double coeff2 = res[0] * aaa2 + dv[7] * uuu + cross2 * res[6];
  double coeff3 = res[0] * (ssh - ssy2 * pv[6]) + dv[0] * rr * uuu + res[6] * ssy2;
  double mm = b1 * dv[0] * (ss + c[0] * cross1) - c[1] * ssy1 + c[2] * ss;
  mm = 1.0 / mm;
  x[0] = (c[3] * cross1 * (res[0] * pv[6] - res[6]) - c[1] * coeff1 + c[2] * coeff2 +
          dv[0] * b1 * (coeff2 + cross1 * res[5] - cross1 * pv[5] * res[0])) * mm;
  x[1] = (res[1] - res[0] * pv[1]) * i_b1;
  x[2] = (res[2] - res[0] * pv[2]) * i_b1;
  x[3] = (res[3] - res[0] * pv[3]) * i_b1;
  x[4] = (c[3] * i_b1 * ssy1 * (res[6] - res[0] * pv[6]) + c[0] * coeff1 - c[2] * i_b1 * coeff3 -
          (coeff3 - ssy1 * pv[5] * res[0] + res[5] * ssy1)) * mm;
  x[5] = (ss * (res[5] - res[0] * pv[5]) - c[3] * ss * i_b1 * (res[6] - res[0] * pv[6]) - c[0] * coeff2 +
          c[1] * i_b1 * coeff3) * mm;
  x[6] = (res[6] - res[0] * pv[6]) * i_b1;
  if (cf.npv > 7) {
    double tt = 1.0 / (t[1] * t[2] - (t[0] + b1 * dv[0]) * (t[3] + b1 * dv[0]));
    x[7] = ((res[8] - res[0] * pv[8]) * t[1] - (b1 * dv[0] + t[3]) * (res[7] - res[0] * pv[7])) * tt;
    x[8] = ((res[7] - res[0] * pv[7]) * t[2] - (b1 * dv[0] + t[0]) * (res[8] - res[0] * pv[8])) * tt;
  }
  for (int n = 0; n < cf.npv; ++n) x[n] = x[n] * a;
}

/* flowonly_ex / flowturball_ex (src/lhs_module.f90:247-344): the explicit schemes' diagonal
 * solve, without spectral radii, viscous shift or source couplings; a = dt/vol. */
static inline void lhs_getx_ex(const Cfg& cf, const LhsIn& L, const double* res, double* x) {
  const double* pv = L.pv;
  const double* dv = L.dv;
  double bb = (cf.nsteady == 1) ? 1.0 : ((cf.nsteady == 2) ? 0.75 : 0.0);
  double a = L.dt / L.grd[0];
  double b = (cf.nsteady >= 1) ? (double)cf.nsteady * bb * L.grd[0] / cf.dt_phy * a : 0.0;
  double b1 = 1.0 + b;
  double i_b1 = 1.0 / (b1 * dv[0]);
  double uv2 = sq(pv[1]) + sq(pv[2]) + sq(pv[3]);
  double ss = dv[0] * dv[11] * (1.0 / sndp2_of(cf, dv[5], uv2) + b / dv[5]);
  double rr = 1.0 / sndp2_of(cf, dv[5], uv2) - 1.0 / dv[5] + b1 * dv[6];
  double hst = dv[1] + 0.5 * (sq(pv[1]) + sq(pv[2]) + sq(pv[3])) - rot_q(cf, L.grd + 1) - uv2;
  double cross = dv[13] * dv[8] - dv[12] * dv[9];
  double cross1 = dv[12] * dv[7] - dv[11] * dv[8];
  double cross2 = dv[13] * dv[7] - dv[11] * dv[9];
  double dhdp1 = 1.0 - dv[10] * dv[0];
  double ssy1 = dv[12] * dv[0] * rr + b1 * dv[8] * dhdp1;
  double ssy2 = dv[13] * dv[0] * rr + b1 * dv[9] * dhdp1;
  double ssh = dv[0] * rr * hst - b1 * dhdp1 * dv[0];
  double aaa2 = dv[7] * hst + dv[11] * dv[0] - cross2 * pv[6];
  double uuu = res[1] * pv[1] + res[2] * pv[2] + res[3] * pv[3] - res[4];
  double coeff2 = res[0] * aaa2 + dv[7] * uuu + cross2 * res[6];
  double coeff3 = res[0] * (ssh - ssy2 * pv[6]) + dv[0] * rr * uuu + res[6] * ssy2;
  double mm = 1.0 / ss;
  (void)cross;
  x[0] = (coeff2 + cross1 * res[5] - cross1 * pv[5] * res[0]) * mm;
  x[1] = (res[1] - res[0] * pv[1]) * i_b1;
  x[2] = (res[2] - res[0] * pv[2]) * i_b1;
  x[3] = (res[3] - res[0] * pv[3]) * i_b1;
  x[4] = -(coeff3 - ssy1 * pv[5] * res[0] + res[5] * ssy1) * mm * i_b1;
  for (int n = 5; n < cf.npv; ++n) x[n] = (res[n] - res[0] * pv[n]) * i_b1;
  for (int n = 0; n < cf.npv; ++n) x[n] = x[n] * a;
}

/* ================= split Jacobian (src/jacobian_module.f90:182-403) ================= */
static inline void caljac(const Cfg& cf, const double* nx, const double* grd, const double* pv, const double* dv,
                          const double* tv, int sign, double a[NPV_MAX][NPV_MAX]) {
  const double cappa = 1.05;
  double ds = sq(nx[0]) + sq(nx[1]) + sq(nx[2]);
  double u = nx[0] * pv[1] + nx[1] * pv[2] + nx[2] * pv[3];
  double sndp2 = sndp2_of(cf, dv[5], sq(pv[1]) + sq(pv[2]) + sq(pv[3]));
  double up = 0.5 * (1.0 + sndp2 / dv[5]) * u;
  double d = 0.5 * std::sqrt(sq(u) * sq(1.0 - sndp2 / dv[5]) + 4.0 * sndp2 * ds);
  double lamda = (double)sign * cappa * (std::fabs(up) + d);
  double vis = (double)sign * 2.0 * eigenvis_of(cf, dv, tv) * ds / grd[0];
  double beta = 1.0 / sndp2 - 1.0 / dv[5] + dv[6];
  double a1 = u * dv[6], a2 = nx[0] * dv[0], a3 = nx[1] * dv[0], a4 = nx[2] * dv[0];
  double a5 = u * dv[7], a6 = u * dv[8], a7 = u * dv[9];
  double g1 = lamda * beta, g5 = lamda * dv[7], g6 = lamda * dv[8], g7 = lamda * dv[9];
  double ge1 = vis * dv[6], ge5 = vis * dv[7], ge6 = vis * dv[8], ge7 = vis * dv[9];
  double uuu = u + lamda + vis;
  const int np = cf.npv;
  for (int i = 0; i < np; ++i) for (int j = 0; j < np; ++j) a[i][j] = 0.0;
  a[0][0] = a1 + g1 + ge1; a[0][1] = a2; a[0][2] = a3; a[0][3] = a4;
  a[0][4] = a5 + g5 + ge5; a[0][5] = a6 + g6 + ge6; a[0][6] = a7 + g7 + ge7;
  for (int r = 1; r <= 3; ++r) {
    for (int j = 0; j < 7; ++j) a[r][j] = pv[r] * a[0][j];
    a[r][0] = pv[r] * a[0][0] + nx[r - 1];
    a[r][r] = pv[r] * a[0][r] + dv[0] * uuu;
  }
  double h = dv[1] + 0.5 * (sq(pv[1]) + sq(pv[2]) + sq(pv[3])) - rot_q(cf, grd + 1);
  a[4][0] = dv[0] * uuu * dv[10] + h * a[0][0] - lamda - vis;
  a[4][1] = dv[0] * uuu * pv[1] + h * a[0][1];
  a[4][2] = dv[0] * uuu * pv[2] + h * a[0][2];
  a[4][3] = dv[0] * uuu * pv[3] + h * a[0][3];
  a[4][4] = dv[0] * uuu * dv[11] + h * a[0][4];
  a[4][5] = dv[0] * uuu * dv[12] + h * a[0][5];
  a[4][6] = dv[0] * uuu * dv[13] + h * a[0][6];
  for (int r = 5; r <= 6; ++r) {
    for (int j = 0; j < 7; ++j) a[r][j] = pv[r] * a[0][j];
    a[r][r] = pv[r] * a[0][r] + dv[0] * uuu;
  }
  if (np > 7) {
    for (int r = 7; r <= 8; ++r) {
      for (int j = 0; j < 7; ++j) a[r][j] = pv[r] * a[0][j];
      a[r][r] = uuu * dv[0];
    }
  }
  for (int i = 0; i < np; ++i) for (int j = 0; j < np; ++j) a[i][j] = a[i][j] * 0.5;
}

}  // namespace orc
#endif
