/*
 * cfd3d_oracle.cpp -- TEST INFRASTRUCTURE ONLY: the CPU oracle.
 *
 * A line-by-line FP64 restatement of kwonhwi1/3dcode's per-pseudo-iteration hot path
 * (LU-SGS `lusgs`, src/update_module.f90:455-733, with everything it calls), plus the
 * set-up it depends on (grid metrics src/grid_module.f90:609-1241, wall distance
 * :350-607, BC/edge/corner/halo descriptors src/bc_module.f90:71-1188, initial state
 * src/initial_module.f90:678-771).  Storage follows the reference: AoS arrays with the
 * variable index fastest and the padded index ranges of src/variable_module.f90:69-77.
 *
 * Used only by tests/ (to verify the GPU path) and by bench.py's CPU-baseline arm (timed).  The product
 * library never links or calls it.
 *
 * parity unpinned: the reference cannot be compiled here (Fortran + MPI + CGNS) and has
 * no tests or golden vectors of its own.
 *
 * Multi-block: the MPI ranks of the reference become blocks processed in turn; the
 * per-rank phases are kept (all face BCs, then every halo copy, then edges, then
 * corners), which is the order an MPI run produces.
 */
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <thread>
#include "../include/cfd3d.h"
#include "oracle_schemes.h"

namespace orc {
long g_snd2_fallbacks = 0;
}
using namespace orc;

namespace {

/* ---------------- Fortran-style array with lower bounds ---------------- */
struct A4 {
  std::vector<double> d;
  int nv = 0, lo[3] = {0, 0, 0}, n[3] = {0, 0, 0};
  void init(int nv_, int l1, int h1, int l2, int h2, int l3, int h3) {
    nv = nv_; lo[0] = l1; lo[1] = l2; lo[2] = l3;
    n[0] = h1 - l1 + 1; n[1] = h2 - l2 + 1; n[2] = h3 - l3 + 1;
    d.assign((size_t)nv * n[0] * n[1] * n[2], 0.0);
  }
  size_t off(int i, int j, int k) const {
    return (size_t)nv * ((size_t)(i - lo[0]) + (size_t)n[0] * ((size_t)(j - lo[1]) + (size_t)n[1] * (size_t)(k - lo[2])));
  }
  double* at(int i, int j, int k) { return &d[off(i, j, k)]; }
  const double* at(int i, int j, int k) const { return &d[off(i, j, k)]; }
  double& operator()(int v, int i, int j, int k) { return d[off(i, j, k) + v]; }
};

enum Face { F_IMIN, F_IMAX, F_JMIN, F_JMAX, F_KMIN, F_KMAX, F_KMIN_CAP, F_KMAX_CAP, F_NONE };

enum BcKind {
  K_WALL_INVISCID, K_WALL_VISCOUS, K_WALL_KW, K_FARFIELD, K_EXTRAP, K_SYMMETRY, K_NOOP,
  K_INFLOW_SUB, K_OUTFLOW_SUB, K_INFLOW_SUP, K_CRWALL_KW, K_MASSFLOW_IN, K_SHIFTED, K_HFWALL_KW, K_WALL_KE, K_TOTALP,
  K_CRWALL, K_CRWALL_INV,
  K_EDGE_WALLWALL, K_EDGE_WALLWALL_KW, K_EDGE_NOWALL, K_CORNER_WALLWALL, K_CORNER_WALLWALL_KW, K_CORNER_NOWALL
};

struct BcInfo {
  int type = 0;   /* cfd3d BC type for face patches */
  BcKind kind = K_NOOP;
  Face face = F_NONE;
  int istart[3], iend[3], origin[3] = {0, 0, 0}, dir[3] = {0, 0, 0};
  int nb[6][3];
  double pressure = 0;
  double pv[NPV_MAX], dv[NDV], tv[3];
  std::vector<double> tdata, heatflux;   /* HeatFlux walls: the <family>.dat history */
  double time = 0.0;                     /* bcinfo%time, set by setbc */
  /* total-pressure inlets: the pooled Newton solution (p, T) and |u_avg|^2, set by setbc */
  double tpx[2] = {0.0, 0.0}, tpuu = 0.0;
};

struct Conn {
  int donor;
  int istart[3], iend[3], istart_d[3], iend_d[3];
  int tm[3][3];
  int face;
};

struct Block {
  int imax, jmax, kmax;
  A4 x, cx, ex, tx, grd;
  A4 pv, dv, tv, qq, rcav;
  A4 res, icav, itt, omega_cut, dt;
  A4 dqs, dcv, qres;
  A4 vfg, csf;                  /* csf = 1: volume-fraction gradient, surface-tension source */
  std::vector<BcInfo> bcs;
  BcInfo edge[12], corner[8];
  std::vector<Conn> cons;       /* state halo (3 layers) */
  std::vector<Conn> gcons;      /* metric halo (1 layer) */
};

struct Oracle {
  Cfg c;
  std::vector<Block> b;
  double time_acc = 0.0;        /* the SAVE'd `time` of localtime (src/timestep_module.f90:146) */
  double time_cur = 0.0;
  int nthreads = 1;
  std::string err;
};

/* ---------------- config (src/config_module.f90:90-199) ---------------- */
static bool make_cfg(const cfd3d_config* in, Cfg& c, std::string& err) {
  c = Cfg();   /* value-initialised: zeros, empty histories */
  c.nsteady = in->nsteady; c.dt_phy = in->dt_phy;
  c.iturb = in->iturb; c.ides = in->ides; c.nscheme = in->nscheme; c.nmuscl = in->nmuscl; c.nlim = in->nlim;
  c.local = in->local; c.prec = in->prec; c.cfl = in->cfl; c.fluid = in->fluid; c.ngas = in->ngas;
  c.ncav = in->ncav; c.c_v = in->c_v; c.c_c = in->c_c; c.pref = in->pref; c.uref = in->uref;
  c.tref = in->tref; c.y1ref = in->y1ref; c.y2ref = in->y2ref; c.l_chord = in->l_chord;
  c.l_character = in->l_character; c.scale = in->scale; c.l_domain = in->l_domain;
  c.fix_cav_clamp = in->fix_cav_clamp;
  c.pi = std::atan(1.0) * 4.0;
  c.aoa = in->aoa * c.pi / 180.0; c.aos = in->aos * c.pi / 180.0;
  c.str = c.l_character / c.pi / c.dt_phy;
  c.timemethod = in->timemethod;
  /* gravity (src/gravity_module.f90:24-66): a constant axis acceleration or the history */
  c.gravity = in->gravity;
  if (c.gravity == 4) {
    if (in->ngravity < 1 || !in->gravity_data) { err = "gravity = 4 without its history"; return false; }
    for (int m = 0; m < in->ngravity; ++m) {
      c.grav_t.push_back(in->gravity_data[4 * m]);
      for (int e = 0; e < 3; ++e) c.grav_a.push_back(in->gravity_data[4 * m + 1 + e]);
    }
  } else if (c.gravity >= -3 && c.gravity <= 3 && c.gravity != 0) {
    c.grav_t = {0.0};
    c.grav_a = {0.0, 0.0, 0.0};
    c.grav_a[std::abs(c.gravity) - 1] = (c.gravity > 0 ? 1.0 : -1.0) * 9.80665;
  } else if (c.gravity != 0) { err = "gravity must be 0, +-1, +-2, +-3 or 4"; return false; }
  c.csf = in->csf;
  if (c.csf != 0 && c.csf != 1) { err = "csf must be 0 or 1"; return false; }
  /* rotation, rpm: omega along +-x, +-y, +-z (src/config_module.f90:126-141) */
  c.rotation = in->rotation;
  if (c.rotation < -3 || c.rotation > 3) { err = "rotation must be 0, +-1, +-2 or +-3"; return false; }
  for (int e = 0; e < 3; ++e) c.omega[e] = 0.0;
  if (c.rotation != 0)
    c.omega[std::abs(c.rotation) - 1] = (c.rotation > 0 ? 1.0 : -1.0) * in->rpm * 2.0 * c.pi / 60.0;
  if (c.timemethod < 1 || c.timemethod > 3) { err = "timemethod must be 1 (Euler), 2 (RK3) or 3 (LU-SGS)"; return false; }
  if (c.iturb == -3) { c.npv = 7; c.ntv = 0; }
  else if (c.iturb == -2) { c.npv = 7; c.ntv = 2; }
  else if (c.iturb == 0 || c.iturb == -1) { c.npv = 9; c.ntv = 3; }
  else { err = "iturb must be -3, -2, -1 or 0"; return false; }
  if (c.iturb == 0 && (c.ides < 0 || c.ides > 4)) { err = "ides must be 0..4"; return false; }
  c.nqq = c.nsteady >= 1 ? 2 : 0;
  c.ngrd = (c.iturb >= -1) ? 5 : 4;
  if (c.fluid != 1 && c.fluid != 2) { err = "fluid must be 1 or 2"; return false; }
  if (c.ngas != 1) { err = "ngas must be 1"; return false; }
  if (c.nscheme < 1 || c.nscheme > 4 || c.nmuscl < 0 || c.nmuscl > 2 || c.nlim < 0 || c.nlim > 10) {
    err = "bad scheme"; return false;
  }
  if (c.local < -1 || c.local > 1) { err = "bad local"; return false; }
  c.with_prop = (c.iturb != -3);
  c.eos.fluid = c.fluid; c.eos.ngas = c.ngas;
  /* main.f90:31-32: deteos at the reference state, then setref */
  double dv[NDV], tv[3] = {0, 0, 0};
  deteos(c.eos, c.with_prop, c.pref, c.tref, c.y1ref, c.y2ref, dv, tv);
  c.rhoref = dv[0];
  {   /* the total-pressure inlet's construct (src/bc_module.f90:318-321, 336) */
    c.tp_pt = 51551.30907;
    c.tp_tt = 300.0003719;
    double dvt[NDV], tvt[3] = {0, 0, 0};
    deteos(c.eos, c.with_prop, c.tp_pt, c.tp_tt, c.y1ref, c.y2ref, dvt, tvt);
    c.tp_ht = dvt[1];
  }
  c.visref = tv[0];
  if (c.iturb == -1) {   /* config%setref for k-epsilon (src/config_module.f90:191-194) */
    c.kref = 1.5 * sq(0.0001 * c.uref);
    c.emutref = std::pow(10.0, -5) * tv[0];
    c.oref = 0.09 * c.rhoref * sq(c.kref) / c.emutref;
    if (in->kinf > 0) c.kref = in->kinf;
    if (in->oinf > 0) c.oref = in->oinf;
  }
  if (c.iturb == 0) {
    c.oref = 10.0 * c.uref / c.l_domain;
    c.emutref = std::pow(10.0, -5) * tv[0];
    c.kref = c.emutref / c.rhoref * c.oref;
    if (in->kinf > 0) c.kref = in->kinf;
    if (in->oinf > 0) c.oref = in->oinf;
  }
  return true;
}

/* ---------------- grid metrics (src/grid_module.f90:609-1241) ---------------- */
static double pyramid(const double* pa, const double* pb, const double* pc, const double* pd, double xc, double yc, double zc) {
  double csx = 0.25 * (pa[0] + pb[0] + pc[0] + pd[0]);
  double csy = 0.25 * (pa[1] + pb[1] + pc[1] + pd[1]);
  double csz = 0.25 * (pa[2] + pb[2] + pc[2] + pd[2]);
  double vax = pc[0] - pa[0], vay = pc[1] - pa[1], vaz = pc[2] - pa[2];
  double vbx = pd[0] - pb[0], vby = pd[1] - pb[1], vbz = pd[2] - pb[2];
  double volpx = (xc - csx) * (vay * vbz - vaz * vby);
  double volpy = (yc - csy) * (vaz * vbx - vax * vbz);
  double volpz = (zc - csz) * (vax * vby - vay * vbx);
  return std::fabs(volpx + volpy + volpz);
}

static void face_vectors(Block& B) {
  const int im = B.imax, jm = B.jmax, km = B.kmax;
  A4& X = B.x;
  B.cx.init(3, 1, im, 1, jm + 1, 1, km + 1);
  B.ex.init(3, 1, im + 1, 1, jm, 1, km + 1);
  B.tx.init(3, 1, im + 1, 1, jm + 1, 1, km);
  for (int k = 2; k <= km; ++k)
    for (int j = 2; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        double xe = X(0, i + 1, j + 1, k) - X(0, i + 1, j, k + 1), ye = X(1, i + 1, j + 1, k) - X(1, i + 1, j, k + 1),
               ze = X(2, i + 1, j + 1, k) - X(2, i + 1, j, k + 1);
        double xs = X(0, i + 1, j + 1, k + 1) - X(0, i + 1, j, k), ys = X(1, i + 1, j + 1, k + 1) - X(1, i + 1, j, k),
               zs = X(2, i + 1, j + 1, k + 1) - X(2, i + 1, j, k);
        B.cx(0, i, j, k) = 0.5 * (ye * zs - ys * ze);
        B.cx(1, i, j, k) = 0.5 * (xs * ze - xe * zs);
        B.cx(2, i, j, k) = 0.5 * (xe * ys - xs * ye);
      }
  for (int i = 2; i <= im; ++i)
    for (int k = 2; k <= km; ++k)
      for (int j = 1; j <= jm; ++j) {
        double xc = X(0, i, j + 1, k) - X(0, i + 1, j + 1, k + 1), yc = X(1, i, j + 1, k) - X(1, i + 1, j + 1, k + 1),
               zc = X(2, i, j + 1, k) - X(2, i + 1, j + 1, k + 1);
        double xs = X(0, i, j + 1, k + 1) - X(0, i + 1, j + 1, k), ys = X(1, i, j + 1, k + 1) - X(1, i + 1, j + 1, k),
               zs = X(2, i, j + 1, k + 1) - X(2, i + 1, j + 1, k);
        B.ex(0, i, j, k) = 0.5 * (yc * zs - ys * zc);
        B.ex(1, i, j, k) = 0.5 * (xs * zc - xc * zs);
        B.ex(2, i, j, k) = 0.5 * (xc * ys - xs * yc);
      }
  for (int j = 2; j <= jm; ++j)
    for (int i = 2; i <= im; ++i)
      for (int k = 1; k <= km; ++k) {
        double xc = X(0, i + 1, j, k + 1) - X(0, i, j + 1, k + 1), yc = X(1, i + 1, j, k + 1) - X(1, i, j + 1, k + 1),
               zc = X(2, i + 1, j, k + 1) - X(2, i, j + 1, k + 1);
        double xe = X(0, i + 1, j + 1, k + 1) - X(0, i, j, k + 1), ye = X(1, i + 1, j + 1, k + 1) - X(1, i, j, k + 1),
               ze = X(2, i + 1, j + 1, k + 1) - X(2, i, j, k + 1);
        B.tx(0, i, j, k) = 0.5 * (yc * ze - ye * zc);
        B.tx(1, i, j, k) = 0.5 * (xe * zc - xc * ze);
        B.tx(2, i, j, k) = 0.5 * (xc * ye - xe * yc);
      }
  /* degenerate faces */
  for (auto& bc : B.bcs) {
    if (bc.type != CFD3D_BC_DEGENERATE) continue;
    auto zero = [](A4& a, int axis, int idx) {
      for (int k = a.lo[2]; k < a.lo[2] + a.n[2]; ++k)
        for (int j = a.lo[1]; j < a.lo[1] + a.n[1]; ++j)
          for (int i = a.lo[0]; i < a.lo[0] + a.n[0]; ++i) {
            int q = axis == 0 ? i : (axis == 1 ? j : k);
            if (q == idx) for (int v = 0; v < 3; ++v) a(v, i, j, k) = 0.0;
          }
    };
    if (bc.face == F_IMIN) zero(B.cx, 0, 1);
    if (bc.face == F_IMAX) zero(B.cx, 0, im);
    if (bc.face == F_JMIN) zero(B.ex, 1, 1);
    if (bc.face == F_JMAX) zero(B.ex, 1, jm);
    if (bc.face == F_KMIN) zero(B.tx, 2, 1);
    if (bc.face == F_KMAX) zero(B.tx, 2, km);
  }
  /* ghost edges of the face arrays */
  for (int k = 1; k <= km + 1; ++k) for (int i = 1; i <= im; ++i) for (int v = 0; v < 3; ++v) {
    B.cx(v, i, 1, k) = B.cx(v, i, 2, k); B.cx(v, i, jm + 1, k) = B.cx(v, i, jm, k);
  }
  for (int j = 1; j <= jm + 1; ++j) for (int i = 1; i <= im; ++i) for (int v = 0; v < 3; ++v) {
    B.cx(v, i, j, 1) = B.cx(v, i, j, 2); B.cx(v, i, j, km + 1) = B.cx(v, i, j, km);
  }
  for (int k = 1; k <= km + 1; ++k) for (int j = 1; j <= jm; ++j) for (int v = 0; v < 3; ++v) {
    B.ex(v, 1, j, k) = B.ex(v, 2, j, k); B.ex(v, im + 1, j, k) = B.ex(v, im, j, k);
  }
  for (int j = 1; j <= jm; ++j) for (int i = 1; i <= im + 1; ++i) for (int v = 0; v < 3; ++v) {
    B.ex(v, i, j, 1) = B.ex(v, i, j, 2); B.ex(v, i, j, km + 1) = B.ex(v, i, j, km);
  }
  for (int k = 1; k <= km; ++k) for (int j = 1; j <= jm + 1; ++j) for (int v = 0; v < 3; ++v) {
    B.tx(v, 1, j, k) = B.tx(v, 2, j, k); B.tx(v, im + 1, j, k) = B.tx(v, im, j, k);
  }
  for (int k = 1; k <= km; ++k) for (int i = 1; i <= im + 1; ++i) for (int v = 0; v < 3; ++v) {
    B.tx(v, i, 1, k) = B.tx(v, i, 2, k); B.tx(v, i, jm + 1, k) = B.tx(v, i, jm, k);
  }
}

static void volumes(const Cfg& c, Block& B) {
  const int im = B.imax, jm = B.jmax, km = B.kmax;
  A4& X = B.x;
  /* volumes and centroids */
  B.grd.init(c.ngrd, 1, im + 1, 1, jm + 1, 1, km + 1);
  A4& G = B.grd;
  for (int k = 2; k <= km; ++k)
    for (int j = 2; j <= jm; ++j)
      for (int i = 2; i <= im; ++i) {
        for (int v = 0; v < 3; ++v)
          G(1 + v, i, j, k) = 0.125 * (X(v, i, j, k) + X(v, i + 1, j, k) + X(v, i, j + 1, k) + X(v, i, j, k + 1) +
                                       X(v, i + 1, j + 1, k) + X(v, i, j + 1, k + 1) + X(v, i + 1, j, k + 1) +
                                       X(v, i + 1, j + 1, k + 1));
        const double xc = G(1, i, j, k), yc = G(2, i, j, k), zc = G(3, i, j, k);
        auto P = [&](int a, int b2, int c2, double* out) { for (int v = 0; v < 3; ++v) out[v] = X(v, a, b2, c2); };
        double pa[3], pb[3], pc[3], pd[3], vol = 0.0;
        double v6[6];
        P(i, j, k, pa); P(i + 1, j, k, pb); P(i + 1, j + 1, k, pc); P(i, j + 1, k, pd); v6[0] = pyramid(pa, pb, pc, pd, xc, yc, zc);
        P(i, j, k + 1, pa); P(i + 1, j, k + 1, pb); P(i + 1, j + 1, k + 1, pc); P(i, j + 1, k + 1, pd); v6[1] = pyramid(pa, pb, pc, pd, xc, yc, zc);
        P(i, j, k, pa); P(i + 1, j, k, pb); P(i + 1, j, k + 1, pc); P(i, j, k + 1, pd); v6[2] = pyramid(pa, pb, pc, pd, xc, yc, zc);
        P(i, j + 1, k, pa); P(i + 1, j + 1, k, pb); P(i + 1, j + 1, k + 1, pc); P(i, j + 1, k + 1, pd); v6[3] = pyramid(pa, pb, pc, pd, xc, yc, zc);
        P(i, j, k, pa); P(i, j + 1, k, pb); P(i, j + 1, k + 1, pc); P(i, j, k + 1, pd); v6[4] = pyramid(pa, pb, pc, pd, xc, yc, zc);
        P(i + 1, j, k, pa); P(i + 1, j + 1, k, pb); P(i + 1, j + 1, k + 1, pc); P(i + 1, j, k + 1, pd); v6[5] = pyramid(pa, pb, pc, pd, xc, yc, zc);
        vol = (v6[0] + v6[1] + v6[2] + v6[3] + v6[4] + v6[5]) / 6.0;
        G(0, i, j, k) = vol;
      }
  for (int k = 2; k <= km; ++k)
    for (int i = 2; i <= im; ++i) {
      G(0, i, 1, k) = G(0, i, 2, k);
      for (int v = 1; v <= 3; ++v) G(v, i, 1, k) = 2.0 * G(v, i, 2, k) - G(v, i, 3, k);
      G(0, i, jm + 1, k) = G(0, i, jm, k);
      for (int v = 1; v <= 3; ++v) G(v, i, jm + 1, k) = 2.0 * G(v, i, jm, k) - G(v, i, jm - 1, k);
    }
  for (int k = 2; k <= km; ++k)
    for (int j = 1; j <= jm + 1; ++j) {
      G(0, 1, j, k) = G(0, 2, j, k);
      for (int v = 1; v <= 3; ++v) G(v, 1, j, k) = 2.0 * G(v, 2, j, k) - G(v, 3, j, k);
      G(0, im + 1, j, k) = G(0, im, j, k);
      for (int v = 1; v <= 3; ++v) G(v, im + 1, j, k) = 2.0 * G(v, im, j, k) - G(v, im - 1, j, k);
    }
  for (int j = 1; j <= jm + 1; ++j)
    for (int i = 1; i <= im + 1; ++i) {
      G(0, i, j, 1) = G(0, i, j, 2);
      /* the reference extrapolates with the fixed cell (3, j, 3) here (src/grid_module.f90:1104-1106) */
      for (int v = 1; v <= 3; ++v) G(v, i, j, 1) = 2.0 * G(v, i, j, 2) - G(v, 3, j, 3);
      G(0, i, j, km + 1) = G(0, i, j, km);
      for (int v = 1; v <= 3; ++v) G(v, i, j, km + 1) = 2.0 * G(v, i, j, km) - G(v, i, j, km - 1);
    }
}

/* wall distance: the nearest wall-face centre over all blocks (src/grid_module.f90:350-607) */
static void wall_distance(Oracle& O) {
  if (O.c.ngrd < 5) return;
  std::vector<double> wx, wy, wz;
  for (auto& B : O.b) {
    A4& X = B.x;
    for (auto& bc : B.bcs) {
      if (bc.type != CFD3D_BC_WALL && bc.type != CFD3D_BC_WALL_COUNTERROTATING && bc.type != CFD3D_BC_WALL_HEATFLUX) continue;
      /* the patch ranges here are the grid module's (cell ranges before ghost extension) */
      int s[3], e[3];
      for (int d = 0; d < 3; ++d) { s[d] = bc.istart[d]; e[d] = bc.iend[d]; }
      if (bc.face == F_IMIN) s[0] = e[0] = 1;
      if (bc.face == F_JMIN) s[1] = e[1] = 1;
      if (bc.face == F_KMIN) s[2] = e[2] = 1;
      if (bc.face == F_IMAX) { s[0] = B.imax + 1; e[0] = s[0]; }
      if (bc.face == F_JMAX) { s[1] = B.jmax + 1; e[1] = s[1]; }
      if (bc.face == F_KMAX) { s[2] = B.kmax + 1; e[2] = s[2]; }
      if (bc.face == F_IMIN || bc.face == F_IMAX) {
        int ip = (bc.face == F_IMIN) ? 2 : B.imax + 1;
        for (int k = s[2]; k <= e[2]; ++k) for (int j = s[1]; j <= e[1]; ++j) {
          wx.push_back(0.25 * (X(0, ip, j, k) + X(0, ip, j + 1, k) + X(0, ip, j, k + 1) + X(0, ip, j + 1, k + 1)));
          wy.push_back(0.25 * (X(1, ip, j, k) + X(1, ip, j + 1, k) + X(1, ip, j, k + 1) + X(1, ip, j + 1, k + 1)));
          wz.push_back(0.25 * (X(2, ip, j, k) + X(2, ip, j + 1, k) + X(2, ip, j, k + 1) + X(2, ip, j + 1, k + 1)));
        }
      } else if (bc.face == F_JMIN || bc.face == F_JMAX) {
        int jp = (bc.face == F_JMIN) ? 2 : B.jmax + 1;
        for (int k = s[2]; k <= e[2]; ++k) for (int i = s[0]; i <= e[0]; ++i) {
          wx.push_back(0.25 * (X(0, i, jp, k) + X(0, i + 1, jp, k) + X(0, i, jp, k + 1) + X(0, i + 1, jp, k + 1)));
          wy.push_back(0.25 * (X(1, i, jp, k) + X(1, i + 1, jp, k) + X(1, i, jp, k + 1) + X(1, i + 1, jp, k + 1)));
          wz.push_back(0.25 * (X(2, i, jp, k) + X(2, i + 1, jp, k) + X(2, i, jp, k + 1) + X(2, i + 1, jp, k + 1)));
        }
      } else {
        int kp = (bc.face == F_KMIN) ? 2 : B.kmax + 1;
        for (int j = s[1]; j <= e[1]; ++j) for (int i = s[0]; i <= e[0]; ++i) {
          wx.push_back(0.25 * (X(0, i, j, kp) + X(0, i + 1, j, kp) + X(0, i, j + 1, kp) + X(0, i + 1, j + 1, kp)));
          wy.push_back(0.25 * (X(1, i, j, kp) + X(1, i + 1, j, kp) + X(1, i, j + 1, kp) + X(1, i + 1, j + 1, kp)));
          wz.push_back(0.25 * (X(2, i, j, kp) + X(2, i + 1, j, kp) + X(2, i, j + 1, kp) + X(2, i + 1, j + 1, kp)));
        }
      }
    }
  }
  /* The reference scans every wall-face centre for every cell.  The same minimum comes
     from a uniform grid of bins over the centres: bins are visited in shells of growing
     Chebyshev radius around the cell's bin until the nearest centre found is closer than
     any unvisited bin can be.  The distance of each candidate is the same expression, so
     the minimum is the scan's (the scan's 1e6 start value only matters with no wall). */
  const size_t nw = wx.size();
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (size_t m = 0; m < nw; ++m) {
    const double w3[3] = {wx[m], wy[m], wz[m]};
    for (int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], w3[d]); hi[d] = std::max(hi[d], w3[d]); }
  }
  int nb[3] = {1, 1, 1};
  double hb[3] = {1.0, 1.0, 1.0};
  std::vector<int> first, items;
  if (nw > 0) {
    double ext[3], vol = 1.0;
    int nd = 0;
    for (int d = 0; d < 3; ++d) { ext[d] = hi[d] - lo[d]; if (ext[d] > 0.0) { vol *= ext[d]; ++nd; } }
    const double side = (nd > 0) ? std::pow(vol / (double)nw, 1.0 / nd) : 1.0;   /* about one centre per bin */
    for (int d = 0; d < 3; ++d) {
      nb[d] = (ext[d] > 0.0) ? (int)std::min(512.0, std::max(1.0, std::ceil(ext[d] / side))) : 1;
      hb[d] = (ext[d] > 0.0) ? ext[d] / nb[d] : 0.0;   /* zero width: every centre in one plane */
    }
  }
  auto bin_of = [&](const double* q, int* b) {
    for (int d = 0; d < 3; ++d)
      b[d] = (hb[d] > 0.0) ? std::min(nb[d] - 1, std::max(0, (int)std::floor((q[d] - lo[d]) / hb[d]))) : 0;
  };
  if (nw > 0) {
    first.assign((size_t)nb[0] * nb[1] * nb[2] + 1, 0);
    std::vector<int> bi(nw);
    for (size_t m = 0; m < nw; ++m) {
      const double w3[3] = {wx[m], wy[m], wz[m]};
      int b[3];
      bin_of(w3, b);
      bi[m] = (b[2] * nb[1] + b[1]) * nb[0] + b[0];
      ++first[bi[m] + 1];
    }
    for (size_t q = 1; q < first.size(); ++q) first[q] += first[q - 1];
    items.resize(nw);
    std::vector<int> fill(first.begin(), first.end() - 1);
    for (size_t m = 0; m < nw; ++m) items[fill[bi[m]]++] = (int)m;
  }
  for (auto& B : O.b) {
    A4& X = B.x; A4& G = B.grd;
    const int im = B.imax, jm = B.jmax, km = B.kmax;
    for (int k = 2; k <= km; ++k)
      for (int j = 2; j <= jm; ++j)
        for (int i = 2; i <= im; ++i) {
          double c3[3];
          for (int v = 0; v < 3; ++v)
            c3[v] = 0.125 * (X(v, i, j, k) + X(v, i + 1, j, k) + X(v, i, j + 1, k) + X(v, i, j, k + 1) + X(v, i + 1, j + 1, k) +
                             X(v, i, j + 1, k + 1) + X(v, i + 1, j, k + 1) + X(v, i + 1, j + 1, k + 1));
          double ymin = 1.0e6;
          if (nw > 0) {
            int b[3];
            bin_of(c3, b);
            const int rmax = std::max(nb[0], std::max(nb[1], nb[2]));
            for (int r = 0; r <= rmax; ++r) {
              const int z0 = std::max(0, b[2] - r), z1 = std::min(nb[2] - 1, b[2] + r);
              const int y0 = std::max(0, b[1] - r), y1 = std::min(nb[1] - 1, b[1] + r);
              const int x0 = std::max(0, b[0] - r), x1 = std::min(nb[0] - 1, b[0] + r);
              for (int z = z0; z <= z1; ++z)
                for (int y = y0; y <= y1; ++y)
                  for (int x = x0; x <= x1; ++x) {
                    if (std::max(std::abs(z - b[2]), std::max(std::abs(y - b[1]), std::abs(x - b[0]))) != r) continue;
                    const int q = (z * nb[1] + y) * nb[0] + x;
                    for (int it = first[q]; it < first[q + 1]; ++it) {
                      const int m = items[it];
                      double yt = std::sqrt(sq(c3[0] - wx[m]) + sq(c3[1] - wy[m]) + sq(c3[2] - wz[m]));
                      if (yt < ymin) ymin = yt;
                    }
                  }
              /* the nearest any unvisited bin can be: past the visited slab along one
                 axis, and within the bins' extent along the other two; less a margin far
                 above rounding */
              double out[3];
              for (int d = 0; d < 3; ++d) {
                const double top = lo[d] + nb[d] * hb[d];
                out[d] = std::max(0.0, std::max(lo[d] - c3[d], c3[d] - top));
              }
              double bound = 1e300;
              for (int d = 0; d < 3; ++d) {
                const double rest = sq(out[(d + 1) % 3]) + sq(out[(d + 2) % 3]);
                if (b[d] - r > 0) bound = std::min(bound, std::sqrt(sq(std::max(0.0, c3[d] - (lo[d] + (b[d] - r) * hb[d]))) + rest));
                if (b[d] + r < nb[d] - 1) bound = std::min(bound, std::sqrt(sq(std::max(0.0, lo[d] + (b[d] + r + 1) * hb[d] - c3[d])) + rest));
              }
              if (bound >= 1e299 || ymin < bound - 1e-9 * (hb[0] + hb[1] + hb[2])) break;
            }
          }
          G(4, i, j, k) = ymin;
        }
    for (int k = 2; k <= km; ++k) for (int i = 2; i <= im; ++i) { G(4, i, 1, k) = G(4, i, 2, k); G(4, i, jm + 1, k) = G(4, i, jm, k); }
    for (int k = 2; k <= km; ++k) for (int j = 1; j <= jm + 1; ++j) { G(4, 1, j, k) = G(4, 2, j, k); G(4, im + 1, j, k) = G(4, im, j, k); }
    for (int j = 1; j <= jm + 1; ++j) for (int i = 1; i <= im + 1; ++i) { G(4, i, j, 1) = G(4, i, j, 2); G(4, i, j, km + 1) = G(4, i, j, km); }
  }
}

/* ---------------- BC descriptors (src/bc_module.f90:71-1188) ---------------- */
static void bc_reference_state(const Cfg& c, BcInfo& bi) {
  bi.pressure = c.pref;
  bi.pv[0] = c.pref;
  bi.pv[1] = c.uref * std::cos(c.aos) * std::cos(c.aoa);
  bi.pv[2] = c.uref * std::cos(c.aos) * std::sin(c.aoa);
  bi.pv[3] = c.uref * std::sin(c.aos);
  bi.pv[4] = c.tref; bi.pv[5] = c.y1ref; bi.pv[6] = c.y2ref;
  bi.tv[0] = bi.tv[1] = bi.tv[2] = 0.0;
  if (c.iturb >= -1) { bi.tv[2] = c.emutref; bi.pv[7] = c.kref; bi.pv[8] = c.oref; }
  deteos(c.eos, c.with_prop, bi.pressure, bi.pv[4], bi.pv[5], bi.pv[6], bi.dv, bi.tv);
}

static BcKind wall_kind(const Cfg& c) {
  if (c.iturb == 0) return K_WALL_KW;
  if (c.iturb == -1) return K_WALL_KE;   /* bcwallviscouske :2324-2366 */
  if (c.iturb == -2) return K_WALL_VISCOUS;
  return K_WALL_INVISCID;
}

static bool build_bcs(const Cfg& c, Block& B, const cfd3d_block_desc& d, std::string& err) {
  for (int n = 0; n < d.nbc; ++n) {
    const cfd3d_bc_patch& p = d.bc[n];
    BcInfo bi;
    bi.type = p.type;
    const int* ip = p.pnts;
    int axis = -1;
    for (int j = 0; j < 3; ++j) if (ip[j] == ip[3 + j]) { axis = j; }
    if (axis < 0) { err = "bc patch is not a face"; return false; }
    int nmax[3] = {B.imax, B.jmax, B.kmax};
    for (int j = 0; j < 3; ++j) {
      /* src/grid_module.f90:153-205: transverse ranges start one past the first node */
      if (j == axis) continue;
      bi.istart[j] = ip[j] + 1; bi.iend[j] = ip[3 + j];
    }
    bool mn = (ip[axis] == 1);
    if (!mn && ip[axis] != nmax[axis]) { err = "bc patch not on a block face"; return false; }
    bi.istart[axis] = mn ? 1 : ip[axis] + 1;
    bi.iend[axis] = bi.istart[axis];
    for (int q = 0; q < 3; ++q) { bi.dir[q] = 1; bi.origin[q] = 0; }
    bi.dir[axis] = -1;
    if (mn) { bi.istart[axis] -= 2; bi.origin[axis] = 2 * bi.iend[axis] + 1; }
    else { bi.iend[axis] += 2; bi.origin[axis] = 2 * bi.istart[axis] - 1; }
    bi.face = (Face)(2 * axis + (mn ? 0 : 1));
    switch (p.type) {
      case CFD3D_BC_WALL: bi.kind = wall_kind(c); break;
      /* the CounterRotating family (:3516-3810): the wall at rest while the grid turns */
      case CFD3D_BC_WALL_COUNTERROTATING:
        if (c.iturb == -1) { err = "counter-rotating walls under k-epsilon are not built"; return false; }
        bi.kind = (c.iturb == 0) ? K_CRWALL_KW : (c.iturb == -2 ? K_CRWALL : K_CRWALL_INV);
        break;
      case CFD3D_BC_WALL_HEATFLUX:   /* the HeatFlux family: bcheatfluxwallviscouskw :4184-4273 */
        if (c.iturb != 0) { err = "heat-flux walls need the SST model (iturb = 0)"; return false; }
        if (p.ndata < 1 || !p.tdata || !p.heatflux) { err = "heat-flux wall without its history"; return false; }
        bi.kind = K_HFWALL_KW;
        bi.tdata.assign(p.tdata, p.tdata + p.ndata);
        bi.heatflux.assign(p.heatflux, p.heatflux + p.ndata);
        break;
      case CFD3D_BC_MASSFLOWRATE_IN: bi.kind = K_MASSFLOW_IN; break;   /* bcmassflowratein :3812-4012 */
      case CFD3D_BC_TOTALPRESSURE_IN: bi.kind = K_TOTALP; break;       /* bctotalpressurein :3299-3514 */
      case CFD3D_BC_SHIFTED_PERIODIC: bi.kind = K_SHIFTED; break;      /* bcshiftedperiodic :3134-3297 */
      case CFD3D_BC_SYMMETRY: bi.kind = K_SYMMETRY; break;
      case CFD3D_BC_FARFIELD: bi.kind = K_FARFIELD; break;
      case CFD3D_BC_EXTRAPOLATE: case CFD3D_BC_DEGENERATE: bi.kind = K_EXTRAP; break;
      case CFD3D_BC_INFLOW: case CFD3D_BC_OUTFLOW: bi.kind = K_NOOP; break;   /* bcinflow, bcoutflow */
      case CFD3D_BC_INFLOW_SUBSONIC: bi.kind = K_INFLOW_SUB; break;    /* bcinflowsubsonic :2464-2640 */
      case CFD3D_BC_OUTFLOW_SUBSONIC: bi.kind = K_OUTFLOW_SUB; break;  /* bcoutflowsubsonic :2699-2869 */
      case CFD3D_BC_INFLOW_SUPERSONIC: bi.kind = K_INFLOW_SUP; break;  /* bcinflowsupersonic :2642-2678 */
      default: err = "unknown bc type"; return false;
    }
    if (bi.kind == K_SHIFTED && (bi.face == F_JMIN || bi.face == F_JMAX || bi.face == F_KMIN || bi.face == F_KMAX)) {
      /* the 16-cell sources must lie in the padded block */
      const int ax = (bi.face == F_JMIN || bi.face == F_JMAX) ? 1 : 2;
      const int nmx[3] = {B.imax, B.jmax, B.kmax};
      const bool lo = (bi.face == F_JMIN || bi.face == F_KMIN);
      const bool ok = lo ? (bi.iend[ax] + 16 <= nmx[ax] + 3 && bi.iend[0] <= B.imax + 3)
                         : (bi.istart[ax] - 16 >= -1 && bi.istart[0] >= -1);
      if (!ok) { err = "shifted periodic patch: the 16-cell source lies outside the block"; return false; }
    }
    bc_reference_state(c, bi);
    for (int q = 0; q < 6; ++q) for (int r = 0; r < 3; ++r) bi.nb[q][r] = 0;
    B.bcs.push_back(bi);
  }
  const int im = B.imax, jm = B.jmax, km = B.kmax;
  /* 12 edges (src/bc_module.f90:505-627) */
  struct ED { int is[3], ie[3], n1[3], n2[3], n3[3], o[3]; };
  const ED E[12] = {
      {{-1, -1, 2}, {1, 1, km}, {1, 2, 0}, {2, 1, 0}, {0, 0, 0}, {2, 2, 0}},
      {{im + 1, -1, 2}, {im + 3, 1, km}, {im + 1, 2, 0}, {im, 1, 0}, {0, 0, 0}, {im, 2, 0}},
      {{-1, jm + 1, 2}, {1, jm + 3, km}, {1, jm, 0}, {2, jm + 1, 0}, {0, 0, 0}, {2, jm, 0}},
      {{im + 1, jm + 1, 2}, {im + 3, jm + 3, km}, {im + 1, jm, 0}, {im, jm + 1, 0}, {0, 0, 0}, {im, jm, 0}},
      {{-1, 2, -1}, {1, jm, 1}, {1, 0, 2}, {0, 0, 0}, {2, 0, 1}, {2, 0, 2}},
      {{im + 1, 2, -1}, {im + 3, jm, 1}, {im + 1, 0, 2}, {0, 0, 0}, {im, 0, 1}, {im, 0, 2}},
      {{-1, 2, km + 1}, {1, jm, km + 3}, {1, 0, km}, {0, 0, 0}, {2, 0, km + 1}, {2, 0, km}},
      {{im + 1, 2, km + 1}, {im + 3, jm, km + 3}, {im + 1, 0, km}, {0, 0, 0}, {im, 0, km + 1}, {im, 0, km}},
      {{2, -1, -1}, {im, 1, 1}, {0, 0, 0}, {0, 1, 2}, {0, 2, 1}, {0, 2, 2}},
      {{2, jm + 1, -1}, {im, jm + 3, 1}, {0, 0, 0}, {0, jm + 1, 2}, {0, jm, 1}, {0, jm, 2}},
      {{2, -1, km + 1}, {im, 1, km + 3}, {0, 0, 0}, {0, 1, km}, {0, 2, km + 1}, {0, 2, km}},
      {{2, jm + 1, km + 1}, {im, jm + 3, km + 3}, {0, 0, 0}, {0, jm + 1, km}, {0, jm, km + 1}, {0, jm, km}},
  };
  auto is_surf = [&](const int* pnt, int a0, int a1) {
    for (auto& bc : B.bcs) {
      if (bc.type != CFD3D_BC_WALL && bc.type != CFD3D_BC_WALL_COUNTERROTATING && bc.type != CFD3D_BC_WALL_HEATFLUX &&
          bc.type != CFD3D_BC_SYMMETRY) continue;
      if (bc.istart[a0] <= pnt[a0] && bc.iend[a0] >= pnt[a0] && bc.istart[a1] <= pnt[a1] && bc.iend[a1] >= pnt[a1])
        return true;
    }
    return false;
  };
  for (int m = 0; m < 12; ++m) {
    BcInfo& e = B.edge[m];
    for (int q = 0; q < 3; ++q) {
      e.istart[q] = E[m].is[q]; e.iend[q] = E[m].ie[q]; e.origin[q] = E[m].o[q];
      e.nb[0][q] = E[m].n1[q]; e.nb[1][q] = E[m].n2[q]; e.nb[2][q] = E[m].n3[q];
      e.nb[3][q] = e.nb[4][q] = e.nb[5][q] = 0; e.dir[q] = 0;
    }
    bc_reference_state(c, e);
    bool s1 = false, s2 = false;
    /* isurf/jsurf/ksurf flags and the resulting edge type (src/bc_module.f90:651-865) */
    if (m < 4) { s1 = is_surf(e.nb[0], 0, 1); s2 = is_surf(e.nb[1], 0, 1); }
    else if (m < 8) { s1 = is_surf(e.nb[0], 0, 2); s2 = is_surf(e.nb[2], 0, 2); }
    else { s1 = is_surf(e.nb[1], 1, 2); s2 = is_surf(e.nb[2], 1, 2); }
    int along = (m < 4) ? 2 : ((m < 8) ? 1 : 0);
    if (s1 && s2) {
      e.kind = (c.iturb == 0) ? K_EDGE_WALLWALL_KW : K_EDGE_WALLWALL;
    } else if (s1 || s2) {
      e.kind = wall_kind(c);
      if (m < 4) {
        if (s1) { e.face = (m == 0 || m == 2) ? F_IMIN : F_IMAX; e.origin[0] = e.nb[1][0]; e.origin[1] = e.nb[1][1]; }
        else { e.face = (m == 0 || m == 1) ? F_JMIN : F_JMAX; e.origin[0] = e.nb[0][0]; e.origin[1] = e.nb[0][1]; }
      } else if (m < 8) {
        if (s1) { e.face = (m == 4 || m == 6) ? F_IMIN : F_IMAX; e.origin[0] = e.nb[2][0]; e.origin[2] = e.nb[2][2]; }
        else { e.face = (m == 4 || m == 5) ? F_KMIN : F_KMAX; e.origin[0] = e.nb[0][0]; e.origin[2] = e.nb[0][2]; }
      } else {
        if (s1) { e.face = (m == 8 || m == 10) ? F_JMIN : F_JMAX; e.origin[1] = e.nb[2][1]; e.origin[2] = e.nb[2][2]; }
        else { e.face = (m == 8 || m == 9) ? F_KMIN : F_KMAX; e.origin[1] = e.nb[1][1]; e.origin[2] = e.nb[1][2]; }
      }
    } else {
      e.kind = K_EDGE_NOWALL;
    }
    e.dir[along] = 1;
  }
  /* 8 corners (src/bc_module.f90:870-1186) */
  const int I1 = 1, I2 = 2, IA = im + 1, IB = im, J1 = 1, J2 = 2, JA = jm + 1, JB = jm, K1 = 1, K2 = 2, KA = km + 1, KB = km;
  struct CD { int r[3][2]; int n[6][3]; int o[3]; };
  auto mk = [&](int im0, int jm0, int km0) {
    /* im0/jm0/km0: 0 = min side, 1 = max side */
    CD d;
    int ilo = im0 ? im + 1 : -1, ihi = im0 ? im + 3 : 1;
    int jlo = jm0 ? jm + 1 : -1, jhi = jm0 ? jm + 3 : 1;
    int klo = km0 ? km + 1 : -1, khi = km0 ? km + 3 : 1;
    d.r[0][0] = ilo; d.r[0][1] = ihi; d.r[1][0] = jlo; d.r[1][1] = jhi; d.r[2][0] = klo; d.r[2][1] = khi;
    int gi = im0 ? IA : I1, ci = im0 ? IB : I2;
    int gj = jm0 ? JA : J1, cj = jm0 ? JB : J2;
    int gk = km0 ? KA : K1, ck = km0 ? KB : K2;
    int n1[3] = {gi, cj, ck}, n2[3] = {ci, gj, ck}, n3[3] = {ci, cj, gk};
    int n4[3] = {ci, gj, gk}, n5[3] = {gi, cj, gk}, n6[3] = {gi, gj, ck};
    for (int q = 0; q < 3; ++q) {
      d.n[0][q] = n1[q]; d.n[1][q] = n2[q]; d.n[2][q] = n3[q]; d.n[3][q] = n4[q]; d.n[4][q] = n5[q]; d.n[5][q] = n6[q];
    }
    d.o[0] = ci; d.o[1] = cj; d.o[2] = ck;
    return d;
  };
  const CD C8[8] = {mk(0, 0, 0), mk(1, 0, 0), mk(0, 1, 0), mk(1, 1, 0), mk(0, 0, 1), mk(1, 0, 1), mk(0, 1, 1), mk(1, 1, 1)};
  auto is_surf3 = [&](const int* pnt) {
    for (auto& bc : B.bcs) {
      if (bc.type != CFD3D_BC_WALL && bc.type != CFD3D_BC_WALL_COUNTERROTATING && bc.type != CFD3D_BC_WALL_HEATFLUX &&
          bc.type != CFD3D_BC_SYMMETRY) continue;
      bool in = true;
      for (int q = 0; q < 3; ++q) in = in && bc.istart[q] <= pnt[q] && bc.iend[q] >= pnt[q];
      if (in) return true;
    }
    return false;
  };
  for (int m = 0; m < 8; ++m) {
    BcInfo& e = B.corner[m];
    for (int q = 0; q < 3; ++q) {
      e.istart[q] = C8[m].r[q][0]; e.iend[q] = C8[m].r[q][1]; e.origin[q] = C8[m].o[q]; e.dir[q] = 0;
      for (int r = 0; r < 6; ++r) e.nb[r][q] = C8[m].n[r][q];
    }
    bc_reference_state(c, e);
    bool si = is_surf3(e.nb[0]), sj = is_surf3(e.nb[1]), sk = is_surf3(e.nb[2]);
    auto cp = [&](int dst, int src) { for (int q = 0; q < 3; ++q) e.nb[dst][q] = (src < 0) ? 0 : e.nb[src][q]; };
    auto org = [&](int src) { for (int q = 0; q < 3; ++q) e.origin[q] = e.nb[src][q]; };
    const BcKind ww = (c.iturb == 0) ? K_EDGE_WALLWALL_KW : K_EDGE_WALLWALL;
    if (si && sj && sk) {
      e.kind = (c.iturb == 0) ? K_CORNER_WALLWALL_KW : K_CORNER_WALLWALL;
    } else if (!si && sj && sk) {
      org(0); cp(0, -1); cp(1, 4); cp(2, 5); e.kind = ww;
    } else if (si && !sj && sk) {
      org(1); cp(0, 3); cp(1, -1); cp(2, 5); e.kind = ww;
    } else if (si && sj && !sk) {
      org(2); cp(0, 3); cp(1, 4); cp(2, -1); e.kind = ww;
    } else if (!si && !sj && sk) {
      /* the reference labels this face 'Kmin'/'Kmax' (capital K), which no face case
         matches (src/bc_module.f90:1121-1126) */
      e.face = (m < 4) ? F_KMIN_CAP : F_KMAX_CAP; org(5); e.kind = wall_kind(c);
    } else if (si && !sj && !sk) {
      e.face = (m % 2 == 0) ? F_IMIN : F_IMAX; org(3); e.kind = wall_kind(c);
    } else if (!si && sj && !sk) {
      e.face = (m == 0 || m == 1 || m == 4 || m == 5) ? F_JMIN : F_JMAX; org(4); e.kind = wall_kind(c);
    } else {
      e.kind = K_CORNER_NOWALL;
    }
    if ((e.face == F_KMIN_CAP || e.face == F_KMAX_CAP) && e.kind == K_WALL_INVISCID) {
      err = "corner with only a k-side wall under inviscid walls reads undefined data in the reference";
      return false;
    }
  }
  return true;
}

/* ---------------- connections (src/grid_module.f90:226-300, src/bc_module.f90:355-497) ---------------- */
static bool build_cons(Block& B, const cfd3d_block_desc& d, int nblocks, std::string& err) {
  for (int n = 0; n < d.ncon; ++n) {
    const cfd3d_connection& cc = d.con[n];
    if (cc.donor < 0 || cc.donor >= nblocks) { err = "bad donor"; return false; }
    Conn g;
    g.donor = cc.donor;
    for (int a = 0; a < 3; ++a) for (int b2 = 0; b2 < 3; ++b2) g.tm[a][b2] = 0;
    for (int q = 0; q < 3; ++q) {
      int tv = cc.transform[q];
      if (tv == 0 || std::abs(tv) > 3) { err = "bad transform"; return false; }
      g.tm[std::abs(tv) - 1][q] = tv / std::abs(tv);
    }
    const int* ip = cc.pnts;
    const int* id = cc.pnts_donor;
    for (int m = 0; m < 3; ++m) {
      if (ip[m] == ip[3 + m]) {
        if (ip[m] == 1) {
          for (int q = 0; q < 3; ++q) { g.istart[q] = ip[q]; g.iend[q] = ip[3 + q]; }
          g.istart[m] = ip[m] + 1; g.iend[m] = ip[3 + m] + 1;
        } else {
          for (int q = 0; q < 3; ++q) { g.istart[q] = ip[q]; g.iend[q] = ip[3 + q]; }
        }
      }
      if (id[m] == id[3 + m]) {
        for (int q = 0; q < 3; ++q) { g.istart_d[q] = id[q]; g.iend_d[q] = id[3 + q]; }
        if (id[m] != 1) { g.istart_d[m] = id[m] + 1; g.iend_d[m] = id[3 + m] + 1; }
      }
    }
    B.gcons.push_back(g);
  }
  return true;
}


/* map an own cell through a connection to the donor's cell */
static inline void conn_map(const Conn& g, int i, int j, int k, int& ii, int& jj, int& kk) {
  ii = g.tm[0][0] * (i - g.istart[0]) + g.tm[0][1] * (j - g.istart[1]) + g.tm[0][2] * (k - g.istart[2]) + g.istart_d[0];
  jj = g.tm[1][0] * (i - g.istart[0]) + g.tm[1][1] * (j - g.istart[1]) + g.tm[1][2] * (k - g.istart[2]) + g.istart_d[1];
  kk = g.tm[2][0] * (i - g.istart[0]) + g.tm[2][1] * (j - g.istart[1]) + g.tm[2][2] * (k - g.istart[2]) + g.istart_d[2];
}

/* face-vector halo of calnormal (src/grid_module.f90:725-918): the sender packs the two
   transverse face arrays of its own face axis, the receiver stores them with signs taken
   from the donor range orientation */
static void exchange_face_vectors(Oracle& O) {
  for (size_t bi = 0; bi < O.b.size(); ++bi) {
    Block& S = O.b[bi];
    for (auto& g : S.gcons) {
      Block& D = O.b[g.donor];
      int sign1 = 1, sign2 = 1;
      if (g.istart_d[0] == g.iend_d[0]) {
        if (g.istart_d[1] > g.iend_d[1]) sign1 = -sign1;
        if (g.istart_d[2] > g.iend_d[2]) sign2 = -sign2;
      } else if (g.istart_d[1] == g.iend_d[1]) {
        if (g.istart_d[2] > g.iend_d[2]) sign1 = -sign1;
        if (g.istart_d[0] > g.iend_d[0]) sign2 = -sign2;
      } else if (g.istart_d[2] == g.iend_d[2]) {
        if (g.istart_d[0] > g.iend_d[0]) sign1 = -sign1;
        if (g.istart_d[1] > g.iend_d[1]) sign2 = -sign2;
      }
      for (int k = g.istart[2]; k <= g.iend[2]; ++k)
        for (int j = g.istart[1]; j <= g.iend[1]; ++j)
          for (int i = g.istart[0]; i <= g.iend[0]; ++i) {
            int ii, jj, kk;
            conn_map(g, i, j, k, ii, jj, kk);
            for (int m = 0; m < 3; ++m) {
              double a, b2;
              if (g.istart[0] == g.iend[0]) { a = S.ex(m, i, j, k); b2 = S.tx(m, i, j, k); }
              else if (g.istart[1] == g.iend[1]) { a = S.tx(m, i, j, k); b2 = S.cx(m, i, j, k); }
              else { a = S.cx(m, i, j, k); b2 = S.ex(m, i, j, k); }
              if (g.istart_d[0] == g.iend_d[0]) { D.ex(m, ii, jj, kk) = sign1 * a; D.tx(m, ii, jj, kk) = sign2 * b2; }
              else if (g.istart_d[1] == g.iend_d[1]) { D.tx(m, ii, jj, kk) = sign1 * a; D.cx(m, ii, jj, kk) = sign2 * b2; }
              else { D.cx(m, ii, jj, kk) = sign1 * a; D.ex(m, ii, jj, kk) = sign2 * b2; }
            }
          }
    }
  }
}

/* "reodering" at the end of calnormal (src/grid_module.f90:926-940): transverse ranges
   move from node-based to cell-based */
static void reorder_cons(Oracle& O) {
  for (auto& B : O.b)
    for (auto& g : B.gcons)
      for (int m = 0; m < 3; ++m) {
        if (g.istart[m] != g.iend[m]) g.istart[m] += 1;
        if (g.istart_d[m] != g.iend_d[m]) {
          if (g.istart_d[m] < g.iend_d[m]) g.istart_d[m] += 1;
          else if (g.istart_d[m] > g.iend_d[m]) g.iend_d[m] += 1;
        }
      }
}

/* scalar metric halo: grd(var) of the own layer into the donor's ghost layer
   (calvolume :1115-1212 for the volume, calydns :525-606 for the wall distance) */
static void exchange_grd(Oracle& O, int var) {
  for (size_t bi = 0; bi < O.b.size(); ++bi) {
    Block& S = O.b[bi];
    for (auto& g : S.gcons) {
      Block& D = O.b[g.donor];
      for (int k = g.istart[2]; k <= g.iend[2]; ++k)
        for (int j = g.istart[1]; j <= g.iend[1]; ++j)
          for (int i = g.istart[0]; i <= g.iend[0]; ++i) {
            int ii, jj, kk;
            conn_map(g, i, j, k, ii, jj, kk);
            D.grd(var, ii, jj, kk) = S.grd(var, i, j, k);
          }
    }
  }
}

/* state-halo descriptors: 3 layers along the face normal (src/bc_module.f90:355-463) */
static bool build_state_halos(Oracle& O, std::string& err) {
  for (auto& B : O.b) {
    for (auto& g : B.gcons) {
      Conn s = g;
      int ax;
      if (s.istart[1] == s.iend[1]) ax = 1;
      else if (s.istart[0] == s.iend[0]) ax = 0;
      else if (s.istart[2] == s.iend[2]) ax = 2;
      else { err = "connection is not a face"; return false; }
      int row = -1, sgn = 0;
      for (int r = 0; r < 3; ++r) if (s.tm[r][ax] != 0) { row = r; sgn = s.tm[r][ax]; }
      if (row < 0) { err = "bad transform"; return false; }
      if (s.istart[ax] == 2) {
        s.iend[ax] += 2; s.face = 2 * ax + 1;
        s.iend_d[row] += 2 * sgn;
      } else {
        s.istart[ax] -= 2; s.face = 2 * ax + 2;
        s.istart_d[row] -= 2 * sgn;
      }
      B.cons.push_back(s);
    }
  }
  return true;
}

/* ---------------- BC application (src/bc_module.f90:1806-2902) ---------------- */
struct BcCtx { const Cfg& c; Block& B; };

static void put_cell(const Cfg& c, Block& B, int i, int j, int k, const double* pv, const double* dv, const double* tv) {
  double* P = B.pv.at(i, j, k);
  double* D = B.dv.at(i, j, k);
  for (int m = 0; m < c.npv; ++m) P[m] = pv[m];
  for (int m = 0; m < NDV; ++m) D[m] = dv[m];
  if (c.ntv) { double* T = B.tv.at(i, j, k); for (int m = 0; m < c.ntv; ++m) T[m] = tv[m]; }
}
static void get_cell(const Cfg& c, Block& B, int i, int j, int k, double* pv, double* dv, double* tv) {
  const double* P = B.pv.at(i, j, k);
  const double* D = B.dv.at(i, j, k);
  for (int m = 0; m < c.npv; ++m) pv[m] = P[m];
  for (int m = 0; m < NDV; ++m) dv[m] = D[m];
  for (int m = 0; m < 3; ++m) tv[m] = 0.0;
  if (c.ntv) { const double* T = B.tv.at(i, j, k); for (int m = 0; m < c.ntv; ++m) tv[m] = T[m]; }
}

/* boundary cell index and outward/inward face normal used by wall/symmetry/farfield */
static void face_cell(const BcInfo& bi, Block& B, int i, int j, int k, int& ii, int& jj, int& kk, double* nx,
                      bool farfield_sign) {
  /* symmetry/wall use +inward normal at min faces; farfield uses the opposite sign */
  double s = farfield_sign ? -1.0 : 1.0;
  switch (bi.face) {
    case F_IMIN: ii = bi.origin[0] + bi.dir[0] * bi.iend[0]; jj = bi.origin[1] + bi.dir[1] * j; kk = bi.origin[2] + bi.dir[2] * k;
      for (int v = 0; v < 3; ++v) nx[v] = s * B.cx(v, ii - 1, jj, kk); break;
    case F_IMAX: ii = bi.origin[0] + bi.dir[0] * bi.istart[0]; jj = bi.origin[1] + bi.dir[1] * j; kk = bi.origin[2] + bi.dir[2] * k;
      for (int v = 0; v < 3; ++v) nx[v] = -s * B.cx(v, ii, jj, kk); break;
    case F_JMIN: ii = bi.origin[0] + bi.dir[0] * i; jj = bi.origin[1] + bi.dir[1] * bi.iend[1]; kk = bi.origin[2] + bi.dir[2] * k;
      for (int v = 0; v < 3; ++v) nx[v] = s * B.ex(v, ii, jj - 1, kk); break;
    case F_JMAX: ii = bi.origin[0] + bi.dir[0] * i; jj = bi.origin[1] + bi.dir[1] * bi.istart[1]; kk = bi.origin[2] + bi.dir[2] * k;
      for (int v = 0; v < 3; ++v) nx[v] = -s * B.ex(v, ii, jj, kk); break;
    case F_KMIN: ii = bi.origin[0] + bi.dir[0] * i; jj = bi.origin[1] + bi.dir[1] * j; kk = bi.origin[2] + bi.dir[2] * bi.iend[2];
      for (int v = 0; v < 3; ++v) nx[v] = s * B.tx(v, ii, jj, kk - 1); break;
    case F_KMAX: ii = bi.origin[0] + bi.dir[0] * i; jj = bi.origin[1] + bi.dir[1] * j; kk = bi.origin[2] + bi.dir[2] * bi.istart[2];
      for (int v = 0; v < 3; ++v) nx[v] = -s * B.tx(v, ii, jj, kk); break;
    default: break;  /* 'Kmin'/'Kmax' corners: the indices keep their previous values */
  }
}

/* The grid velocity of a boundary face (gridvel of the counter-rotating walls, the
   mass-flow and total-pressure inlets): omega x r at the mean of the centroids of the
   boundary cell (ii, jj, kk) and the ghost cell across the face (e.g. :3539-3559). */
static void face_gridvel(const Cfg& c, Block& B, const BcInfo& bi, int ii, int jj, int kk, double* gv) {
  int gi = ii, gj = jj, gk = kk;
  switch (bi.face) {
    case F_IMIN: gi = ii - 1; break;
    case F_IMAX: gi = ii + 1; break;
    case F_JMIN: gj = jj - 1; break;
    case F_JMAX: gj = jj + 1; break;
    case F_KMIN: gk = kk - 1; break;
    case F_KMAX: gk = kk + 1; break;
    default: break;
  }
  double r[3];
  for (int e = 0; e < 3; ++e) r[e] = 0.5 * (B.grd(1 + e, ii, jj, kk) + B.grd(1 + e, gi, gj, gk));
  grid_vel(c, r, gv);
}

/* newt / funcv / fdjac / lnsrch / ludcmp / lubksb (src/bc_module.f90:4305-4622) for the
   total-pressure inlet, n = 2: as written, newt's fvec is evaluated once at its start */
struct TpSys { const Cfg* c; double uu, gam; };
static void tp_funcv(const TpSys& S, const double* x, double* f) {
  double dv[NDV];
  deteos_simple(S.c->eos, x[0], x[1], S.c->y1ref, S.c->y2ref, dv);
  f[0] = S.c->tp_pt - x[0] * std::pow(S.c->tp_tt / x[1], S.gam / (S.gam - 1.0));
  f[1] = S.c->tp_ht - (dv[1] + 0.5 * S.uu);
}
static double tp_fmin(const TpSys& S, const double* x, double* f) {
  tp_funcv(S, x, f);
  return 0.5 * (sq(f[0]) + sq(f[1]));
}
static void tp_ludcmp(double a[2][2], int* indx) {
  double vv[2];
  for (int i = 0; i < 2; ++i) { double aamax = 0.0; for (int j = 0; j < 2; ++j) aamax = dmax(aamax, std::fabs(a[i][j])); vv[i] = 1.0 / aamax; }
  for (int j = 0; j < 2; ++j) {
    for (int i = 0; i < j; ++i) { double sum = a[i][j]; for (int k = 0; k < i; ++k) sum -= a[i][k] * a[k][j]; a[i][j] = sum; }
    double aamax = 0.0; int imax = j;
    for (int i = j; i < 2; ++i) {
      double sum = a[i][j];
      for (int k = 0; k < j; ++k) sum -= a[i][k] * a[k][j];
      a[i][j] = sum;
      double dum = vv[i] * std::fabs(sum);
      if (dum >= aamax) { imax = i; aamax = dum; }
    }
    if (j != imax) { for (int k = 0; k < 2; ++k) std::swap(a[imax][k], a[j][k]); vv[imax] = vv[j]; }
    indx[j] = imax;
    if (a[j][j] == 0.0) a[j][j] = 1.0e-20;
    if (j != 1) { double dum = 1.0 / a[j][j]; for (int i = j + 1; i < 2; ++i) a[i][j] *= dum; }
  }
}
static void tp_lubksb(double a[2][2], const int* indx, double* b) {
  int ii = -1;
  for (int i = 0; i < 2; ++i) {
    int ll = indx[i]; double sum = b[ll]; b[ll] = b[i];
    if (ii >= 0) { for (int j = ii; j < i; ++j) sum -= a[i][j] * b[j]; }
    else if (sum != 0.0) ii = i;
    b[i] = sum;
  }
  for (int i = 1; i >= 0; --i) { double sum = b[i]; for (int j = i + 1; j < 2; ++j) sum -= a[i][j] * b[j]; b[i] = sum / a[i][i]; }
}
static void tp_newt(const TpSys& S, double* x) {
  const double tolf = 1.0e-4, tolx = 1.0e-7, stpmx = 100.0, alf = 1.0e-4;
  double fvec[2], fjac[2][2], g[2], p[2], xold[2];
  double f = tp_fmin(S, x, fvec);
  if (dmax(std::fabs(fvec[0]), std::fabs(fvec[1])) < 0.01 * tolf) return;
  double stpmax = stpmx * dmax(std::sqrt(sq(x[0]) + sq(x[1])), 2.0);
  for (int its = 1; its <= 200; ++its) {
    for (int j = 0; j < 2; ++j) {
      double temp[2] = {x[0], x[1]}, fj[2];
      double h = 1.0e-4 * std::fabs(temp[j]);
      if (h == 0.0) h = 1.0e-4;
      temp[j] = temp[j] + h;
      h = temp[j] - x[j];
      tp_funcv(S, temp, fj);
      for (int i = 0; i < 2; ++i) fjac[i][j] = (fj[i] - fvec[i]) / h;
    }
    for (int i = 0; i < 2; ++i) { double sum = 0.0; for (int j = 0; j < 2; ++j) sum += fjac[j][i] * fvec[j]; g[i] = sum; }
    xold[0] = x[0]; xold[1] = x[1];
    double fold = f;
    p[0] = -fvec[0]; p[1] = -fvec[1];
    int indx[2];
    tp_ludcmp(fjac, indx);
    tp_lubksb(fjac, indx, p);
    bool check = false;
    { /* lnsrch */
      double sum = std::sqrt(sq(p[0]) + sq(p[1]));
      if (sum > stpmax) for (int i = 0; i < 2; ++i) p[i] = p[i] * stpmax / sum;
      double slope = g[0] * p[0] + g[1] * p[1];
      double test = 0.0;
      for (int i = 0; i < 2; ++i) { double temp = std::fabs(p[i]) / dmax(std::fabs(xold[i]), 1.0); if (temp > test) test = temp; }
      double alamin = tolx / test, alam = 1.0, alam2 = 0.0, f2 = 0.0, fold2 = 0.0, tmplam = 0.0;
      for (;;) {
        for (int i = 0; i < 2; ++i) x[i] = xold[i] + alam * p[i];
        double fl[2];
        f = tp_fmin(S, x, fl);
        if (alam < alamin) { x[0] = xold[0]; x[1] = xold[1]; check = true; break; }
        if (f <= fold + alf * alam * slope) break;
        if (alam == 1.0) tmplam = -slope / (2.0 * (f - fold - slope));
        else {
          double rhs1 = f - fold - alam * slope, rhs2 = f2 - fold2 - alam2 * slope;
          double a = (rhs1 / sq(alam) - rhs2 / sq(alam2)) / (alam - alam2);
          double b = (-alam2 * rhs1 / sq(alam) + alam * rhs2 / sq(alam2)) / (alam - alam2);
          if (a == 0.0) tmplam = -slope / (2.0 * b);
          else {
            double disc = b * b - 3.0 * a * slope;
            if (disc < 0.0) tmplam = 0.5 * alam;
            else if (b <= 0.0) tmplam = (-b + std::sqrt(disc)) / (3.0 * a);
            else tmplam = -slope / (b + std::sqrt(disc));
          }
          if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
        }
        alam2 = alam; f2 = f; fold2 = fold;
        alam = dmax(tmplam, 0.1 * alam);
      }
    }
    if (dmax(std::fabs(fvec[0]), std::fabs(fvec[1])) < tolf) return;
    if (check) return;
    double test = 0.0;
    for (int i = 0; i < 2; ++i) { double temp = std::fabs(x[i] - xold[i]) / dmax(std::fabs(x[i]), 1.0); if (temp > test) test = temp; }
    if (test < tolx) return;
  }
}

/* one total-pressure patch's area-weighted sums over its boundary faces (:3320-3409):
   pa[0..4] += pv(1..5) dl, the velocities with the grid velocity added, pa[5] += dl */
static void tp_patch_sums(const Cfg& c, const Block& B, const BcInfo& bi, double* pa) {
  double nx[3];
  const int ax = (int)bi.face / 2;
  for (int k = bi.istart[2]; k <= bi.iend[2]; ++k)
    for (int j = bi.istart[1]; j <= bi.iend[1]; ++j)
      for (int i = bi.istart[0]; i <= bi.iend[0]; ++i) {
        const int idx[3] = {i, j, k};
        if (idx[ax] != (((int)bi.face % 2 == 0) ? bi.istart[ax] : bi.iend[ax])) continue;
        int ii = 0, jj = 0, kk = 0;
        face_cell(bi, const_cast<Block&>(B), i, j, k, ii, jj, kk, nx, true);
        const double dl = std::sqrt(sq(nx[0]) + sq(nx[1]) + sq(nx[2]));
        const double* P = const_cast<Block&>(B).pv.at(ii, jj, kk);
        double gv[3];
        face_gridvel(c, const_cast<Block&>(B), bi, ii, jj, kk, gv);
        pa[0] += P[0] * dl;
        pa[4] += P[4] * dl;
        for (int m = 1; m <= 3; ++m) pa[m] += (P[m] + gv[m - 1]) * dl;
        pa[5] += dl;
      }
}

/* The reference reduces the sums over bc_comm_world (mpi_reduce + mpi_bcast, :3411-3416),
   the communicator of every rank that carries a total-pressure inlet (icolor 12, :321,349),
   and each rank's n-th inlet meets the others' n-th in the collective.  So pool n holds the
   n-th total-pressure patch of every block; its averages feed one newt, whose solution all
   of the pool's patches take. */
static void tp_solve_pools(Oracle& O);
static void calvfg_block(Block& B);
static void exchange_vfg(Oracle& O);

static void apply_bc(const Cfg& c, Block& B, const BcInfo& bi) {
  double pv[NPV_MAX], dv[NDV], tv[3], pvs[NPV_MAX], dvs[NDV], tvs[3], ppv[NPV_MAX], nx[3];
  const double* tpx = bi.tpx;
  const double tpuu = bi.tpuu;
  for (int k = bi.istart[2]; k <= bi.iend[2]; ++k)
    for (int j = bi.istart[1]; j <= bi.iend[1]; ++j)
      for (int i = bi.istart[0]; i <= bi.iend[0]; ++i) {
        int mi = bi.origin[0] + bi.dir[0] * i, mj = bi.origin[1] + bi.dir[1] * j, mk = bi.origin[2] + bi.dir[2] * k;
        switch (bi.kind) {
          case K_NOOP: break;
          case K_HFWALL_KW: {
            /* heat flux of the history at bcinfo%time (:4196-4203; the first value before
               the first time, where the routine leaves it undefined) */
            const int nd = (int)bi.tdata.size();
            double hf = bi.heatflux[0];
            for (int m = 0; m < nd - 1; ++m)
              if (bi.time >= bi.tdata[m] && bi.time < bi.tdata[m + 1]) {
                hf = bi.heatflux[m] + (bi.heatflux[m + 1] - bi.heatflux[m]) * (bi.time - bi.tdata[m]) / (bi.tdata[m + 1] - bi.tdata[m]);
                break;
              }
            if (bi.time >= bi.tdata[nd - 1]) hf = bi.heatflux[nd - 1];
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            int ii = mi, jj = mj, kk = mk;
            face_cell(bi, B, i, j, k, ii, jj, kk, nx, false);
            const double* Pb = B.pv.at(ii, jj, kk);
            const double yb = B.grd(4, ii, jj, kk), mub = B.tv(0, ii, jj, kk), kb = B.tv(1, ii, jj, kk);
            const double rb = B.dv(0, ii, jj, kk);
            /* the routine's EOS call takes the mirror's state: the ghost keeps its dv, tv(1:2) */
            pv[1] = -pv[1]; pv[2] = -pv[2]; pv[3] = -pv[3]; pv[7] = -pv[7];
            pv[4] = 2.0 * ((hf * yb + 0.5 * mub * (sq(Pb[1]) + sq(Pb[2]) + sq(Pb[3]))) / kb + Pb[4]) - pv[4];
            pv[8] = 1600.0 * mub / rb / sq(yb) - pv[8];
            tv[2] = -tv[2];
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_WALL_KE:
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            pv[1] = -pv[1]; pv[2] = -pv[2]; pv[3] = -pv[3]; pv[7] = -pv[7]; pv[8] = -pv[8];
            tv[2] = -tv[2];
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          case K_TOTALP: {
            int ii = 0, jj = 0, kk = 0;
            face_cell(bi, B, i, j, k, ii, jj, kk, nx, true);
            const double dl = 1.0 / std::sqrt(sq(nx[0]) + sq(nx[1]) + sq(nx[2]));
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            double gv[3];
            face_gridvel(c, B, bi, ii, jj, kk, gv);
            pv[0] = 2.0 * (tpx[0] - bi.pv[0]) - pv[0];
            for (int q = 0; q < 3; ++q) pv[1 + q] = 2.0 * (-std::sqrt(tpuu) * nx[q] * dl - gv[q]) - pv[1 + q];
            pv[4] = 2.0 * tpx[1] - pv[4];
            for (int m = 5; m < c.npv; ++m) pv[m] = 2.0 * bi.pv[m] - pv[m];
            pv[6] = 2.0 * bi.pv[6] - pv[6];
            pv[5] = dmin(dmax(pv[5], 0.0), 1.0);
            pv[6] = dmin(dmax(pv[6], 0.0), 1.0);
            deteos(c.eos, c.with_prop, pv[0] + bi.pv[0], pv[4], pv[5], pv[6], dv, tv);
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_CRWALL:
          case K_CRWALL_KW: {
            /* bccounterrotatingwallviscous (:3516-3580) and its k-omega variant (:3654-3731):
               u = -u_mirror - 2 gridvel; k-omega: k and mu_t reflected, omega the mirror's
               (the routine computes the wall value and discards it) */
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            int ii = mi, jj = mj, kk = mk;
            face_cell(bi, B, i, j, k, ii, jj, kk, nx, false);
            double gv[3];
            face_gridvel(c, B, bi, ii, jj, kk, gv);
            for (int q = 0; q < 3; ++q) pv[1 + q] = -pv[1 + q] - 2.0 * gv[q];
            if (bi.kind == K_CRWALL_KW) { pv[7] = -pv[7]; tv[2] = -tv[2]; }
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_CRWALL_INV: {
            /* bccounterrotatingwallinviscid (:3733-3810): the symmetry reflection of the
               boundary cell's velocity less the grid velocity */
            int ii = 0, jj = 0, kk = 0;
            face_cell(bi, B, i, j, k, ii, jj, kk, nx, false);
            const double* P = B.pv.at(ii, jj, kk);
            for (int m = 0; m < c.npv; ++m) pvs[m] = P[m];
            double gv[3];
            face_gridvel(c, B, bi, ii, jj, kk, gv);
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            double v3[3];
            for (int q = 0; q < 3; ++q)
              v3[q] = 2.0 * (pvs[1 + q] - nx[q] * (pvs[1] * nx[0] + pvs[2] * nx[1] + pvs[3] * nx[2]) /
                                              (sq(nx[0]) + sq(nx[1]) + sq(nx[2])) - gv[q]) - pv[1 + q];
            pv[1] = v3[0]; pv[2] = v3[1]; pv[3] = v3[2];
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_MASSFLOW_IN: {
            /* massflowrate = 0 (construct): v = 0, so u = 2 (0 - gridvel) - u_mirror; p stays
               the mirror's */
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            int ii = mi, jj = mj, kk = mk;
            face_cell(bi, B, i, j, k, ii, jj, kk, nx, false);
            double gv[3];
            face_gridvel(c, B, bi, ii, jj, kk, gv);
            for (int q = 0; q < 3; ++q) pv[1 + q] = 2.0 * (0.0 - gv[q]) - pv[1 + q];
            for (int m = 4; m < c.npv; ++m) pv[m] = 2.0 * bi.pv[m] - pv[m];
            pv[5] = dmin(dmax(pv[5], 0.0), 1.0);
            pv[6] = dmin(dmax(pv[6], 0.0), 1.0);
            deteos(c.eos, c.with_prop, pv[0] + bi.pv[0], pv[4], pv[5], pv[6], dv, tv);
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_SHIFTED: {
            /* j / k faces: from (i +- 16, j +- 16, k) or (i +- 16, j, k +- 16); the last 16
               cells along i from the mirror; i faces untouched */
            if (bi.face == F_IMIN || bi.face == F_IMAX) break;
            const bool lo = (bi.face == F_JMIN || bi.face == F_KMIN);
            int si = mi, sj = mj, sk = mk;
            if (lo ? (i <= bi.iend[0] - 16) : (i >= bi.istart[0] + 16)) {
              const int di = lo ? 16 : -16;
              si = i + di; sj = j; sk = k;
              if (bi.face == F_JMIN || bi.face == F_JMAX) sj = j + di;
              else sk = k + di;
            }
            get_cell(c, B, si, sj, sk, pv, dv, tv);
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_EXTRAP:
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          case K_WALL_VISCOUS:
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            pv[1] = -pv[1]; pv[2] = -pv[2]; pv[3] = -pv[3];
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          case K_WALL_KW: {
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            int ii = mi, jj = mj, kk = mk;
            face_cell(bi, B, i, j, k, ii, jj, kk, nx, false);
            const double* dvb = B.dv.at(ii, jj, kk);
            const double* tvb = B.tv.at(ii, jj, kk);
            double y5 = B.grd(4, ii, jj, kk);
            double om = 1600.0 * tvb[0] / dvb[0] / sq(y5) - pv[8];
            pv[1] = -pv[1]; pv[2] = -pv[2]; pv[3] = -pv[3]; pv[7] = -pv[7]; pv[8] = om;
            tv[2] = -tv[2];
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_WALL_INVISCID:
          case K_SYMMETRY: {
            int ii = 0, jj = 0, kk = 0;
            face_cell(bi, B, i, j, k, ii, jj, kk, nx, false);
            const double* P = B.pv.at(ii, jj, kk);
            for (int m = 0; m < c.npv; ++m) pvs[m] = P[m];
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            double un = (pvs[1] * nx[0] + pvs[2] * nx[1] + pvs[3] * nx[2]) / (sq(nx[0]) + sq(nx[1]) + sq(nx[2]));
            double v1 = 2.0 * (pvs[1] - nx[0] * (pvs[1] * nx[0] + pvs[2] * nx[1] + pvs[3] * nx[2]) / (sq(nx[0]) + sq(nx[1]) + sq(nx[2]))) - pv[1];
            double v2 = 2.0 * (pvs[2] - nx[1] * (pvs[1] * nx[0] + pvs[2] * nx[1] + pvs[3] * nx[2]) / (sq(nx[0]) + sq(nx[1]) + sq(nx[2]))) - pv[2];
            double v3 = 2.0 * (pvs[3] - nx[2] * (pvs[1] * nx[0] + pvs[2] * nx[1] + pvs[3] * nx[2]) / (sq(nx[0]) + sq(nx[1]) + sq(nx[2]))) - pv[3];
            (void)un;
            pv[1] = v1; pv[2] = v2; pv[3] = v3;
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_FARFIELD:
          case K_INFLOW_SUB:
          case K_OUTFLOW_SUB:
          case K_INFLOW_SUP: {
            int ii = 0, jj = 0, kk = 0;
            face_cell(bi, B, i, j, k, ii, jj, kk, nx, true);
            const double* Pb = B.pv.at(ii, jj, kk);
            const double* Db = B.dv.at(ii, jj, kk);
            for (int m = 0; m < c.npv; ++m) pvs[m] = Pb[m];
            for (int m = 0; m < NDV; ++m) dvs[m] = Db[m];
            double dl = 1.0 / std::sqrt(sq(nx[0]) + sq(nx[1]) + sq(nx[2]));
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            double vel = (pvs[1] * nx[0] + pvs[2] * nx[1] + pvs[3] * nx[2]) * dl;
            double mach = vel / std::sqrt(dvs[5]);
            double a = std::sqrt(sndp2_of(c, dvs[5], sq(vel)));
            /* the dedicated BCs are the farfield branch of their name, whatever the Mach number */
            if (bi.kind == K_OUTFLOW_SUB) mach = 0.0;
            else if (bi.kind == K_INFLOW_SUP) mach = -1.0;
            else if (bi.kind == K_INFLOW_SUB) mach = -0.5;
            if (mach >= 0.0) {
              if (mach < 1.0) {
                pv[0] = 2.0 * (bi.pressure - bi.pv[0]) - pv[0];
                for (int q = 0; q < 3; ++q)
                  pv[1 + q] = 2.0 * (pvs[1 + q] + nx[q] * (pvs[0] + bi.pv[0] - bi.pressure) / dvs[0] / a * dl) - pv[1 + q];
              }
            } else {
              if (mach <= -1.0) {
                pv[0] = 2.0 * (bi.pressure - bi.pv[0]) - pv[0];
                for (int m = 1; m < c.npv; ++m) pv[m] = 2.0 * bi.pv[m] - pv[m];
                pv[5] = dmin(dmax(pv[5], 0.0), 1.0);
                pv[6] = dmin(dmax(pv[6], 0.0), 1.0);
              } else {
                double var = bi.pressure - bi.pv[0] + pvs[0] -
                             dvs[0] * a * (nx[0] * (bi.pv[1] - pvs[1]) + nx[1] * (bi.pv[2] - pvs[2]) + nx[2] * (bi.pv[3] - pvs[3])) * dl;
                pv[0] = var - pv[0];
                for (int q = 0; q < 3; ++q) pv[1 + q] = 2.0 * (bi.pv[1 + q] + nx[q] * 0.5 * var / dvs[0] / a * dl) - pv[1 + q];
                for (int m = 4; m < c.npv; ++m) pv[m] = 2.0 * bi.pv[m] - pv[m];
                pv[5] = dmin(dmax(pv[5], 0.0), 1.0);
                pv[6] = dmin(dmax(pv[6], 0.0), 1.0);
              }
            }
            deteos(c.eos, c.with_prop, pv[0] + bi.pv[0], pv[4], pv[5], pv[6], dv, tv);
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_EDGE_WALLWALL:
          case K_EDGE_WALLWALL_KW:
          case K_CORNER_WALLWALL:
          case K_CORNER_WALLWALL_KW: {
            get_cell(c, B, mi, mj, mk, pv, dv, tv);
            for (int m = 0; m < c.npv; ++m) ppv[m] = -pv[m];
            double var = 0.0;
            if (bi.kind == K_EDGE_WALLWALL_KW || bi.kind == K_CORNER_WALLWALL_KW)
              var = 800.0 * tv[0] / dv[0] / sq(B.grd(4, mi, mj, mk));
            int nn = (bi.kind == K_CORNER_WALLWALL || bi.kind == K_CORNER_WALLWALL_KW) ? 6 : 3;
            for (int q = 0; q < nn; ++q) {
              const int* nb = bi.nb[q];
              if (nn == 3 && nb[0] == 0 && nb[1] == 0 && nb[2] == 0) continue;
              const double* P = B.pv.at(nb[0] + bi.dir[0] * i, nb[1] + bi.dir[1] * j, nb[2] + bi.dir[2] * k);
              for (int m = 0; m < c.npv; ++m) ppv[m] = ppv[m] - P[m];
            }
            if (bi.kind == K_EDGE_WALLWALL || bi.kind == K_CORNER_WALLWALL) {
              for (int m = 1; m <= 3; ++m) pv[m] = ppv[m];
              if (c.npv > 7) { pv[7] = ppv[7]; pv[8] = ppv[8]; }
            } else {
              /* edgewallwallkw: omega = 4*var + ppv(9); cornerwallwallkw handled alike */
              for (int m = 1; m <= 3; ++m) pv[m] = ppv[m];
              pv[7] = ppv[7];
              pv[8] = ((bi.kind == K_CORNER_WALLWALL_KW) ? 8.0 : 4.0) * var + ppv[8];
            }
            put_cell(c, B, i, j, k, pv, dv, tv);
            break;
          }
          case K_EDGE_NOWALL:
          case K_CORNER_NOWALL: {
            const double* P = B.pv.at(mi, mj, mk);
            double acc[NPV_MAX], tacc[3] = {0, 0, 0};
            for (int m = 0; m < c.npv; ++m) acc[m] = P[m];
            if (c.ntv) { const double* T = B.tv.at(mi, mj, mk); for (int m = 0; m < c.ntv; ++m) tacc[m] = T[m]; }
            int nn = (bi.kind == K_CORNER_NOWALL) ? 6 : 3;
            int cnt = 1;
            for (int q = 0; q < nn; ++q) {
              const int* nb = bi.nb[q];
              if (bi.kind == K_EDGE_NOWALL && nb[0] == 0 && nb[1] == 0 && nb[2] == 0) continue;
              int a = nb[0] + bi.dir[0] * i, b2 = nb[1] + bi.dir[1] * j, c2 = nb[2] + bi.dir[2] * k;
              const double* Q = B.pv.at(a, b2, c2);
              for (int m = 0; m < c.npv; ++m) acc[m] = acc[m] + Q[m];
              if (c.ntv) { const double* T = B.tv.at(a, b2, c2); for (int m = 0; m < c.ntv; ++m) tacc[m] = tacc[m] + T[m]; }
              ++cnt;
            }
            double f = (bi.kind == K_CORNER_NOWALL) ? 1.0 / 7.0 : 1.0 / 3.0;
            for (int m = 0; m < c.npv; ++m) pv[m] = f * acc[m];
            for (int m = 0; m < 3; ++m) tv[m] = f * tacc[m];
            deteos(c.eos, c.with_prop, pv[0] + bi.pv[0], pv[4], pv[5], pv[6], dv, tv);
            put_cell(c, B, i, j, k, pv, dv, tv);
            (void)cnt;
            break;
          }
        }
      }
}

/* state halos: own slab -> donor ghosts (src/bc_module.f90:1254-1386) */
static void apply_halos(Oracle& O) {
  const Cfg& c = O.c;
  for (size_t bi = 0; bi < O.b.size(); ++bi) {
    Block& S = O.b[bi];
    for (auto& g : S.cons) {
      Block& D = O.b[g.donor];
      for (int k = g.istart[2]; k <= g.iend[2]; ++k)
        for (int j = g.istart[1]; j <= g.iend[1]; ++j)
          for (int i = g.istart[0]; i <= g.iend[0]; ++i) {
            int ii = g.tm[0][0] * (i - g.istart[0]) + g.tm[0][1] * (j - g.istart[1]) + g.tm[0][2] * (k - g.istart[2]) + g.istart_d[0];
            int jj = g.tm[1][0] * (i - g.istart[0]) + g.tm[1][1] * (j - g.istart[1]) + g.tm[1][2] * (k - g.istart[2]) + g.istart_d[1];
            int kk = g.tm[2][0] * (i - g.istart[0]) + g.tm[2][1] * (j - g.istart[1]) + g.tm[2][2] * (k - g.istart[2]) + g.istart_d[2];
            double pv[NPV_MAX], dv[NDV], tv[3];
            get_cell(c, S, i, j, k, pv, dv, tv);
            put_cell(c, D, ii, jj, kk, pv, dv, tv);
          }
    }
  }
}

static void tp_solve_pools(Oracle& O) {
  std::vector<std::vector<double>> sums;
  for (auto& B : O.b) {
    size_t n = 0;
    for (auto& bc : B.bcs) {
      if (bc.kind != K_TOTALP) continue;
      if (sums.size() <= n) sums.emplace_back(6, 0.0);
      tp_patch_sums(O.c, B, bc, sums[n].data());
      ++n;
    }
  }
  std::vector<double> x(2 * sums.size()), uu(sums.size());
  for (size_t n = 0; n < sums.size(); ++n) {
    double pa[5];
    for (int m = 0; m < 5; ++m) pa[m] = sums[n][m] / sums[n][5];
    TpSys S{&O.c, sq(pa[1]) + sq(pa[2]) + sq(pa[3]), (1.0 - O.c.y2ref) * 1.33 + O.c.y2ref * 1.4};
    x[2 * n] = pa[0] + O.c.pref;
    x[2 * n + 1] = pa[4];
    uu[n] = S.uu;
    tp_newt(S, &x[2 * n]);
  }
  for (auto& B : O.b) {
    size_t n = 0;
    for (auto& bc : B.bcs) {
      if (bc.kind != K_TOTALP) continue;
      bc.tpx[0] = x[2 * n]; bc.tpx[1] = x[2 * n + 1]; bc.tpuu = uu[n];
      ++n;
    }
  }
}

static void setbc(Oracle& O) {
  tp_solve_pools(O);
  for (auto& B : O.b) for (auto& bc : B.bcs) { bc.time = O.time_cur; apply_bc(O.c, B, bc); }
  apply_halos(O);
  for (auto& B : O.b) for (int m = 0; m < 12; ++m) apply_bc(O.c, B, B.edge[m]);
  for (auto& B : O.b) for (int m = 0; m < 8; ++m) apply_bc(O.c, B, B.corner[m]);
  /* with the surface-tension source every setbc is followed by calvfg and setbc_vfg
     (src/update_module.f90:240-243, 359-362, 479-482) */
  if (O.c.csf) {
    for (auto& B : O.b) calvfg_block(B);
    exchange_vfg(O);
  }
}

/* ---------------- local time step (src/timestep_module.f90:127-316) ---------------- */
static double timestep_block(const Cfg& c, Block& B) {
  double dtmin = 1.0e10;
  for (int k = 2; k <= B.kmax; ++k)
    for (int j = 2; j <= B.jmax; ++j)
      for (int i = 2; i <= B.imax; ++i) {
        if (c.local == -1) { B.dt(0, i, j, k) = c.cfl; continue; }
        const double* pv = B.pv.at(i, j, k);
        const double* dv = B.dv.at(i, j, k);
        double tv[3] = {0, 0, 0};
        if (c.ntv) for (int m = 0; m < c.ntv; ++m) tv[m] = B.tv(m, i, j, k);
        const double* grd = B.grd.at(i, j, k);
        double c1 = 0.5 * (B.cx(0, i - 1, j, k) + B.cx(0, i, j, k)), c2 = 0.5 * (B.cx(1, i - 1, j, k) + B.cx(1, i, j, k)),
               c3 = 0.5 * (B.cx(2, i - 1, j, k) + B.cx(2, i, j, k));
        double e1 = 0.5 * (B.ex(0, i, j - 1, k) + B.ex(0, i, j, k)), e2 = 0.5 * (B.ex(1, i, j - 1, k) + B.ex(1, i, j, k)),
               e3 = 0.5 * (B.ex(2, i, j - 1, k) + B.ex(2, i, j, k));
        double t1 = 0.5 * (B.tx(0, i, j, k - 1) + B.tx(0, i, j, k)), t2 = 0.5 * (B.tx(1, i, j, k - 1) + B.tx(1, i, j, k)),
               t3 = 0.5 * (B.tx(2, i, j, k - 1) + B.tx(2, i, j, k));
        double uc = std::fabs(c1 * pv[1] + c2 * pv[2] + c3 * pv[3]);
        double vc = std::fabs(e1 * pv[1] + e2 * pv[2] + e3 * pv[3]);
        double wc = std::fabs(t1 * pv[1] + t2 * pv[2] + t3 * pv[3]);
        double s1 = sq(c1) + sq(c2) + sq(c3), s2 = sq(e1) + sq(e2) + sq(e3), s3 = sq(t1) + sq(t2) + sq(t3);
        double uv2 = sq(pv[1]) + sq(pv[2]) + sq(pv[3]);
        double sndp2 = sndp2_of(c, dv[5], uv2);
        double up = uc * (1.0 + sndp2 / dv[5]);
        double d = std::sqrt(sq(uc) * sq(1.0 - sndp2 / dv[5]) + 4.0 * sndp2 * s1);
        double eigx = 0.5 * (up + d);
        up = vc * (1.0 + sndp2 / dv[5]);
        d = std::sqrt(sq(vc) * sq(1.0 - sndp2 / dv[5]) + 4.0 * sndp2 * s2);
        double eigy = 0.5 * (up + d);
        up = wc * (1.0 + sndp2 / dv[5]);
        d = std::sqrt(sq(wc) * sq(1.0 - sndp2 / dv[5]) + 4.0 * sndp2 * s3);
        double eigz = 0.5 * (up + d);
        double ev = eigenvis_of(c, dv, tv) * (s1 + s2 + s3) / grd[0];
        double dt = c.cfl * grd[0] / (eigx + eigy + eigz + 4.0 * ev);
        B.dt(0, i, j, k) = dt;
        if (dtmin >= dt) dtmin = dt;
      }
  return (c.local == -1) ? c.cfl : dtmin;
}

/* ---------------- RHS (src/rhs_module.f90:260-643) ---------------- */
static void gather_pv(const Cfg& c, Block& B, int i, int j, int k, double* out) {
  const double* P = B.pv.at(i, j, k);
  for (int m = 0; m < c.npv; ++m) out[m] = P[m];
}

/* ---------------- surface tension (csf = 1) ---------------- */
/* calvfg (src/variable_module.f90:304-351): vf = rho (y1 / rho_v + y2 / rho_g), the volume
   fraction of vapour and gas, over 0..imax+2, and its Green-Gauss gradient calgrad_gg
   (:353-377) over the cells 1..imax+1, the interior and the first ghost layer.  For the
   ghost layer the reference reads face vectors past the ends of its arrays (cx(0),
   cx(imax+1), ex(.,0,.), ex(.,jmax+1,.), tx(.,.,0), tx(.,.,kmax+1)), which hold no defined
   values; here such a face takes the vector of the nearest face of its row. */
static void calvfg_block(Block& B) {
  const int im = B.imax, jm = B.jmax, km = B.kmax;
  A4 vf;
  vf.init(1, 0, im + 2, 0, jm + 2, 0, km + 2);
  for (int k = 0; k <= km + 2; ++k)
    for (int j = 0; j <= jm + 2; ++j)
      for (int i = 0; i <= im + 2; ++i)
        vf(0, i, j, k) = B.dv(0, i, j, k) * (B.pv(5, i, j, k) / B.dv(3, i, j, k) + B.pv(6, i, j, k) / B.dv(4, i, j, k));
  auto clampi = [](int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); };
  for (int k = 1; k <= km + 1; ++k)
    for (int j = 1; j <= jm + 1; ++j)
      for (int i = 1; i <= im + 1; ++i) {
        const double x[7] = {vf(0, i - 1, j, k), vf(0, i + 1, j, k), vf(0, i, j - 1, k), vf(0, i, j + 1, k),
                             vf(0, i, j, k - 1), vf(0, i, j, k + 1), vf(0, i, j, k)};
        const double* n6[6] = {B.cx.at(clampi(i - 1, 1, im), j, k), B.cx.at(clampi(i, 1, im), j, k),
                               B.ex.at(i, clampi(j - 1, 1, jm), k), B.ex.at(i, clampi(j, 1, jm), k),
                               B.tx.at(i, j, clampi(k - 1, 1, km)), B.tx.at(i, j, clampi(k, 1, km))};
        const double sg[6] = {-1.0, 1.0, -1.0, 1.0, -1.0, 1.0};
        double g[3] = {0.0, 0.0, 0.0};
        for (int l = 0; l < 6; ++l) {
          const double xm = 0.5 * (x[6] + x[l]);
          for (int e = 0; e < 3; ++e) g[e] = g[e] + xm * (sg[l] * n6[l][e]);
        }
        for (int e = 0; e < 3; ++e) B.vfg(e, i, j, k) = g[e] / B.grd(0, i, j, k);
      }
}

/* setbc_vfg (src/bc_module.f90:1398-1804): across each 1-to-1 interface the donor's first
   ghost layer takes the block's first interior layer of vfg */
static void exchange_vfg(Oracle& O) {
  for (size_t bi = 0; bi < O.b.size(); ++bi) {
    Block& S = O.b[bi];
    for (auto& g : S.gcons) {
      Block& D = O.b[g.donor];
      for (int k = g.istart[2]; k <= g.iend[2]; ++k)
        for (int j = g.istart[1]; j <= g.iend[1]; ++j)
          for (int i = g.istart[0]; i <= g.iend[0]; ++i) {
            int ii, jj, kk;
            conn_map(g, i, j, k, ii, jj, kk);
            for (int e = 0; e < 3; ++e) D.vfg(e, ii, jj, kk) = S.vfg(e, i, j, k);
          }
    }
  }
}

/* csfsource (src/csf_module.f90:97-175) for cell (i, j, k), as calrhs calls it
   (src/rhs_module.f90:607-635): the cell (7) and its six neighbours' vfg, the outward face
   vectors -cx(i-1), cx(i), -ex(j-1), ex(j), -tx(k-1), tx(k).  Below |vfg| = 0.04 there is no
   interface and the source is zero.  The surface tension is the reference's constant
   0.071684196047 N/m in every cell, so its tangential (Marangoni) part, which is made of
   its differences, is zero. */
static void csf_source(Block& B, int i, int j, int k, const double* grd, const double* pv7, double* out) {
  for (int n = 0; n < 5; ++n) out[n] = 0.0;
  const double* v[7] = {B.vfg.at(i - 1, j, k), B.vfg.at(i + 1, j, k), B.vfg.at(i, j - 1, k), B.vfg.at(i, j + 1, k),
                        B.vfg.at(i, j, k - 1), B.vfg.at(i, j, k + 1), B.vfg.at(i, j, k)};
  const double delta = std::sqrt(v[6][0] * v[6][0] + v[6][1] * v[6][1] + v[6][2] * v[6][2]);
  if (delta <= 0.04) return;
  const double sigma = 0.071684196047;
  double nv[7][3];
  for (int l = 0; l < 7; ++l) {
    const double dl = v[l][0] * v[l][0] + v[l][1] * v[l][1] + v[l][2] * v[l][2];
    for (int e = 0; e < 3; ++e) nv[l][e] = (dl > 0.0) ? v[l][e] / std::sqrt(dl) : 0.0;
  }
  const double* n6[6] = {B.cx.at(i - 1, j, k), B.cx.at(i, j, k), B.ex.at(i, j - 1, k),
                         B.ex.at(i, j, k), B.tx.at(i, j, k - 1), B.tx.at(i, j, k)};
  const double sg[6] = {-1.0, 1.0, -1.0, 1.0, -1.0, 1.0};
  double kappa = 0.0;
  for (int m = 0; m < 6; ++m)
    for (int e = 0; e < 3; ++e) kappa = kappa + 0.5 * (nv[6][e] + nv[m][e]) * (sg[m] * n6[m][e]);
  kappa = -kappa / grd[0];
  for (int e = 0; e < 3; ++e) out[1 + e] = sigma * kappa * v[6][e];
  out[4] = out[1] * pv7[1] + out[2] * pv7[2] + out[3] * pv7[3];
  for (int n = 0; n < 5; ++n) out[n] = out[n] * grd[0];
}

static void calrhs_block(const Cfg& c, Block& B, double time) {
  const int im = B.imax, jm = B.jmax, km = B.kmax, npv = c.npv;
  const bool vis = c.iturb != -3;
  std::vector<double> ea((size_t)npv * (std::max(im, std::max(jm, km)) + 2)), eva(ea.size());
  double x[STENCIL][NPV_MAX];
  double pvl[NPV_MAX], pvr[NPV_MAX], dvl[NDV], dvr[NDV], fx[NPV_MAX];
  for (auto& v : B.res.d) v = 0.0;
  auto face = [&](int dir, int i, int j, int k, double* fi, double* fv) {
    /* stencil: cells along the face normal offsets (0,1) fastest, then the two transverse offsets */
    int di[3] = {0, 0, 0};
    auto cell = [&](int a, int t1, int t2, int* out) {
      /* a: normal offset, t1: first transverse, t2: second transverse */
      if (dir == 0) { out[0] = i + a; out[1] = j + t1; out[2] = k + t2; }
      else if (dir == 1) { out[0] = i + t2; out[1] = j + a; out[2] = k + t1; }
      else { out[0] = i + t1; out[1] = j + t2; out[2] = k + a; }
    };
    (void)di;
    int ll = 0, q[3];
    for (int t2 = -1; t2 <= 1; ++t2)
      for (int t1 = -1; t1 <= 1; ++t1)
        for (int a = 0; a <= 1; ++a) { cell(a, t1, t2, q); gather_pv(c, B, q[0], q[1], q[2], x[ll++]); }
    int ci[3], cr[3];
    cell(0, 0, 0, ci); cell(1, 0, 0, cr);
    if (c.nmuscl > 0) {
      for (int t2 = -1; t2 <= 1; ++t2) for (int t1 = -1; t1 <= 1; ++t1) { cell(-1, t1, t2, q); gather_pv(c, B, q[0], q[1], q[2], x[ll++]); }
      for (int t2 = -1; t2 <= 1; ++t2) for (int t1 = -1; t1 <= 1; ++t1) { cell(2, t1, t2, q); gather_pv(c, B, q[0], q[1], q[2], x[ll++]); }
      cell(-2, 0, 0, q); gather_pv(c, B, q[0], q[1], q[2], x[ll]);
      cell(3, 0, 0, q); gather_pv(c, B, q[0], q[1], q[2], x[ll + 1]);
      muscl(c, x, pvl, pvr);
      deteos_simple(c.eos, pvl[0] + c.pref, pvl[4], pvl[5], pvl[6], dvl);
      deteos_simple(c.eos, pvr[0] + c.pref, pvr[4], pvr[5], pvr[6], dvr);
    } else {
      gather_pv(c, B, ci[0], ci[1], ci[2], pvl);
      gather_pv(c, B, cr[0], cr[1], cr[2], pvr);
      std::memcpy(dvl, B.dv.at(ci[0], ci[1], ci[2]), sizeof(dvl));
      std::memcpy(dvr, B.dv.at(cr[0], cr[1], cr[2]), sizeof(dvr));
    }
    const double* nx = (dir == 0) ? B.cx.at(i, j, k) : (dir == 1 ? B.ex.at(i, j, k) : B.tx.at(i, j, k));
    double sdst[18];
    for (int l = 0; l < 18; ++l) sdst[l] = x[l][0];
    FaceIn f{nx, pvl, pvr, dvl, dvr, sdst, rot_q(c, B.grd.at(ci[0], ci[1], ci[2]) + 1),
             rot_q(c, B.grd.at(cr[0], cr[1], cr[2]) + 1)};
    calflux(c, f, fi);
    if (vis) {
      const double *e1, *e2, *e3, *e4, *t1, *t2, *t3, *t4;
      if (dir == 0) {
        e1 = B.ex.at(i, j - 1, k); e2 = B.ex.at(i + 1, j - 1, k); e3 = B.ex.at(i, j, k); e4 = B.ex.at(i + 1, j, k);
        t1 = B.tx.at(i, j, k - 1); t2 = B.tx.at(i + 1, j, k - 1); t3 = B.tx.at(i, j, k); t4 = B.tx.at(i + 1, j, k);
      } else if (dir == 1) {
        e1 = B.tx.at(i, j, k - 1); e2 = B.tx.at(i, j + 1, k - 1); e3 = B.tx.at(i, j, k); e4 = B.tx.at(i, j + 1, k);
        t1 = B.cx.at(i - 1, j, k); t2 = B.cx.at(i, j, k); t3 = B.cx.at(i - 1, j + 1, k); t4 = B.cx.at(i, j + 1, k);
      } else {
        e1 = B.cx.at(i - 1, j, k); e2 = B.cx.at(i - 1, j, k + 1); e3 = B.cx.at(i, j, k); e4 = B.cx.at(i, j, k + 1);
        t1 = B.ex.at(i, j - 1, k); t2 = B.ex.at(i, j, k); t3 = B.ex.at(i, j - 1, k + 1); t4 = B.ex.at(i, j, k + 1);
      }
      double tvl[3] = {0, 0, 0}, tvr[3] = {0, 0, 0};
      for (int m = 0; m < c.ntv; ++m) { tvl[m] = B.tv(m, ci[0], ci[1], ci[2]); tvr[m] = B.tv(m, cr[0], cr[1], cr[2]); }
      VsIn s{nx, e1, e2, e3, e4, t1, t2, t3, t4, B.grd.at(ci[0], ci[1], ci[2]), B.grd.at(cr[0], cr[1], cr[2]),
             B.dv.at(ci[0], ci[1], ci[2]), B.dv.at(cr[0], cr[1], cr[2]), tvl, tvr, x};
      vsflux(c, s, fv);
    }
  };
  /* i-faces */
  for (int k = 2; k <= km; ++k)
    for (int j = 2; j <= jm; ++j) {
      for (int i = 1; i <= im; ++i) face(0, i, j, k, &ea[(size_t)npv * i], &eva[(size_t)npv * i]);
      for (int i = 2; i <= im; ++i)
        for (int n = 0; n < npv; ++n) {
          double r = -(ea[npv * i + n] - ea[npv * (i - 1) + n]);
          if (vis) r = r + (eva[npv * i + n] - eva[npv * (i - 1) + n]);
          B.res(n, i, j, k) = r;
        }
    }
  /* j-faces */
  for (int i = 2; i <= im; ++i)
    for (int k = 2; k <= km; ++k) {
      for (int j = 1; j <= jm; ++j) face(1, i, j, k, &ea[(size_t)npv * j], &eva[(size_t)npv * j]);
      for (int j = 2; j <= jm; ++j)
        for (int n = 0; n < npv; ++n) {
          double r = B.res(n, i, j, k) - (ea[npv * j + n] - ea[npv * (j - 1) + n]);
          if (vis) r = r + (eva[npv * j + n] - eva[npv * (j - 1) + n]);
          B.res(n, i, j, k) = r;
        }
    }
  /* k-faces */
  for (int j = 2; j <= jm; ++j)
    for (int i = 2; i <= im; ++i) {
      for (int k = 1; k <= km; ++k) face(2, i, j, k, &ea[(size_t)npv * k], &eva[(size_t)npv * k]);
      for (int k = 2; k <= km; ++k)
        for (int n = 0; n < npv; ++n) {
          double r = B.res(n, i, j, k) - (ea[npv * k + n] - ea[npv * (k - 1) + n]);
          if (vis) r = r + (eva[npv * k + n] - eva[npv * (k - 1) + n]);
          B.res(n, i, j, k) = r;
        }
    }
  (void)fx;
  /* cell sources */
  for (int k = 2; k <= km; ++k)
    for (int j = 2; j <= jm; ++j)
      for (int i = 2; i <= im; ++i) {
        double x7[7][NPV_MAX];
        gather_pv(c, B, i - 1, j, k, x7[0]); gather_pv(c, B, i, j, k, x7[1]); gather_pv(c, B, i + 1, j, k, x7[2]);
        gather_pv(c, B, i, j - 1, k, x7[3]); gather_pv(c, B, i, j + 1, k, x7[4]);
        gather_pv(c, B, i, j, k - 1, x7[5]); gather_pv(c, B, i, j, k + 1, x7[6]);
        const double* grd = B.grd.at(i, j, k);
        const double* dv = B.dv.at(i, j, k);
        if (c.ncav > 0) {
          CavOut co = cavsource(c, x7[1], dv, grd[0]);
          B.res(5, i, j, k) = B.res(5, i, j, k) + co.r_v - co.r_c;
          for (int q = 0; q < 4; ++q) B.icav(q, i, j, k) = co.icav[q];
          B.rcav(0, i, j, k) = co.r_c; B.rcav(1, i, j, k) = co.r_v;
        }
        if (c.iturb == 0) {
          double tv[3];
          for (int m = 0; m < 3; ++m) tv[m] = B.tv(m, i, j, k);
          TurbOut to = kwsst_source(x7, B.cx.at(i - 1, j, k), B.cx.at(i, j, k), B.ex.at(i, j - 1, k), B.ex.at(i, j, k),
                                    B.tx.at(i, j, k - 1), B.tx.at(i, j, k), grd, dv, tv, c.ides);
          B.omega_cut(0, i, j, k) = to.omega_cut;
          B.res(7, i, j, k) = B.res(7, i, j, k) + to.source[0];
          B.res(8, i, j, k) = B.res(8, i, j, k) + to.source[1];
          for (int q = 0; q < 4; ++q) B.itt(q, i, j, k) = to.itt[q];
        }
        if (c.iturb == -1) {
          double tv[3];
          for (int m = 0; m < 3; ++m) tv[m] = B.tv(m, i, j, k);
          TurbOut to = kepsilon_source(x7, B.cx.at(i - 1, j, k), B.cx.at(i, j, k), B.ex.at(i, j - 1, k), B.ex.at(i, j, k),
                                       B.tx.at(i, j, k - 1), B.tx.at(i, j, k), grd, dv, tv);
          B.omega_cut(0, i, j, k) = to.omega_cut;
          B.res(7, i, j, k) = B.res(7, i, j, k) + to.source[0];
          B.res(8, i, j, k) = B.res(8, i, j, k) + to.source[1];
          for (int q = 0; q < 4; ++q) B.itt(q, i, j, k) = to.itt[q];
        }
        if (c.nsteady >= 1) {
          double us[NPV_MAX];
          const double* qq = B.qq.at(i, j, k);
          unsteady_source(c, x7[1], dv, qq, qq + npv, grd[0], us);
          for (int n = 0; n < npv; ++n) B.res(n, i, j, k) = B.res(n, i, j, k) - us[n];
        }
        if (c.gravity) {
          /* gravity%getgravitysource (src/gravity_module.f90:110-131) */
          double a[3];
          const int nd = (int)c.grav_t.size();
          for (int e = 0; e < 3; ++e) a[e] = c.grav_a[e];
          for (int m = 0; m < nd - 1; ++m)
            if (time >= c.grav_t[m] && time < c.grav_t[m + 1]) {
              for (int e = 0; e < 3; ++e)
                a[e] = c.grav_a[3 * m + e] + (c.grav_a[3 * (m + 1) + e] - c.grav_a[3 * m + e]) * (time - c.grav_t[m]) /
                                                 (c.grav_t[m + 1] - c.grav_t[m]);
              break;
            }
          if (time >= c.grav_t[nd - 1]) for (int e = 0; e < 3; ++e) a[e] = c.grav_a[3 * (nd - 1) + e];
          for (int e = 0; e < 3; ++e) B.res(1 + e, i, j, k) = B.res(1 + e, i, j, k) + dv[0] * grd[0] * a[e];
          B.res(4, i, j, k) = B.res(4, i, j, k) +
                              dv[0] * grd[0] * (a[0] * x7[1][1] + a[1] * x7[1][2] + a[2] * x7[1][3]);
        }
        if (c.rotation) {
          /* rotation%getrotationsource (src/rotation_module.f90:75-97), subtracted
             (src/rhs_module.f90:600-605): rho vol (2 omega x u + omega x (omega x r)) */
          const double* w = c.omega;
          const double* u = x7[1];
          const double* r = grd + 1;
          const double cor[3] = {2.0 * (w[1] * u[3] - w[2] * u[2]), 2.0 * (w[2] * u[1] - w[0] * u[3]),
                                 2.0 * (w[0] * u[2] - w[1] * u[1])};
          const double cen[3] = {w[0] * (w[1] * r[1] + w[2] * r[2]) - r[0] * (w[1] * w[1] + w[2] * w[2]),
                                 w[1] * (w[0] * r[0] + w[2] * r[2]) - r[1] * (w[0] * w[0] + w[2] * w[2]),
                                 w[2] * (w[0] * r[0] + w[1] * r[1]) - r[2] * (w[0] * w[0] + w[1] * w[1])};
          for (int e = 0; e < 3; ++e) B.res(1 + e, i, j, k) = B.res(1 + e, i, j, k) - dv[0] * grd[0] * (cor[e] + cen[e]);
        }
        if (c.csf) {
          double cs[5];
          csf_source(B, i, j, k, grd, B.pv.at(i, j, k), cs);
          for (int n = 0; n < 5; ++n) B.res(n, i, j, k) = B.res(n, i, j, k) + cs[n];
          for (int e = 0; e < 3; ++e) B.csf(e, i, j, k) = cs[1 + e];
        }
      }
}

/* ---------------- LU-SGS (src/update_module.f90:455-733) ---------------- */
static void lhs_in(const Cfg& c, Block& B, int i, int j, int k, LhsIn& L, double* tvbuf, const double* zero4) {
  L.cx1 = B.cx.at(i - 1, j, k); L.cx2 = B.cx.at(i, j, k);
  L.ex1 = B.ex.at(i, j - 1, k); L.ex2 = B.ex.at(i, j, k);
  L.tx1 = B.tx.at(i, j, k - 1); L.tx2 = B.tx.at(i, j, k);
  L.grd = B.grd.at(i, j, k); L.pv = B.pv.at(i, j, k); L.dv = B.dv.at(i, j, k);
  for (int m = 0; m < 3; ++m) tvbuf[m] = 0.0;
  for (int m = 0; m < c.ntv; ++m) tvbuf[m] = B.tv(m, i, j, k);
  L.tv = tvbuf;
  L.dt = B.dt(0, i, j, k);
  L.c = (c.ncav > 0) ? B.icav.at(i, j, k) : zero4;
  L.t = (c.iturb >= -1) ? B.itt.at(i, j, k) : zero4;
}

static void jac_apply(const Cfg& c, Block& B, const double* nx, int i, int j, int k, int sign, const double* dq,
                      double* acc, int sgn_acc) {
  double a[NPV_MAX][NPV_MAX];
  double tv[3] = {0, 0, 0};
  for (int m = 0; m < c.ntv; ++m) tv[m] = B.tv(m, i, j, k);
  caljac(c, nx, B.grd.at(i, j, k), B.pv.at(i, j, k), B.dv.at(i, j, k), tv, sign, a);
  for (int n = 0; n < c.npv; ++n)
    for (int l = 0; l < c.npv; ++l) acc[n] = (sgn_acc > 0) ? acc[n] + a[n][l] * dq[l] : acc[n] - a[n][l] * dq[l];
}

/* eddy%caleddy over the block after an update (src/update_module.f90:701-732, :300-330) */
static void eddy_block(const Cfg& c, Block& B) {
  const int im = B.imax, jm = B.jmax, km = B.kmax;
  if (c.iturb == -1) {
    for (int k = 2; k <= km; ++k)
      for (int j = 2; j <= jm; ++j)
        for (int i = 2; i <= im; ++i) {
          double tv[3];
          for (int m = 0; m < 3; ++m) tv[m] = B.tv(m, i, j, k);
          B.tv(2, i, j, k) = kepsilon_eddy(B.pv.at(i, j, k), B.dv.at(i, j, k), tv, B.grd.at(i, j, k));
        }
  }
  if (c.iturb == 0) {
    for (int k = 2; k <= km; ++k)
      for (int j = 2; j <= jm; ++j)
        for (int i = 2; i <= im; ++i) {
          double x7[7][NPV_MAX];
          gather_pv(c, B, i - 1, j, k, x7[0]); gather_pv(c, B, i, j, k, x7[1]); gather_pv(c, B, i + 1, j, k, x7[2]);
          gather_pv(c, B, i, j - 1, k, x7[3]); gather_pv(c, B, i, j + 1, k, x7[4]);
          gather_pv(c, B, i, j, k - 1, x7[5]); gather_pv(c, B, i, j, k + 1, x7[6]);
          double tv[3];
          for (int m = 0; m < 3; ++m) tv[m] = B.tv(m, i, j, k);
          B.tv(2, i, j, k) = kwsst_eddy(x7, B.cx.at(i - 1, j, k), B.cx.at(i, j, k), B.ex.at(i, j - 1, k), B.ex.at(i, j, k),
                                        B.tx.at(i, j, k - 1), B.tx.at(i, j, k), B.grd.at(i, j, k), B.dv.at(i, j, k), tv);
        }
  }
}

static void lusgs_block(const Cfg& c, Block& B) {
  const int im = B.imax, jm = B.jmax, km = B.kmax, npv = c.npv;
  const double zero4[4] = {0, 0, 0, 0};
  std::fill(B.dcv.d.begin(), B.dcv.d.end(), 0.0);
  std::fill(B.dqs.d.begin(), B.dqs.d.end(), 0.0);
  double tvb[3];
  for (int k = 2; k <= km; ++k)
    for (int j = 2; j <= jm; ++j)
      for (int i = 2; i <= im; ++i) {
        double* dcv = B.dcv.at(i, j, k);
        for (int n = 0; n < npv; ++n) dcv[n] = B.res(n, i, j, k);
        jac_apply(c, B, B.cx.at(i - 1, j, k), i - 1, j, k, 1, B.dqs.at(i - 1, j, k), dcv, 1);
        jac_apply(c, B, B.ex.at(i, j - 1, k), i, j - 1, k, 1, B.dqs.at(i, j - 1, k), dcv, 1);
        jac_apply(c, B, B.tx.at(i, j, k - 1), i, j, k - 1, 1, B.dqs.at(i, j, k - 1), dcv, 1);
        LhsIn L;
        lhs_in(c, B, i, j, k, L, tvb, zero4);
        lhs_getx(c, L, dcv, B.dqs.at(i, j, k));
      }
  std::fill(B.dqs.d.begin(), B.dqs.d.end(), 0.0);
  for (int k = km; k >= 2; --k)
    for (int j = jm; j >= 2; --j)
      for (int i = im; i >= 2; --i) {
        double* dcv = B.dcv.at(i, j, k);
        jac_apply(c, B, B.cx.at(i, j, k), i + 1, j, k, -1, B.dqs.at(i + 1, j, k), dcv, -1);
        jac_apply(c, B, B.ex.at(i, j, k), i, j + 1, k, -1, B.dqs.at(i, j + 1, k), dcv, -1);
        jac_apply(c, B, B.tx.at(i, j, k), i, j, k + 1, -1, B.dqs.at(i, j, k + 1), dcv, -1);
        LhsIn L;
        lhs_in(c, B, i, j, k, L, tvb, zero4);
        lhs_getx(c, L, dcv, B.dqs.at(i, j, k));
      }
  /* update + EOS */
  for (int k = 2; k <= km; ++k)
    for (int j = 2; j <= jm; ++j)
      for (int i = 2; i <= im; ++i) {
        double* pv = B.pv.at(i, j, k);
        const double* dq = B.dqs.at(i, j, k);
        double p[NPV_MAX];
        for (int n = 0; n < npv; ++n) p[n] = pv[n] + dq[n];
        p[0] = dmax(-c.pref + 1.0e1, p[0]);
        p[5] = dmin(1.0, dmax(0.0, p[5]));
        p[6] = dmin(1.0, dmax(0.0, p[6]));
        if (c.iturb >= -1) {
          p[7] = dmax(p[7], 1.0e-16);
          p[8] = dmax3(p[8], 1.0e-16, B.omega_cut(0, i, j, k));
        }
        for (int n = 0; n < npv; ++n) pv[n] = p[n];
        double tv[3] = {0, 0, 0};
        for (int m = 0; m < c.ntv; ++m) tv[m] = B.tv(m, i, j, k);
        deteos(c.eos, c.with_prop, p[0] + c.pref, p[4], p[5], p[6], B.dv.at(i, j, k), tv);
        for (int m = 0; m < c.ntv; ++m) B.tv(m, i, j, k) = tv[m];
      }
  eddy_block(c, B);
}

/* One stage of eulerex (src/update_module.f90:214-322) or rk3rd (:324-453): pv = a1 rk +
 * a2 pv + a3 getx(res) with the explicit diagonal solve, the update's clips, deteos and the
 * eddy viscosity.  rk (the state before the iteration) is kept in dqs at stage 1. */
static void explicit_block(const Cfg& c, Block& B, int m) {
  static const double a1[3] = {0.0, 0.75, 1.0 / 3.0}, a2[3] = {1.0, 0.25, 2.0 / 3.0}, a3[3] = {1.0, 0.25, 2.0 / 3.0};
  const bool rk3 = c.timemethod == 2;
  const double c1 = rk3 ? a1[m - 1] : 0.0, c2 = rk3 ? a2[m - 1] : 1.0, c3 = rk3 ? a3[m - 1] : 1.0;
  const int im = B.imax, jm = B.jmax, km = B.kmax, npv = c.npv;
  const double zero4[4] = {0, 0, 0, 0};
  double tvb[3];
  for (int k = 2; k <= km; ++k)
    for (int j = 2; j <= jm; ++j)
      for (int i = 2; i <= im; ++i) {
        double* pv = B.pv.at(i, j, k);
        double* rk = B.dqs.at(i, j, k);
        if (m == 1) for (int n = 0; n < npv; ++n) rk[n] = pv[n];
        LhsIn L;
        lhs_in(c, B, i, j, k, L, tvb, zero4);
        double res[NPV_MAX], x[NPV_MAX];
        for (int n = 0; n < npv; ++n) res[n] = B.res(n, i, j, k);
        lhs_getx_ex(c, L, res, x);
        double p[NPV_MAX];
        for (int n = 0; n < npv; ++n) p[n] = c1 * rk[n] + c2 * pv[n] + c3 * x[n];
        p[0] = dmax(-c.pref + 1.0e1, p[0]);
        p[5] = dmin(1.0, dmax(0.0, p[5]));
        p[6] = dmin(1.0, dmax(0.0, p[6]));
        if (c.iturb >= -1) {
          p[7] = dmax(p[7], 1.0e-16);
          p[8] = dmax3(p[8], 1.0e-16, B.omega_cut(0, i, j, k));
        }
        for (int n = 0; n < npv; ++n) pv[n] = p[n];
        double tv[3] = {0, 0, 0};
        for (int q = 0; q < c.ntv; ++q) tv[q] = B.tv(q, i, j, k);
        deteos(c.eos, c.with_prop, p[0] + c.pref, p[4], p[5], p[6], B.dv.at(i, j, k), tv);
        for (int q = 0; q < c.ntv; ++q) B.tv(q, i, j, k) = tv[q];
      }
  eddy_block(c, B);
}

template <class F>
static void for_blocks(Oracle& O, F f) {
  int nt = std::max(1, std::min<int>(O.nthreads, (int)O.b.size()));
  if (nt == 1) { for (size_t b = 0; b < O.b.size(); ++b) f((int)b); return; }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t] { for (size_t b = t; b < O.b.size(); b += nt) f((int)b); });
  for (auto& x : th) x.join();
}

static void alloc_block(const Cfg& c, Block& B) {
  const int im = B.imax, jm = B.jmax, km = B.kmax;
  B.pv.init(c.npv, -1, im + 3, -1, jm + 3, -1, km + 3);
  B.dv.init(NDV, -1, im + 3, -1, jm + 3, -1, km + 3);
  B.tv.init(std::max(c.ntv, 1), -1, im + 3, -1, jm + 3, -1, km + 3);
  B.qq.init(std::max(c.npv * c.nqq, 1), 2, im, 2, jm, 2, km);
  B.rcav.init(2, 2, im, 2, jm, 2, km);
  B.res.init(c.npv, 2, im, 2, jm, 2, km);
  B.icav.init(4, 2, im, 2, jm, 2, km);
  B.itt.init(4, 2, im, 2, jm, 2, km);
  B.omega_cut.init(1, 2, im, 2, jm, 2, km);
  B.dt.init(1, 2, im, 2, jm, 2, km);
  B.dqs.init(c.npv, 1, im + 1, 1, jm + 1, 1, km + 1);
  B.dcv.init(c.npv, 1, im + 1, 1, jm + 1, 1, km + 1);
  B.qres.init(c.npv, 2, im, 2, jm, 2, km);
  if (c.csf) {
    B.vfg.init(3, 1, im + 1, 1, jm + 1, 1, km + 1);
    B.csf.init(3, 2, im, 2, jm, 2, km);
  }
}

}  // namespace

/* ================================ C entry points ================================ */
extern "C" {

void* orc_create(const cfd3d_config* cfg, int nblocks, const cfd3d_block_desc* blocks, char* errbuf, int errlen) {
  Oracle* O = new Oracle();
  std::string err;
  if (!make_cfg(cfg, O->c, err)) goto fail;
  O->b.resize(nblocks);
  for (int n = 0; n < nblocks; ++n) {
    Block& B = O->b[n];
    const cfd3d_block_desc& d = blocks[n];
    B.imax = d.imax; B.jmax = d.jmax; B.kmax = d.kmax;
    if (B.imax < 4 || B.jmax < 4 || B.kmax < 4) { err = "block too small"; goto fail; }
    B.x.init(3, 2, B.imax + 1, 2, B.jmax + 1, 2, B.kmax + 1);
    for (int k = 0; k < d.kmax; ++k)
      for (int j = 0; j < d.jmax; ++j)
        for (int i = 0; i < d.imax; ++i)
          for (int v = 0; v < 3; ++v)
            B.x(v, i + 2, j + 2, k + 2) = d.xyz[v + 3 * ((size_t)i + (size_t)d.imax * ((size_t)j + (size_t)d.jmax * k))] * O->c.scale;
    if (!build_bcs(O->c, B, d, err)) goto fail;
    if (!build_cons(B, d, nblocks, err)) goto fail;
    face_vectors(B);
    alloc_block(O->c, B);
  }
  /* grid%construct order: face vectors + halo, reordering, volumes + halo, wall distance + halo */
  exchange_face_vectors(*O);
  reorder_cons(*O);
  for (auto& B : O->b) volumes(O->c, B);
  exchange_grd(*O, 0);
  if (O->c.ngrd == 5) { wall_distance(*O); exchange_grd(*O, 4); }
  if (!build_state_halos(*O, err)) goto fail;
  return O;
fail:
  if (errbuf && errlen > 0) { std::snprintf(errbuf, errlen, "%s", err.c_str()); }
  delete O;
  return nullptr;
}

void orc_destroy(void* h) { delete (Oracle*)h; }
void orc_set_threads(void* h, int n) { ((Oracle*)h)->nthreads = n; }
long orc_snd2_fallbacks(void) { return orc::g_snd2_fallbacks; }

int orc_sizes(void* h, int* npv, int* ntv, int* nqq, int* ngrd) {
  Oracle* O = (Oracle*)h;
  *npv = O->c.npv; *ntv = O->c.ntv; *nqq = O->c.nqq; *ngrd = O->c.ngrd;
  return 0;
}

/* reference values: rhoref, visref, kref, oref, emutref, str */
int orc_refs(void* h, double* out) {
  Oracle* O = (Oracle*)h;
  out[0] = O->c.rhoref; out[1] = O->c.visref; out[2] = O->c.kref; out[3] = O->c.oref; out[4] = O->c.emutref; out[5] = O->c.str;
  return 0;
}

/* t_ini_initial + set_others (src/initial_module.f90:678-771) */
int orc_initialize(void* h, int b, const double* pv_in) {
  Oracle* O = (Oracle*)h;
  const Cfg& c = O->c;
  Block& B = O->b[b];
  size_t q = 0;
  for (int k = 2; k <= B.kmax; ++k)
    for (int j = 2; j <= B.jmax; ++j)
      for (int i = 2; i <= B.imax; ++i) {
        double* pv = B.pv.at(i, j, k);
        if (pv_in) {
          for (int n = 0; n < c.npv; ++n) pv[n] = pv_in[q * c.npv + n];
        } else {
          pv[0] = 0.0;
          pv[1] = c.uref * std::cos(c.aos) * std::cos(c.aoa);
          pv[2] = c.uref * std::cos(c.aos) * std::sin(c.aoa);
          pv[3] = c.uref * std::sin(c.aos);
          pv[4] = c.tref; pv[5] = c.y1ref; pv[6] = c.y2ref;
          if (c.iturb >= -1) { pv[7] = c.kref; pv[8] = c.oref; }
        }
        ++q;
        double dv[NDV], tv[3] = {0, 0, 0};
        deteos(c.eos, c.with_prop, pv[0] + c.pref, pv[4], pv[5], pv[6], dv, tv);
        std::memcpy(B.dv.at(i, j, k), dv, sizeof(dv));
        if (c.iturb >= -1) tv[2] = c.emutref;
        for (int m = 0; m < c.ntv; ++m) B.tv(m, i, j, k) = tv[m];
        if (c.nsteady >= 1) {
          double qq[NPV_MAX];
          qq[0] = dv[0]; qq[1] = dv[0] * pv[1]; qq[2] = dv[0] * pv[2]; qq[3] = dv[0] * pv[3];
          qq[4] = dv[0] * (dv[1] + 0.5 * (sq(pv[1]) + sq(pv[2]) + sq(pv[3]))) - pv[0] - c.pref;
          for (int n = 5; n < c.npv; ++n) qq[n] = dv[0] * pv[n];
          double* Q = B.qq.at(i, j, k);
          for (int n = 0; n < c.npv; ++n) { Q[n] = qq[n]; Q[c.npv + n] = qq[n]; }
        }
        if (c.ncav > 0) { B.rcav(0, i, j, k) = 0.0; B.rcav(1, i, j, k) = 0.0; }
      }
  O->time_acc = 0.0;
  return 0;
}

int orc_set_state(void* h, int b, const double* pv, const double* dv, const double* tv, const double* qq) {
  Oracle* O = (Oracle*)h;
  Block& B = O->b[b];
  if (pv) std::memcpy(B.pv.d.data(), pv, B.pv.d.size() * 8);
  if (dv) std::memcpy(B.dv.d.data(), dv, B.dv.d.size() * 8);
  if (tv && O->c.ntv) std::memcpy(B.tv.d.data(), tv, B.tv.d.size() * 8);
  if (qq && O->c.nqq) std::memcpy(B.qq.d.data(), qq, B.qq.d.size() * 8);
  return 0;
}

int orc_get_state(void* h, int b, double* pv, double* dv, double* tv, double* qq, double* rcav) {
  Oracle* O = (Oracle*)h;
  Block& B = O->b[b];
  if (pv) std::memcpy(pv, B.pv.d.data(), B.pv.d.size() * 8);
  if (dv) std::memcpy(dv, B.dv.d.data(), B.dv.d.size() * 8);
  if (tv && O->c.ntv) std::memcpy(tv, B.tv.d.data(), B.tv.d.size() * 8);
  if (qq && O->c.nqq) std::memcpy(qq, B.qq.d.data(), B.qq.d.size() * 8);
  if (rcav) std::memcpy(rcav, B.rcav.d.data(), B.rcav.d.size() * 8);
  return 0;
}

/* csf = 1: vfg(3, 1:imax+1, 1:jmax+1, 1:kmax+1) and csf(3, 2:imax, 2:jmax, 2:kmax) of block b */
int orc_get_csf(void* h, int b, double* vfg, double* csf) {
  Oracle* O = (Oracle*)h;
  if (!O->c.csf) return 1;
  Block& B = O->b[b];
  if (vfg) std::memcpy(vfg, B.vfg.d.data(), B.vfg.d.size() * 8);
  if (csf) std::memcpy(csf, B.csf.d.data(), B.csf.d.size() * 8);
  return 0;
}

int orc_metrics(void* h, int b, double* cx, double* ex, double* tx, double* grd) {
  Oracle* O = (Oracle*)h;
  Block& B = O->b[b];
  if (cx) std::memcpy(cx, B.cx.d.data(), B.cx.d.size() * 8);
  if (ex) std::memcpy(ex, B.ex.d.data(), B.ex.d.size() * 8);
  if (tx) std::memcpy(tx, B.tx.d.data(), B.tx.d.size() * 8);
  if (grd) std::memcpy(grd, B.grd.d.data(), B.grd.d.size() * 8);
  return 0;
}

/* bc%setbc + rhs%calrhs on the current state (no update) */
int orc_residual(void* h, int b, double* res, double* icav, double* itt, double* omega_cut) {
  Oracle* O = (Oracle*)h;
  setbc(*O);
  for_blocks(*O, [&](int n) { calrhs_block(O->c, O->b[n], O->time_cur); });
  Block& B = O->b[b];
  if (res) std::memcpy(res, B.res.d.data(), B.res.d.size() * 8);
  if (icav) std::memcpy(icav, B.icav.d.data(), B.icav.d.size() * 8);
  if (itt) std::memcpy(itt, B.itt.d.data(), B.itt.d.size() * 8);
  if (omega_cut) std::memcpy(omega_cut, B.omega_cut.d.data(), B.omega_cut.d.size() * 8);
  return 0;
}

/* setqres + lusgs + residual (src/solve_module.f90:134-136); res_l2[npv], loc[4] */
int orc_iterate(void* h, int nt_phy, int nt, double timeprev, double* time_out, double* res_l2, int* loc) {
  Oracle* O = (Oracle*)h;
  Cfg& c = O->c;
  for (auto& B : O->b)
    for (int k = 2; k <= B.kmax; ++k) for (int j = 2; j <= B.jmax; ++j) for (int i = 2; i <= B.imax; ++i)
      for (int n = 0; n < c.npv; ++n) B.qres(n, i, j, k) = B.pv(n, i, j, k);
  std::vector<double> mins(O->b.size());
  for_blocks(*O, [&](int n) { mins[n] = timestep_block(c, O->b[n]); });
  double dtmin = 1.0e10;
  for (double m : mins) dtmin = dmin(dtmin, m);
  O->time_acc = O->time_acc + dtmin;
  double tstep = O->time_acc + timeprev;
  O->time_cur = (c.nsteady == 0) ? tstep : c.dt_phy * (double)nt_phy;
  if (c.timemethod == 3) {
    setbc(*O);
    for_blocks(*O, [&](int n) { calrhs_block(c, O->b[n], O->time_cur); });
    for_blocks(*O, [&](int n) { lusgs_block(c, O->b[n]); });
  } else {
    /* eulerex: one stage; rk3rd: three, the time step taken at the first only */
    const int nstage = (c.timemethod == 2) ? 3 : 1;
    for (int m = 1; m <= nstage; ++m) {
      setbc(*O);
      for_blocks(*O, [&](int n) { calrhs_block(c, O->b[n], O->time_cur); });
      for_blocks(*O, [&](int n) { explicit_block(c, O->b[n], m); });
    }
  }
  double res[NPV_MAX] = {0};
  double resmax = 1.0e-12;
  int lb = -1, li = 0, lj = 0, lk = 0;
  for (size_t bi = 0; bi < O->b.size(); ++bi) {
    Block& B = O->b[bi];
    for (int k = 2; k <= B.kmax; ++k) for (int j = 2; j <= B.jmax; ++j) for (int i = 2; i <= B.imax; ++i) {
      for (int n = 0; n < c.npv; ++n) {
        double d = std::fabs(B.qres(n, i, j, k) - B.pv(n, i, j, k));
        B.qres(n, i, j, k) = d;
        res[n] = res[n] + sq(d);
      }
      if (B.qres(0, i, j, k) > resmax) { resmax = B.qres(0, i, j, k); lb = (int)bi; li = i; lj = j; lk = k; }
    }
  }
  if (res_l2) for (int n = 0; n < c.npv; ++n) res_l2[n] = std::sqrt(res[n]);
  if (loc) { loc[0] = lb; loc[1] = li; loc[2] = lj; loc[3] = lk; }
  if (time_out) *time_out = O->time_cur;
  (void)nt;
  return 0;
}

/* solve%unsteadyupdate (src/solve_module.f90:155-183) */
int orc_unsteady_shift(void* h) {
  Oracle* O = (Oracle*)h;
  const Cfg& c = O->c;
  if (c.nqq == 0) return 0;
  for (auto& B : O->b)
    for (int k = 2; k <= B.kmax; ++k) for (int j = 2; j <= B.jmax; ++j) for (int i = 2; i <= B.imax; ++i) {
      double* Q = B.qq.at(i, j, k);
      for (int n = 0; n < c.npv; ++n) Q[c.npv + n] = Q[n];
      const double* dv = B.dv.at(i, j, k);
      const double* pv = B.pv.at(i, j, k);
      Q[0] = dv[0]; Q[1] = dv[0] * pv[1]; Q[2] = dv[0] * pv[2]; Q[3] = dv[0] * pv[3];
      Q[4] = dv[0] * (dv[1] + 0.5 * (sq(pv[1]) + sq(pv[2]) + sq(pv[3]))) - pv[0] - c.pref;
      for (int n = 5; n < c.npv; ++n) Q[n] = dv[0] * pv[n];
    }
  return 0;
}

/* pointwise EOS for the tests: deteos_simple (prop = 0) or deteos_prop (prop = 1) */
int orc_eos(int fluid, int ngas, int prop, long n, const double* p, const double* t, const double* y1,
            const double* y2, double* dv, double* tv) {
  EosSel s{fluid, ngas};
  for (long q = 0; q < n; ++q) {
    double tvl[3] = {0, 0, 0};
    deteos(s, prop != 0, p[q], t[q], y1[q], y2[q], dv + NDV * q, tvl);
    if (tv) { tv[2 * q] = tvl[0]; tv[2 * q + 1] = tvl[1]; }
  }
  return 0;
}

double orc_pww(double t) { return h2o_pww(t); }
double orc_tww(double p) { return h2o_tww(p); }

}  /* extern "C" */
