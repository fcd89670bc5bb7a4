// physics.cuh -- device physics of one pseudo-iteration.
//
// Per-point operators of the reference, rewritten for the GPU (one thread per face or
// cell, operands in registers, SoA state in HBM):
//   mixture EOS          deteos_simple / deteos_prop     src/eos_module.f90:1064-1234
//   MUSCL / MLP          tvd, mlp, 11 limiters            src/muscl_module.f90:104-413
//   inviscid fluxes      roe, roem, ausmpwp, ausmpup      src/flux_module.f90:198-721
//   viscous fluxes       vsflux_laminar / _turbulent      src/vsflux_module.f90:182-425
//   cavitation sources   merkle .. lee                    src/cav_module.f90:136-357
//   SST source, eddy     kwsst / calbigf / no_des         src/turbsource_module.f90:269-414,
//                                                         src/eddy_module.f90:135-187
//   dual-time source     unsteadysource                   src/unsteady_module.f90:96-114
//   diagonal operator    flowonly / flowturball, eigen    src/lhs_module.f90:346-534
//   split Jacobians      flowonly / flowturball           src/jacobian_module.f90:182-403
// The split Jacobian is applied matrix-free: its rows are rank-one updates of row 1 plus
// a diagonal, so A*dq costs O(npv) instead of the reference's O(npv^2).
#pragma once
#include <type_traits>
#include "iapws.cuh"
#include "df64.cuh"

namespace cfd {

constexpr int NPVM = 9;
constexpr int NDV = 18;

// solver parameters, passed by value to every kernel
struct Par {
  int npv, ntv, nqq, ngrd;
  int nsteady, iturb, nscheme, nmuscl, nlim, local, prec, fluid, ncav, fix_cav_clamp, with_prop;
  int mixed;   // 1: the mixed-precision form (IF97 sums in df64)
  int timemethod;   // 1 explicit Euler, 2 third-order Runge-Kutta, 3 LU-SGS
  int ides;         // SST length scale: 0 RANS, 1 DES, 2 DDES, 3 IDDES, 4 simplified IDDES
  int gravity;      // gravity source: 0 none, else the device history d.grav
  int csf;          // 1: the surface-tension source (d.vfg, d.csf)
  int rot;          // 1: a rotating frame of angular velocity omega (FP64 form)
  double omega[3];
  double tp_pt, tp_tt, tp_ht;   // total-pressure inlet: p_total, T_total, h(p_total, T_total)
  double dt_phy, cfl, c_v, c_c, pref, uref, str, rhoref, l_chord;
  double kref, oref, emutref;
  double uref_vec[3], tref, y1ref, y2ref;   // free-stream state bcinfo%pv (src/bc_module.f90:133-146)
  // mixed form: reference density / enthalpy and the gauge flux tensor of the uniform
  // free stream, phi[v][e] = e-component of the flux of variable v (pressure part omitted)
  double href;
  double phi[NPVM][3];
  // the same free-stream constants as float pairs (hi, lo) for the df64 flux terms:
  // rho_ref, h_ref, U, m = rho_ref U, and s with Phi[v][e] = m[e] s[v]
  float rhoref2[2], href2[2], U2[3][2], m2[3][2], sc2[NPVM][2];
};

template <class T>
__device__ __forceinline__ T sq(const T& x) { return x * x; }

// The rotating frame (src/rotation_module.f90, src/config_module.f90:126-141): the grid
// velocity omega x r of the boundary routines (gridvel, e.g. src/bc_module.f90:3557-3559),
// and 0.5 |omega x r|^2, the term that turns the total enthalpy into the rothalpy, written
// as rothalpy_l / rothalpy_r / the lhs's and jacobian's rothalpy write it
// (src/flux_module.f90:697-721, src/lhs_module.f90:573-584, src/jacobian_module.f90:486-495),
// r the cell centroid.
__device__ __forceinline__ void grid_vel(const Par& c, const double* r, double* gv) {
  gv[0] = c.omega[1] * r[2] - c.omega[2] * r[1];
  gv[1] = c.omega[2] * r[0] - c.omega[0] * r[2];
  gv[2] = c.omega[0] * r[1] - c.omega[1] * r[0];
}
__device__ __forceinline__ double rot_q(const Par& c, const double* r) {
  const double* w = c.omega;
  return 0.5 * (w[0] * w[0] * (r[1] * r[1] + r[2] * r[2]) + w[1] * w[1] * (r[0] * r[0] + r[2] * r[2]) +
                w[2] * w[2] * (r[0] * r[0] + r[1] * r[1]) -
                2.0 * (w[0] * w[1] * r[0] * r[1] + w[1] * w[2] * r[1] * r[2] + w[2] * w[0] * r[2] * r[0]));
}

// the preconditioning speed with the squared reference speed uref2 given, for the
// adjoint's derivative with respect to the free-stream speed
template <class R>
__device__ __forceinline__ R sndp2_u(const Par& c, R snd2, R u2, R uref2) {
  if (c.prec == 0) return snd2;
  if (c.prec == 1) return fmin(snd2, fmax(u2, uref2));
  return fmin(snd2, fmax(fmax(u2, uref2), R(c.str * c.str)));
}
template <class R>
__device__ __forceinline__ R sndp2_du_u(const Par& c, R snd2, R u2, R uref2) {
  if (c.prec == 0) return snd2;
  return fmin(snd2, fmax(u2, uref2));
}

template <class R>
__device__ __forceinline__ R sndp2_of(const Par& c, R snd2, R u2) {
  if (c.prec == 0) return snd2;
  if (c.prec == 1) return fmin(snd2, fmax(u2, R(c.uref * c.uref)));
  return fmin(snd2, fmax(fmax(u2, R(c.uref * c.uref)), R(c.str * c.str)));
}
template <class R>
__device__ __forceinline__ R sndp2_du_of(const Par& c, R snd2, R u2) {
  if (c.prec == 0) return snd2;
  return fmin(snd2, fmax(u2, R(c.uref * c.uref)));
}

// ------------------------------------------------------------------ far-field ghost state
// bcfarfield (src/bc_module.f90:2904-3013): the ghost pv from the boundary cell's pressure
// and velocity pb[0..3], density rb and sound speed c2b and the free-stream state bp, by the
// sign and size of the normal Mach number; pv holds the mirror cell's values on entry.  nx
// is the outward face vector, dl its inverse length.  Templated for the adjoint.
// The characteristic ghost state of bcfarfield (src/bc_module.f90:2904-3013): by the sign and
// size of the boundary cell's normal Mach number, the supersonic outflow (mirror), subsonic
// outflow, supersonic inflow or subsonic inflow treatment.  mode forces one branch, as the
// dedicated BCs do: FF_OUT_SUB bcoutflowsubsonic (:2699-2869), FF_IN_SUP bcinflowsupersonic
// (:2642-2678), FF_IN_SUB bcinflowsubsonic (:2464-2640) -- each the same formula as the
// farfield branch of that name, with bcinfo%pressure = pref.
enum FarfieldMode { FF_MACH = 0, FF_OUT_SUB = 1, FF_IN_SUP = 2, FF_IN_SUB = 3 };

template <class T>
__device__ __forceinline__ void farfield_pv(const Par& c, const double* nx, double dl, const T* pb, T rb, T c2b,
                                            const T* bp, T uref2, T* pv, int mode = FF_MACH) {
  T vel = (pb[1] * nx[0] + pb[2] * nx[1] + pb[3] * nx[2]) * dl;
  T a = sqrt(sndp2_u<T>(c, c2b, vel * vel, uref2));
  int br = mode;
  if (mode == FF_MACH) {
    T mach = vel / sqrt(c2b);
    br = (mach >= 0.0) ? ((mach < 1.0) ? FF_OUT_SUB : FF_MACH) : ((mach <= -1.0) ? FF_IN_SUP : FF_IN_SUB);
  }
  if (br == FF_OUT_SUB) {
    pv[0] = 2.0 * (c.pref - bp[0]) - pv[0];
    for (int q3 = 0; q3 < 3; ++q3) pv[1 + q3] = 2.0 * (pb[1 + q3] + nx[q3] * (pb[0] + bp[0] - c.pref) / rb / a * dl) - pv[1 + q3];
  } else if (br == FF_IN_SUP) {
    pv[0] = 2.0 * (c.pref - bp[0]) - pv[0];
    for (int v = 1; v < c.npv; ++v) pv[v] = 2.0 * bp[v] - pv[v];
    pv[5] = fmin(fmax(pv[5], 0.0), 1.0);
    pv[6] = fmin(fmax(pv[6], 0.0), 1.0);
  } else if (br == FF_IN_SUB) {
    T var = c.pref - bp[0] + pb[0] - rb * a * (nx[0] * (bp[1] - pb[1]) + nx[1] * (bp[2] - pb[2]) + nx[2] * (bp[3] - pb[3])) * dl;
    pv[0] = var - pv[0];
    for (int q3 = 0; q3 < 3; ++q3) pv[1 + q3] = 2.0 * (bp[1 + q3] + nx[q3] * 0.5 * var / rb / a * dl) - pv[1 + q3];
    for (int v = 4; v < c.npv; ++v) pv[v] = 2.0 * bp[v] - pv[v];
    pv[5] = fmin(fmax(pv[5], 0.0), 1.0);
    pv[6] = fmin(fmax(pv[6], 0.0), 1.0);
  }
}

// ------------------------------------------------------------------ mixture EOS
struct EosCount { unsigned long long* fallbacks; };

// ---- grouped df64 Gibbs sums for rho and h -----------------------------------------
// g_x = sum n I x^(I-1) y^J and g_y = sum n J x^I y^(J-1) of g = sum n x^I y^J: all that
// the density and the enthalpy need.  The tables are sorted by I, so each distinct power
// of x is factored out of its group's inner sums over powers of y; the coefficient
// products n I and n J are formed at compile time, and the sums accumulate with Dekker's
// add, whose error stays below ~2^-44 of the operands' magnitude.  Against the per-term
// evaluation (three products per term and derivative, IEEE-style df64 adds) this is about
// half the FP32 instructions, at an accuracy still far beyond what a face state needs.
__device__ __forceinline__ df64 dadd(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(__fadd_rn(s.lo, a.lo), b.lo));
}

template <const IJN* TAB, size_t N>
struct IGroups {
  static constexpr bool head(size_t k) { return k == 0 || TAB[k].i != TAB[k - 1].i; }
  static constexpr int count() {
    int c = 0;
    for (size_t k = 0; k < N; ++k) c += head(k) ? 1 : 0;
    return c;
  }
  static constexpr size_t start(int g) {
    int c = -1;
    for (size_t k = 0; k < N; ++k) {
      if (head(k)) ++c;
      if (c == g) return k;
    }
    return N;
  }
};

// one term of a group: n I y^J into px, n J y^(J-1) into py (the first contribution of
// each is assigned, later ones added; `hx`, `hy` say whether one was made)
template <const IJN* TAB, size_t K>
__device__ __forceinline__ void rh_term(df64 y, df64 yi, df64& px, df64& py, bool& hx, bool& hy) {
  constexpr int I = TAB[K].i, J = TAB[K].j;
  constexpr double n = TAB[K].n;
  if constexpr (I != 0) {
    const df64 v = df64(n * (double)I) * cpow<J>(y, yi);
    px = hx ? dadd(px, v) : v;
    hx = true;
  }
  if constexpr (J != 0) {
    const df64 v = df64(n * (double)J) * cpow<J - 1>(y, yi);
    py = hy ? dadd(py, v) : v;
    hy = true;
  }
}

template <const IJN* TAB, size_t S, size_t... K>
__device__ __forceinline__ void rh_group(df64 x, df64 y, df64 yi, df64& ax, df64& ay, bool& hax, bool& hay,
                                         std::index_sequence<K...>) {
  constexpr int I = TAB[S].i;
  df64 px(0.0f, 0.0f), py(0.0f, 0.0f);
  bool hx = false, hy = false;   // (compile-time after unrolling)
  (rh_term<TAB, S + K>(y, yi, px, py, hx, hy), ...);
  if (hx) {
    const df64 v = (I == 1) ? px : cpow<(I > 1 ? I - 1 : 1)>(x, x) * px;
    ax = hax ? dadd(ax, v) : v;
    hax = true;
  }
  if (hy) {
    const df64 v = (I == 0) ? py : cpow<(I > 0 ? I : 1)>(x, x) * py;
    ay = hay ? dadd(ay, v) : v;
    hay = true;
  }
}

template <const IJN* TAB, size_t N, int... G>
__device__ __forceinline__ void rh_groups(df64 x, df64 y, df64 yi, df64& ax, df64& ay,
                                          std::integer_sequence<int, G...>) {
  bool hax = false, hay = false;
  ax = df64(0.0f, 0.0f); ay = df64(0.0f, 0.0f);
  (rh_group<TAB, IGroups<TAB, N>::start(G)>(
       x, y, yi, ax, ay, hax, hay,
       std::make_index_sequence<IGroups<TAB, N>::start(G + 1) - IGroups<TAB, N>::start(G)>{}), ...);
}

template <const IJN* TAB, size_t N>
__device__ __forceinline__ void rh_sum(df64 x, df64 y, df64 yi, df64& ax, df64& ay) {
  rh_groups<TAB, N>(x, y, yi, ax, ay, std::make_integer_sequence<int, IGroups<TAB, N>::count()>{});
}

// region 1 (liquid): gamma_pi (as -g_x) and gamma_tau of the Gibbs sum, and tau
__device__ __forceinline__ void if97_r1_rh(df64 P, df64 T, df64& gp, df64& gt, df64& tau) {
  const df64 pi = P * df64(0.00000006049607);
  tau = df64(1386.0) / T;
  const df64 x = df64(7.1) - pi, y = tau - df64(1.222), yi = df64(1.0) / y;
  df64 ax, ay;
  rh_sum<kR1, 34>(x, y, yi, ax, ay);
  gp = -ax;
  gt = ay;
}
// region 2 (vapour, metastable set when meta): gamma_pi and gamma_tau, and tau
__device__ __forceinline__ void if97_r2_rh(df64 P, df64 T, bool meta, df64& gp, df64& gt, df64& tau) {
  const df64 pi = P * df64(1e-6), pi1 = df64(1.0e6) / P;
  tau = df64(540.0) / T;
  const df64 taui = T * df64(1.0 / 540.0);
  const df64 y = tau - df64(0.5), yi = df64(1.0) / y;
  df64 ix, iy, rx, ry;
  if (meta) {
    rh_sum<kR2MI, 9>(pi, tau, taui, ix, iy);
    rh_sum<kR2MR, 13>(pi, y, yi, rx, ry);
  } else {
    rh_sum<kR2I, 9>(pi, tau, taui, ix, iy);
    rh_sum<kR2R, 43>(pi, y, yi, rx, ry);
  }
  gp = dadd(pi1, rx);
  gt = dadd(iy, ry);
}

// IF97 liquid and vapour phases with the Gibbs sums in df64 on the FP32 pipes; one
// out-of-line copy per FULL flag keeps the expanded sums out of every caller
template <bool FULL>
__device__ __noinline__ void iapws_pair_df64(double p, double t, bool meta, Phase<double>& l, Phase<double>& v) {
  const df64 P(p), T(t);
  if constexpr (FULL) {
    Phase<df64> lx, vx;
    iapws_l<df64, FULL>(P, T, lx);
    iapws_v_meta<df64, FULL>(P, T, meta, vx);
    l.rho = (double)lx.rho; l.h = (double)lx.h;
    v.rho = (double)vx.rho; v.h = (double)vx.h;
    l.drdp = (double)lx.drdp; l.drdt = (double)lx.drdt; l.dhdp = (double)lx.dhdp; l.dhdt = (double)lx.dhdt;
    v.drdp = (double)vx.drdp; v.drdt = (double)vx.drdt; v.dhdp = (double)vx.dhdp; v.dhdt = (double)vx.dhdt;
  } else {
    // rho = c tau / gamma_pi, h = c' gamma_tau (the constants of iapws_l / iapws_v_meta)
    df64 gp, gt, tau;
    if97_r1_rh(P, T, gp, gt, tau);
    l.rho = (double)(df64((double)25.841246054191803727f) * tau / gp);
    l.h = (double)(df64(639675.036) * gt);
    if97_r2_rh(P, T, meta, gp, gt, tau);
    v.rho = (double)(df64(4.01245401527075799) * tau / gp);
    v.h = (double)(df64(249224.04) * gt);
  }
}

// the liquid phase alone (df64 sums): the face EOS of a face state without vapour
template <bool FULL>
__device__ __noinline__ void iapws_liq_df64(double p, double t, Phase<double>& l) {
  if constexpr (FULL) {
    Phase<df64> lx;
    iapws_l<df64, FULL>(df64(p), df64(t), lx);
    l.rho = (double)lx.rho; l.h = (double)lx.h;
    l.drdp = (double)lx.drdp; l.drdt = (double)lx.drdt; l.dhdp = (double)lx.dhdp; l.dhdt = (double)lx.dhdt;
  } else {
    df64 gp, gt, tau;
    if97_r1_rh(df64(p), df64(t), gp, gt, tau);
    l.rho = (double)(df64((double)25.841246054191803727f) * tau / gp);
    l.h = (double)(df64(639675.036) * gt);
  }
}

// The mixed form's face-state EOS: 1/rho and h of the liquid (and of the vapour when VAP)
// from the df64 sums, the reciprocal also taken in df64 (on the FP32 pipes: an FP64
// division costs a GB300 far more), and the gas's 1/rho = t / (p r1) from the same df64
// splits of p and t (each split costs FP64-pipe conversions)
template <bool VAP>
__device__ __noinline__ void iapws_inv_df64(double p, double t, bool meta, double* il, double* hl, double* iv,
                                            double* hv, double* ig) {
  // 1/rho = gamma_pi / (c tau) = gamma_pi T / (c T* ): no division beyond tau's
  const df64 P(p), T(t);
  *ig = (double)(T / (P * df64(0.00348383500557)));
  df64 gp, gt, tau;
  if97_r1_rh(P, T, gp, gt, tau);
  *il = (double)(gp * T * df64(1.0 / ((double)25.841246054191803727f * 1386.0)));
  *hl = (double)(df64(639675.036) * gt);
  if constexpr (VAP) {
    if97_r2_rh(P, T, meta, gp, gt, tau);
    *iv = (double)(gp * T * df64(1.0 / (4.01245401527075799 * 540.0)));
    *hv = (double)(df64(249224.04) * gt);
  }
}

// Phase properties of liquid and vapour.  MX evaluates the IF97 Gibbs sums in df64 (the
// mixed form); FULL = false evaluates only rho and h.  The metastable branch test
// p > p_sat(T) is taken in FP64 in both forms so that they select the same term set.
// vap = false (a state without vapour, y1 = 0, whose caller needs only the mixture's rho,
// h or c2): every vapour term of the mixture carries the factor y1 = 0, so the vapour sums
// (the larger half of the work) are skipped and a neutral vapour phase returned; the
// mixture's rho, h and c2 come out the same.
template <bool MX, bool FULL>
__device__ __forceinline__ void phases(int fluid, double p, double t, Phase<double>& l, Phase<double>& v,
                                       bool vap = true) {
  if (fluid == 1) {
    stiffened(p, t, l);
    ideal_gas(p, t, v);
    return;
  }
  if (!vap) {
    if constexpr (MX) iapws_liq_df64<FULL>(p, t, l);
    else iapws_l<double, FULL>(p, t, l);
    v.rho = 1.0; v.h = 0.0; v.drdp = 0.0; v.drdt = 0.0; v.dhdp = 0.0; v.dhdt = 1.0;
    return;
  }
  const bool meta = above_psat(p, t);
  if constexpr (MX) {
    iapws_pair_df64<FULL>(p, t, meta, l, v);
  } else {
    iapws_l<double, FULL>(p, t, l);
    iapws_v_meta<double, FULL>(p, t, meta, v);
  }
}

template <class T>
__device__ __forceinline__ void mixture(const Phase<T>& l, const Phase<T>& v, const Phase<T>& g, T y1, T y2, T* dv,
                                        unsigned long long* fallbacks, T* irh = nullptr) {
  // irh (optional): the phase reciprocals 1/rho_l, 1/rho_v, 1/rho_g, which the transport
  // properties reuse (three FP64 divisions fewer)
  dv[2] = l.rho; dv[3] = v.rho; dv[4] = g.rho;
  T irhol = 1.0 / dv[2], irhov = 1.0 / dv[3], irhog = 1.0 / dv[4];
  if (irh) { irh[0] = irhol; irh[1] = irhov; irh[2] = irhog; }
  T yl = 1.0 - y1 - y2;
  T irho = yl * irhol + y1 * irhov + y2 * irhog;
  dv[0] = 1.0 / irho;
  dv[1] = yl * l.h + y1 * v.h + y2 * g.h;
  T r2 = dv[0] * dv[0];
  T il2 = irhol * irhol, iv2 = irhov * irhov, ig2 = irhog * irhog;
  dv[6] = r2 * (yl * il2 * l.drdp + y1 * iv2 * v.drdp + y2 * ig2 * g.drdp);
  dv[7] = r2 * (yl * il2 * l.drdt + y1 * iv2 * v.drdt + y2 * ig2 * g.drdt);
  dv[8] = r2 * (irhol - irhov);
  dv[9] = r2 * (irhol - irhog);
  dv[10] = yl * l.dhdp + y1 * v.dhdp + y2 * g.dhdp;
  dv[11] = yl * l.dhdt + y1 * v.dhdt + y2 * g.dhdt;
  dv[12] = v.h - l.h;
  dv[13] = g.h - l.h;
  dv[5] = dv[0] * dv[11] / (dv[0] * dv[6] * dv[11] + dv[7] * (1.0 - dv[0] * dv[10]));
  if (dv[5] <= 0.0) {  // the reference's "alternative calculation for snd2"
    if (fallbacks) atomicAdd(fallbacks, 1ull);
    T ic2l = (dv[2] * l.drdp * l.dhdt + l.drdt * (1.0 - dv[2] * l.dhdp)) / (dv[2] * l.dhdt);
    T ic2v = (dv[3] * v.drdp * v.dhdt + v.drdt * (1.0 - dv[3] * v.dhdp)) / (dv[3] * v.dhdt);
    T ic2g = (dv[4] * g.drdp * g.dhdt + g.drdt * (1.0 - dv[4] * g.dhdp)) / (dv[4] * g.dhdt);
    dv[5] = 1.0 / (r2 * (yl * ic2l * il2 + y1 * ic2v * iv2 + y2 * ic2g * ig2));
  }
  dv[14] = v.drdp; dv[15] = v.drdt; dv[16] = l.drdp; dv[17] = l.drdt;
}

// mixture() for the mixed form's update and ghost states, from the phases' specific
// volumes il, iv, ig and enthalpies hl, hv, hg (FP64 values of df64 sums: no FP64 division
// but the mixture density's) and their FP32 derivatives lf, vf, gf.  The mixture density
// and enthalpy are FP64 -- they reach the residual through the dual-time source, the
// first-order face states and the face-state expansions; the phase densities, the
// derivatives, the enthalpy differences and the sound speed are FP32 -- they shape the
// implicit operator, the preconditioning speed and the FP32 flux and viscous terms only.
// Same formulas and order as mixture().
__device__ __forceinline__ void mixture_split(double il, double hl, double iv, double hv, double ig, double hg,
                                              const Phase<float>& lf, const Phase<float>& vf, const Phase<float>& gf,
                                              double y1, double y2, double* dv, unsigned long long* fallbacks) {
  const double yl = 1.0 - y1 - y2;
  const double irho = yl * il + y1 * iv + y2 * ig;
  dv[0] = 1.0 / irho;
  dv[1] = yl * hl + y1 * hv + y2 * hg;
  const float fil = (float)il, fiv = (float)iv, fig = (float)ig;
  const float rl = 1.0f / fil, rv = 1.0f / fiv, rg = 1.0f / fig;
  dv[2] = rl; dv[3] = rv; dv[4] = rg;
  const float r0 = (float)dv[0], fyl = (float)yl, fy1 = (float)y1, fy2 = (float)y2;
  const float r2 = r0 * r0;
  const float il2 = fil * fil, iv2 = fiv * fiv, ig2 = fig * fig;
  const float d6 = r2 * (fyl * il2 * lf.drdp + fy1 * iv2 * vf.drdp + fy2 * ig2 * gf.drdp);
  const float d7 = r2 * (fyl * il2 * lf.drdt + fy1 * iv2 * vf.drdt + fy2 * ig2 * gf.drdt);
  const float d10 = fyl * lf.dhdp + fy1 * vf.dhdp + fy2 * gf.dhdp;
  const float d11 = fyl * lf.dhdt + fy1 * vf.dhdt + fy2 * gf.dhdt;
  dv[6] = d6; dv[7] = d7;
  dv[8] = r2 * (fil - fiv);
  dv[9] = r2 * (fil - fig);
  dv[10] = d10; dv[11] = d11;
  dv[12] = (float)(hv - hl);
  dv[13] = (float)(hg - hl);
  float c2 = r0 * d11 / (r0 * d6 * d11 + d7 * (1.0f - r0 * d10));
  if (c2 <= 0.0f) {  // the reference's "alternative calculation for snd2"
    if (fallbacks) atomicAdd(fallbacks, 1ull);
    const float ic2l = (rl * lf.drdp * lf.dhdt + lf.drdt * (1.0f - rl * lf.dhdp)) / (rl * lf.dhdt);
    const float ic2v = (rv * vf.drdp * vf.dhdt + vf.drdt * (1.0f - rv * vf.dhdp)) / (rv * vf.dhdt);
    const float ic2g = (rg * gf.drdp * gf.dhdt + gf.drdt * (1.0f - rg * gf.dhdp)) / (rg * gf.dhdt);
    c2 = 1.0f / (r2 * (fyl * ic2l * il2 + fy1 * ic2v * iv2 + fy2 * ic2g * ig2));
  }
  dv[5] = c2;
  dv[14] = vf.drdp; dv[15] = vf.drdt; dv[16] = lf.drdp; dv[17] = lf.drdt;
}

// Phase properties and the mixture EOS in a generic scalar (the adjoint's dual numbers);
// the metastable branch is chosen on the values, as in the FP64 form.
template <class T>
__device__ __forceinline__ void phases_t(int fluid, T p, T t, Phase<T>& l, Phase<T>& v) {
  if (fluid == 1) {
    stiffened<T>(p, t, l);
    ideal_gas<T>(p, t, v);
    return;
  }
  const bool meta = above_psat((double)p, (double)t);
  iapws_l<T, true>(p, t, l);
  iapws_v_meta<T, true>(p, t, meta, v);
}
template <class T>
__device__ __forceinline__ void deteos_t(int fluid, int with_prop, T p, T t, T y1, T y2, T* dv, T* tv) {
  Phase<T> l, v, g;
  phases_t<T>(fluid, p, t, l, v);
  ideal_gas<T>(p, t, g);
  T irh[3];
  mixture<T>(l, v, g, y1, y2, dv, nullptr, irh);
  if (with_prop) {
    T lv, lc, vv, vc;
    if (fluid == 1) {
      lv = stiffened_vis<T>(t); lc = 4598.0 * lv;
      vv = ideal_vis<T>(t); vc = 1395.333333 * vv;
    } else {
      iapws_transport<T>(t, l.rho, lv, lc);
      iapws_transport<T>(t, v.rho, vv, vc);
    }
    T gv = ideal_vis<T>(t), gc = 1395.333333 * gv;
    T yl = 1.0 - y1 - y2;
    const T irhol = irh[0], irhov = irh[1], irhog = irh[2];
    tv[0] = dv[0] * (lv * yl * irhol + vv * y1 * irhov + gv * y2 * irhog);
    tv[1] = dv[0] * (lc * yl * irhol + vc * y1 * irhov + gc * y2 * irhog);
  }
}

// eos%deteos_simple
// (vap = false: the caller reads only dv(1), dv(2), dv(6) of a state with y1 = 0; see phases)
template <bool MX = false>
__device__ __forceinline__ void deteos_simple(int fluid, double p, double t, double y1, double y2, double* dv,
                                              unsigned long long* fb, bool vap = true) {
  Phase<double> l, v, g;
  phases<MX, true>(fluid, p, t, l, v, vap);
  ideal_gas(p, t, g);
  mixture(l, v, g, y1, y2, dv, fb);
}

// mixture density and static enthalpy only: all that the Roe and AUSM+-up fluxes read of
// the reconstructed face states; the same operations as the rho, h of deteos_simple
// the mixed form's face mixture from the phases' 1/rho and h: the gas's reciprocal as
// t / (p r1) in df64, the mixture sums and its one reciprocal in FP64
__device__ __forceinline__ void mix_face_mx(double t, double y1, double y2, double il, double hl, double iv,
                                            double hv, double ig, double& rho, double& h) {
  const double yl = 1.0 - y1 - y2;
  rho = 1.0 / (yl * il + y1 * iv + y2 * ig);
  h = yl * hl + y1 * hv + y2 * (1004.64 * t);
}

template <bool MX = false>
__device__ __forceinline__ void eos_rho_h(int fluid, double p, double t, double y1, double y2, double& rho, double& h) {
  if constexpr (MX) {
    if (fluid != 1) {
      // phase reciprocals in df64
      double il, hl, iv = 0.0, hv = 0.0, ig;
      if (y1 != 0.0) iapws_inv_df64<true>(p, t, above_psat(p, t), &il, &hl, &iv, &hv, &ig);
      else iapws_inv_df64<false>(p, t, false, &il, &hl, &iv, &hv, &ig);
      mix_face_mx(t, y1, y2, il, hl, iv, hv, ig, rho, h);
      return;
    }
  }
  Phase<double> l, v, g;
  phases<MX, false>(fluid, p, t, l, v, y1 != 0.0);
  ideal_gas(p, t, g);
  double irhol = 1.0 / l.rho, irhov = 1.0 / v.rho, irhog = 1.0 / g.rho;
  double yl = 1.0 - y1 - y2;
  double irho = yl * irhol + y1 * irhov + y2 * irhog;
  rho = 1.0 / irho;
  h = yl * l.h + y1 * v.h + y2 * g.h;
}

// eos%deteos: with transport properties when with_prop (tv(1:2) written), else simple
template <bool MX = false>
__device__ __forceinline__ void deteos(int fluid, int with_prop, double p, double t, double y1, double y2,
                                       double* dv, double* tv, unsigned long long* fb) {
  Phase<double> l, v, g;
  phases<MX, true>(fluid, p, t, l, v);
  ideal_gas(p, t, g);
  double irh[3];
  mixture(l, v, g, y1, y2, dv, fb, irh);
  if (with_prop) {
    double lv, lc, vv, vc;
    if (fluid == 1) {
      lv = stiffened_vis(t); lc = 4598.0 * lv;
      vv = ideal_vis(t); vc = 1395.333333 * vv;
    } else {
      iapws_transport(t, l.rho, lv, lc);
      iapws_transport(t, v.rho, vv, vc);
    }
    double gv = ideal_vis(t), gc = 1395.333333 * gv;
    double yl = 1.0 - y1 - y2;
    const double irhol = irh[0], irhov = irh[1], irhog = irh[2];
    tv[0] = dv[0] * (lv * yl * irhol + vv * y1 * irhov + gv * y2 * irhog);
    tv[1] = dv[0] * (lc * yl * irhol + vc * y1 * irhov + gc * y2 * irhog);
  }
}

// eos%deteos of the mixed form's update: phase densities and enthalpies from df64 IF97 sums
// (they enter the residual: dual-time source, face states of first-order schemes), their
// p / T derivatives and the transport properties in FP32 (they only shape the implicit
// operator, the preconditioning speed and the FP32 viscous fluxes); mixture in FP64.
__device__ __forceinline__ void deteos_split(int fluid, int with_prop, double p, double t, double y1, double y2,
                                             double* dv, double* tv, unsigned long long* fb) {
  double il, hl, iv, hv, ig;
  Phase<float> lf, vf, gf;
  const float pf = (float)p, tf = (float)t;
  if (fluid == 1) {
    Phase<double> l, v;
    stiffened(p, t, l);
    ideal_gas(p, t, v);
    il = 1.0 / l.rho; hl = l.h; iv = 1.0 / v.rho; hv = v.h;
    ig = (double)(df64(t) / (df64(p) * df64(0.00348383500557)));   // the gas: t / (p r1)
    lf.drdp = (float)l.drdp; lf.drdt = (float)l.drdt; lf.dhdp = (float)l.dhdp; lf.dhdt = (float)l.dhdt;
    vf.drdp = (float)v.drdp; vf.drdt = (float)v.drdt; vf.dhdp = (float)v.dhdp; vf.dhdt = (float)v.dhdt;
  } else {
    // (the gas's 1/rho = t / (p r1) comes with the phases, from the same df64 splits)
    const bool meta = above_psat(p, t);
    iapws_l<float, true>(pf, tf, lf);
    iapws_v_meta<float, true>(pf, tf, meta, vf);
    if (y1 != 0.0) {
      iapws_inv_df64<true>(p, t, meta, &il, &hl, &iv, &hv, &ig);
    } else {
      // without vapour the vapour's 1/rho and h enter the mixture with the factor y1 = 0:
      // its df64 sums are skipped, and the phase's FP32 values serve the vapour density,
      // enthalpy difference and derivatives the implicit operator and the cavitation
      // source read
      iapws_inv_df64<false>(p, t, meta, &il, &hl, &iv, &hv, &ig);
      iv = (double)(1.0f / vf.rho);
      hv = (double)vf.h;
    }
  }
  ideal_gas<float>(pf, tf, gf);
  const double hg = 1004.64 * t;   // the gas's h = cp T
  mixture_split(il, hl, iv, hv, ig, hg, lf, vf, gf, y1, y2, dv, fb);
  if (with_prop) {
    // the transport properties in FP32: they feed the FP32 viscous fluxes, the SST terms
    // and the operator's viscous eigenvalue
    float lv, lc, vv, vc;
    if (fluid == 1) {
      lv = stiffened_vis<float>(tf); lc = 4598.0f * lv;
      vv = ideal_vis<float>(tf); vc = 1395.333333f * vv;
    } else {
      iapws_transport<float>(tf, (float)dv[2], lv, lc);
      iapws_transport<float>(tf, (float)dv[3], vv, vc);
    }
    float gv = ideal_vis<float>(tf), gc = 1395.333333f * gv;
    const float r0 = (float)dv[0], fyl = (float)(1.0 - y1 - y2), fy1 = (float)y1, fy2 = (float)y2;
    const float fil = (float)il, fiv = (float)iv, fig = (float)ig;
    tv[0] = r0 * (lv * fyl * fil + vv * fy1 * fiv + gv * fy2 * fig);
    tv[1] = r0 * (lc * fyl * fil + vc * fy1 * fiv + gc * fy2 * fig);
  }
}

// isfinite by the exponent bits (integer instructions: the FP64 pipe is the scarce one)
__device__ __forceinline__ bool finite_bits(double x) {
  return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000;
}

// ------------------------------------------------------------------ MUSCL / MLP
// Products and sums without FMA contraction.  A reconstructed state often lands exactly
// on a clip bound (y1 = 0 next to a cell without vapour, when the MLP factor is exactly 2),
// and which side of the bound it rounds to selects the clip; the reference is compiled
// without contraction, so the reconstruction repeats its rounding step for step.
__device__ __forceinline__ double nmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double nadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double nsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float nmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float nadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float nsub(float a, float b) { return __fsub_rn(a, b); }
// quotients of the reconstruction: IEEE division in FP64 (the reference's arithmetic), the
// hardware's fast reciprocal-based quotient (2 ulp) in the mixed form's FP32 (a correctly
// rounded FP32 division is a long instruction sequence, and the reconstruction's several
// per variable swell the face kernel beyond the instruction cache)
template <class R>
__device__ __forceinline__ R rdiv(R a, R b) { return a / b; }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdividef(a, b); }

template <class R>
__device__ __forceinline__ R limiter(int nlim, R r, R r1, R r2, R alp) {
  R c;
  switch (nlim) {
    case 0: return R(1);
    case 1: return fmax(R(0), fmin(R(1), r));
    case 2: return fmax(fmax(R(0), fmin(R(1), alp * r)), fmin(alp, r));
    case 3: c = rdiv(r + fabs(r), R(1) + fabs(r)); return fmax(R(0), fmin(fmin(alp, alp * r), c));
    case 4: c = rdiv(R(1) + r, R(2)); return fmax(R(0), fmin(fmin(alp, alp * r), c));
    case 5: c = rdiv(nadd(nmul(r, r), r), nadd(R(1), nmul(r, r))); return fmax(fmax(R(0), fmin(c * r, R(1))), fmin(r, c));
    case 6: c = fmin(R(1.5), alp); return fmax(fmax(R(0), fmin(c * r, R(1))), fmin(r, c));
    case 7: c = rdiv(nadd(R(1), nmul(R(2), r)), R(3)); return fmax(R(0), fmin(fmin(alp, alp * r), c));
    case 8:
      c = rdiv(nsub(nadd(nadd(nmul(R(-2), r1), R(11)), nmul(R(24), r)), nmul(R(3), r2)), R(30));
      return fmax(R(0), fmin(fmin(alp, alp * r), c));
    case 9: return rdiv(nadd(R(1), nmul(R(2), r)), R(3));
    default: return rdiv(nsub(nadd(nadd(nmul(R(-2), r1), R(11)), nmul(R(24), r)), nmul(R(3), r2)), R(30));
  }
}

template <class R>
__device__ __forceinline__ void muscl_var(const Par& c, const R* x, R& xl, R& xr) {
  const R eps = R(1.0e-30), eps2 = R(1.0e-3);
  R dq = x[9] - x[8];
  R dqm = x[8] - x[22];
  R dqm1 = x[22] - x[36];
  R dqp = x[31] - x[9];
  R dqp1 = x[37] - x[31];
  R dqmm = rdiv(R(1), dqm + eps);
  R r0 = dq * dqmm, r10 = dqm1 * dqmm, r20 = dqp * dqmm;
  R dqpp = rdiv(R(1), dqp + eps);
  R r1 = dq * dqpp, r11 = dqp1 * dqpp, r21 = dqm * dqpp;
  R alp0 = R(2), alp1 = R(2);
  if (c.nmuscl == 2) {
    R rxy_l = fabs(rdiv(x[10] - x[6], x[9] - x[22] + eps));
    R rxz_l = fabs(rdiv(x[14] - x[2], x[9] - x[22] + eps));
    R rxy_r = fabs(rdiv(x[11] - x[7], x[31] - x[8] + eps));
    R rxz_r = fabs(rdiv(x[15] - x[3], x[31] - x[8] + eps));
    // min/max over the 3x3 planes: A = cells 0..17 (both face sides), L = i-1 plane (18..26),
    // R = i+2 plane (27..35); "even" = the 9 cells of the left side (0,2,..,16), "odd" right side
    R mA = x[0], MA = x[0], mE = x[0], ME = x[0], mO = x[1], MO = x[1];
#pragma unroll
    for (int l = 1; l < 18; ++l) { mA = fmin(mA, x[l]); MA = fmax(MA, x[l]); }
#pragma unroll
    for (int l = 2; l < 18; l += 2) { mE = fmin(mE, x[l]); ME = fmax(ME, x[l]); }
#pragma unroll
    for (int l = 3; l < 18; l += 2) { mO = fmin(mO, x[l]); MO = fmax(MO, x[l]); }
    R mL = x[18], ML = x[18], mR = x[27], MR = x[27];
#pragma unroll
    for (int l = 19; l < 27; ++l) { mL = fmin(mL, x[l]); ML = fmax(ML, x[l]); }
#pragma unroll
    for (int l = 28; l < 36; ++l) { mR = fmin(mR, x[l]); MR = fmax(MR, x[l]); }
    R qmin, qmax;
    if (rxy_l < eps2 && rxz_l < eps2) { qmin = fmin(mA, mL); qmax = fmax(MA, ML); }
    else if (x[9] - x[22] > R(0)) { qmax = MA; qmin = fmin(mE, mL); }
    else { qmin = mA; qmax = fmax(ME, ML); }
    R qml = fmin(fabs(qmax - x[8]), fabs(qmin - x[8]));
    if (rxy_r < eps2 && rxz_r < eps2) { qmin = fmin(mA, mR); qmax = fmax(MA, MR); }
    else if (x[31] - x[8] > R(0)) { qmax = fmax(MO, MR); qmin = mA; }
    else { qmin = fmin(mO, mR); qmax = MA; }
    R qmr = fmin(fabs(qmax - x[9]), fabs(qmin - x[9]));
    alp0 = rdiv(rdiv(R(2) * fmax(R(1), r0), fabs(dq) + eps), R(1) + rxy_l + rxz_l) * qml;
    if (fabs(dq) <= eps) alp1 = rdiv(R(2) * fmax(R(1), rdiv(dqp, eps)) * fabs(dqpp), R(1) + rxy_r + rxz_r) * qmr;
    else alp1 = rdiv(R(2) * fmax(R(1), rdiv(R(1), r1)) * fabs(dqpp), R(1) + rxy_r + rxz_r) * qmr;
    alp0 = fmax(R(1), fmin(R(2), alp0));
    alp1 = fmax(R(1), fmin(R(2), alp1));
  }
  xl = nadd(x[8], nmul(nmul(R(0.5), limiter<R>(c.nlim, r0, r10, r20, alp0)), dqm));
  xr = nsub(x[9], nmul(nmul(R(0.5), limiter<R>(c.nlim, r1, r11, r21, alp1)), dqp));
}

// muscl_var in FP32 from the reduced stencil a face needs: the six cells of the line through
// it (cm2 .. c3 at normal offsets -2 .. +3; c0 the left cell, c1 the right), the first and
// second transverse differences of planes 0 and 1 (dt0 = x[10] - x[6], dr0 = x[14] - x[2],
// dt1 = x[11] - x[7], dr1 = x[15] - x[3]) and the minimum and maximum over the 3 x 3 cells
// of planes -1, 0, 1, 2 (mn, mx).  MLP's minima and maxima over the 38-cell stencil are those
// of the planes' (a minimum is exact whatever the grouping), and every other operation is
// muscl_var's, so the result equals muscl_var<float> on the full stencil.
__device__ __forceinline__ void muscl_reduced(const Par& c, float cm2, float cm1, float c0, float c1, float c2,
                                              float c3, float dt0, float dr0, float dt1, float dr1, const float* mn,
                                              const float* mx, float& xl, float& xr) {
  using R = float;
  const R eps = R(1.0e-30), eps2 = R(1.0e-3);
  R dq = c1 - c0;
  R dqm = c0 - cm1;
  R dqm1 = cm1 - cm2;
  R dqp = c2 - c1;
  R dqp1 = c3 - c2;
  R dqmm = rdiv(R(1), dqm + eps);
  R r0 = dq * dqmm, r10 = dqm1 * dqmm, r20 = dqp * dqmm;
  R dqpp = rdiv(R(1), dqp + eps);
  R r1 = dq * dqpp, r11 = dqp1 * dqpp, r21 = dqm * dqpp;
  R alp0 = R(2), alp1 = R(2);
  if (c.nmuscl == 2) {
    R rxy_l = fabs(rdiv(dt0, c1 - cm1 + eps));
    R rxz_l = fabs(rdiv(dr0, c1 - cm1 + eps));
    R rxy_r = fabs(rdiv(dt1, c2 - c0 + eps));
    R rxz_r = fabs(rdiv(dr1, c2 - c0 + eps));
    const R mA = fmin(mn[1], mn[2]), MA = fmax(mx[1], mx[2]);
    const R mE = mn[1], ME = mx[1], mO = mn[2], MO = mx[2];
    const R mL = mn[0], ML = mx[0], mR = mn[3], MR = mx[3];
    R qmin, qmax;
    if (rxy_l < eps2 && rxz_l < eps2) { qmin = fmin(mA, mL); qmax = fmax(MA, ML); }
    else if (c1 - cm1 > R(0)) { qmax = MA; qmin = fmin(mE, mL); }
    else { qmin = mA; qmax = fmax(ME, ML); }
    R qml = fmin(fabs(qmax - c0), fabs(qmin - c0));
    if (rxy_r < eps2 && rxz_r < eps2) { qmin = fmin(mA, mR); qmax = fmax(MA, MR); }
    else if (c2 - c0 > R(0)) { qmax = fmax(MO, MR); qmin = mA; }
    else { qmin = fmin(mO, mR); qmax = MA; }
    R qmr = fmin(fabs(qmax - c1), fabs(qmin - c1));
    alp0 = rdiv(rdiv(R(2) * fmax(R(1), r0), fabs(dq) + eps), R(1) + rxy_l + rxz_l) * qml;
    if (fabs(dq) <= eps) alp1 = rdiv(R(2) * fmax(R(1), rdiv(dqp, eps)) * fabs(dqpp), R(1) + rxy_r + rxz_r) * qmr;
    else alp1 = rdiv(R(2) * fmax(R(1), rdiv(R(1), r1)) * fabs(dqpp), R(1) + rxy_r + rxz_r) * qmr;
    alp0 = fmax(R(1), fmin(R(2), alp0));
    alp1 = fmax(R(1), fmin(R(2), alp1));
  }
  xl = nadd(c0, nmul(nmul(R(0.5), limiter<R>(c.nlim, r0, r10, r20, alp0)), dqm));
  xr = nsub(c1, nmul(nmul(R(0.5), limiter<R>(c.nlim, r1, r11, r21, alp1)), dqp));
}

// post-clipping of the reconstructed states (muscl_module.f90:136-158)
template <class R>
__device__ __forceinline__ void muscl_clip(const Par& c, const R* c9, const R* c10, R* xl, R* xr) {
  xl[0] = fmax(R(-c.pref + 10.0), xl[0]);
  xr[0] = fmax(R(-c.pref + 10.0), xr[0]);
  if (xl[5] < R(0) || xl[5] > R(1)) xl[5] = c9[5];
  if (xr[5] < R(0) || xr[5] > R(1)) xr[5] = c10[5];
  if (xl[6] < R(0) || xl[6] > R(1)) xl[6] = c9[6];
  if (xr[6] < R(0) || xr[6] > R(1)) xr[6] = c10[6];
  if (xl[5] + xl[6] > R(1)) { xl[5] = c9[5]; xl[6] = c9[6]; }
  if (xr[5] + xr[6] > R(1)) { xr[5] = c10[5]; xr[6] = c10[6]; }
  if (c.npv > 7) {
    if (xl[7] < R(0) && c9[7] > R(0)) xl[7] = c9[7];
    if (xr[7] < R(0) && c10[7] > R(0)) xr[7] = c10[7];
    if (xl[8] < R(0) && c9[8] > R(0)) xl[8] = c9[8];
    if (xr[8] < R(0) && c10[8] > R(0)) xr[8] = c10[8];
  }
}

// ------------------------------------------------------------------ inviscid fluxes
// L/R face states: pv (npv), rho, h(static), snd2 in dv slots [0], [1], [5]
// L/R face states: pv (npv), rho, h(static), snd2 in dv slots [0], [1], [5]
template <class T>
struct FaceStateT { T pv[NPVM]; T rho, h, c2; };
using FaceState = FaceStateT<double>;

template <class T>
__device__ __forceinline__ T sdst_ratio_min(const T* s) {
  T v = fmin(s[8] / s[9], s[9] / s[8]);
  v = fmin(v, fmin(s[10] / s[8], s[8] / s[10]));
  v = fmin(v, fmin(s[8] / s[6], s[6] / s[8]));
  v = fmin(v, fmin(s[8] / s[2], s[2] / s[8]));
  v = fmin(v, fmin(s[8] / s[14], s[14] / s[8]));
  v = fmin(v, fmin(s[9] / s[11], s[11] / s[9]));
  v = fmin(v, fmin(s[9] / s[7], s[7] / s[9]));
  v = fmin(v, fmin(s[3] / s[9], s[9] / s[3]));
  v = fmin(v, fmin(s[9] / s[15], s[15] / s[9]));
  return v;
}

// Roe-average state of a face: sqrt(rho)-weighted velocities and scalars, arithmetic
// means of p and T (src/flux_module.f90:222-236)
template <class T>
__device__ __forceinline__ void roe_state(int npv, const FaceStateT<T>& L, const FaceStateT<T>& Rs, T* ravg) {
  const T* pl = L.pv;
  const T* pr = Rs.pv;
  T srl = sqrt(L.rho), srr = sqrt(Rs.rho);
  T ravg_d = 1.0 / (srl + srr);
  ravg[0] = 0.5 * (pl[0] + pr[0]);
  ravg[4] = 0.5 * (pl[4] + pr[4]);
  for (int k = 1; k <= 3; ++k) ravg[k] = (srl * pl[k] + srr * pr[k]) * ravg_d;
  for (int k = 5; k < npv; ++k) ravg[k] = (srl * pl[k] + srr * pr[k]) * ravg_d;
}

// The four inviscid fluxes (src/flux_module.f90:198-641) given the Roe-average state
// ravg, its sound speed rc2 and the squared reference speed uref2; templated on the
// scalar so that the adjoint evaluates the same code on dual numbers.  n is the
// unnormalised face vector; fx (npv) is the face flux.
template <class T>
__device__ inline void inviscid_flux_core(const Par& c, const double* n, const FaceStateT<T>& L,
                                          const FaceStateT<T>& Rs, const T* sdst_in, const T* ravg, T rc2,
                                          T uref2, T* fx) {
  const int npv = c.npv;
  double dl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  if (dl == 0.0) {
    for (int k = 0; k < npv; ++k) fx[k] = T(0.0);
    return;
  }
  double nx = n[0] / dl, ny = n[1] / dl, nz = n[2] / dl;
  const T* pl = L.pv;
  const T* pr = Rs.pv;
  T rrho = sqrt(L.rho * Rs.rho);
  const double pref = c.pref;
  const T srl = sqrt(L.rho), srr = sqrt(Rs.rho);
  const T ravg_d = 1.0 / (srl + srr);
  const T hl = L.h + 0.5 * (pl[1] * pl[1] + pl[2] * pl[2] + pl[3] * pl[3]);
  const T hr = Rs.h + 0.5 * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]);
  const T uull = nx * pl[1] + ny * pl[2] + nz * pl[3];
  const T uurr = nx * pr[1] + ny * pr[2] + nz * pr[3];
  if (c.nscheme == 1 || c.nscheme == 2) {
    T ravg_ht = (srl * hl + srr * hr) * ravg_d;
    T u2 = ravg[1] * ravg[1] + ravg[2] * ravg[2] + ravg[3] * ravg[3];
    T uuu = nx * ravg[1] + ny * ravg[2] + nz * ravg[3];
    if (c.nscheme == 1) {
      T sndp2 = sndp2_u<T>(c, rc2, u2, uref2);
      T q = sndp2 / rc2;
      T uup = 0.5 * (1.0 + q) * uuu;
      T ddd = 0.5 * sqrt((1.0 - q) * (1.0 - q) * uuu * uuu + 4.0 * sndp2);
      T c_star = 0.5 * (fabs(uup + ddd) + fabs(uup - ddd));
      T m_star = 0.5 * (fabs(uup + ddd) - fabs(uup - ddd)) / ddd;
      T du = m_star * (uurr - uull) + (c_star - q * fabs(uuu) - 0.5 * (1.0 - q) * uuu * m_star) * (pr[0] - pl[0]) / rrho / sndp2;
      T dp = m_star * (pr[0] - pl[0]) + (c_star - fabs(uuu) + 0.5 * (1.0 - q) * uuu * m_star) * rrho * (uurr - uull);
      T au = fabs(uuu);
      T df0 = au * (Rs.rho - L.rho) + du * rrho;
      fx[0] = 0.5 * (L.rho * uull + Rs.rho * uurr - df0) * dl;
      const double nn[3] = {nx, ny, nz};
      for (int q3 = 0; q3 < 3; ++q3) {
        T df = au * (Rs.rho * pr[1 + q3] - L.rho * pl[1 + q3]) + du * rrho * ravg[1 + q3] + dp * nn[q3];
        fx[1 + q3] = 0.5 * (L.rho * uull * pl[1 + q3] + nn[q3] * (pl[0] + pref) + Rs.rho * uurr * pr[1 + q3] +
                            nn[q3] * (pr[0] + pref) - df) * dl;
      }
      T df4 = au * (Rs.rho * hr - pr[0] - L.rho * hl + pl[0]) + du * rrho * ravg_ht + dp * uuu;
      fx[4] = 0.5 * (L.rho * uull * hl + Rs.rho * uurr * hr - df4) * dl;
      for (int k = 5; k < npv; ++k) {
        T df = au * (Rs.rho * pr[k] - L.rho * pl[k]) + du * rrho * ravg[k];
        fx[k] = 0.5 * (L.rho * uull * pl[k] + Rs.rho * uurr * pr[k] - df) * dl;
      }
      return;
    }
    // Roe-M
    T am2rmid_du = sndp2_du_u<T>(c, rc2, u2, uref2) / rc2;
    T am2rmid = sndp2_u<T>(c, rc2, u2, uref2) / rc2;
    T fmid = sqrt(am2rmid) * (2.0 - sqrt(am2rmid));
    T fmid_du = sqrt(am2rmid_du) * (2.0 - sqrt(am2rmid_du));
    T amid = sqrt(rc2);
    T b1 = fmax(fmax(0.0, uuu + amid), uurr + amid);
    T b2 = fmin(fmin(0.0, uuu - amid), uull - amid);
    T b1_du = fmax(fmax(0.0, uuu + fmid_du * amid), uurr + fmid_du * amid);
    T b2_du = fmin(fmin(0.0, uuu - fmid_du * amid), uull - fmid_du * amid);
    T m_tilde = copysign(1.0, uuu) * fmin(fabs(uuu) / amid, 1.0);
    T m_tilde_du = copysign(1.0, uuu) * fmin(fabs(uuu) / (fmid_du * amid), 1.0);
    T sd[18];
    T add0 = 0.1 * fmin(L.rho * L.c2, Rs.rho * Rs.c2);
    for (int k = 0; k < 18; ++k) sd[k] = sdst_in[k] + pref + add0;
    T ff = 1.0 - sdst_ratio_min<T>(sd);
    ff = (uuu != 0.0) ? pow(fabs(uuu) / amid, ff) : T(1.0);
    T gg = 1.0 - fmin(sd[8] / sd[9], sd[9] / sd[8]);
    gg = (uuu != 0.0) ? pow(fabs(uuu) / amid, gg) : T(1.0);
    T add = 1.0 + fabs(m_tilde), aaa = 1.0 + fabs(m_tilde_du);
    T dq[NPVM], fl[NPVM], fr[NPVM], bdq[NPVM];
    dq[0] = Rs.rho - L.rho;
    for (int k = 1; k <= 3; ++k) dq[k] = Rs.rho * pr[k] - L.rho * pl[k];
    dq[4] = Rs.rho * hr - L.rho * hl;
    for (int k = 5; k < npv; ++k) dq[k] = Rs.rho * pr[k] - L.rho * pl[k];
    const double nn[3] = {nx, ny, nz};
    fl[0] = L.rho * uull; fr[0] = Rs.rho * uurr;
    for (int q3 = 0; q3 < 3; ++q3) {
      fl[1 + q3] = L.rho * uull * pl[1 + q3] + nn[q3] * (pl[0] + pref);
      fr[1 + q3] = Rs.rho * uurr * pr[1 + q3] + nn[q3] * (pr[0] + pref);
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
  T amid = sqrt(rc2);
  T zmr = uurr / amid, zml = uull / amid;
  T fmid, fmid1, am2mid;
  if (c.nscheme == 3) {
    am2mid = ravg[1] * ravg[1] + ravg[2] * ravg[2] + ravg[3] * ravg[3];
    T a1 = sndp2_du_u<T>(c, rc2, am2mid, uref2) / rc2;
    T a0 = sndp2_u<T>(c, rc2, am2mid, uref2) / rc2;
    fmid = sqrt(a0) * (2.0 - sqrt(a0));
    fmid1 = sqrt(a1) * (2.0 - sqrt(a1));
  } else {
    T un = nx * ravg[1] + ny * ravg[2] + nz * ravg[3];
    am2mid = un * un;
    T a0 = sndp2_u<T>(c, rc2, am2mid, uref2) / rc2;
    fmid = sqrt(a0) * (2.0 - sqrt(a0));
    fmid1 = fmid;
  }
  T alpha = 3.0 / 16.0 * (-4.0 + 5.0 * fmid1 * fmid1);
  alpha = fmax(fmin(alpha, 3.0 / 16.0), -3.0 / 4.0);
  const double beta = 0.125;
  T zmmr, pmr, zmpl, ppl;
  if (fabs(zmr) >= 1.0) { zmmr = 0.5 * (zmr - fabs(zmr)); pmr = 0.5 * (1.0 - zmr / fabs(zmr)); }
  else {
    zmmr = -(0.25 * (zmr - 1.0) * (zmr - 1.0)) - beta * sq(zmr * zmr - 1.0);
    pmr = 0.25 * (zmr - 1.0) * (zmr - 1.0) * (2.0 + zmr) - alpha * zmr * sq(zmr * zmr - 1.0);
  }
  if (fabs(zml) >= 1.0) { zmpl = 0.5 * (zml + fabs(zml)); ppl = 0.5 * (1.0 + zml / fabs(zml)); }
  else {
    zmpl = 0.25 * (zml + 1.0) * (zml + 1.0) + beta * sq(zml * zml - 1.0);
    ppl = 0.25 * (zml + 1.0) * (zml + 1.0) * (2.0 - zml) + alpha * zml * sq(zml * zml - 1.0);
  }
  T zmpl1, zmmr1, pmid;
  if (c.nscheme == 3) {
    T zmid = zmpl + zmmr;
    pmid = ppl * (pl[0] + pref) + pmr * (pr[0] + pref) - 2.0 * ppl * pmr * rrho * fmid1 * amid * (uurr - uull);
    T sd[18];
    T add0 = 0.1 * fmin(L.rho * L.c2, Rs.rho * Rs.c2);
    for (int k = 0; k < 18; ++k) sd[k] = sdst_in[k] + pref + add0;
    T m1 = fmin(sd[8] / sd[9], sd[9] / sd[8]);
    T ww1 = 1.0 - m1 * m1 * m1;
    T m2 = sdst_ratio_min<T>(sd);
    T ww2 = 1.0 - m2 * m2;
    T ww = fmax(ww1, ww2);
    T pmt = rrho * rc2;
    T pwl = ((pl[0] + pref + rrho * rc2) / pmt - 1.0) * (1.0 - ww) / fmid;
    T pwr = ((pr[0] + pref + rrho * rc2) / pmt - 1.0) * (1.0 - ww) / fmid;
    if (zmid >= 0.0) {
      pwl = pwl * rrho / L.rho;
      pwr = pwr * rrho / L.rho;  // both weights scaled by the left density, as the reference does
      zmpl1 = zmpl + zmmr * ((1.0 - ww) * (1.0 + pwr) - pwl);
      zmmr1 = zmmr * ww * (1.0 + pwr);
    } else {
      pwl = pwl * rrho / Rs.rho;
      pwr = pwr * rrho / Rs.rho;
      zmpl1 = zmpl * ww * (1.0 + pwl);
      zmmr1 = zmmr + zmpl * ((1.0 - ww) * (1.0 + pwl) - pwr);
    }
  } else {
    const double kp = 0.25;
    T zmid = zmpl + zmmr - kp * fmax(1.0 - am2mid / rc2, 0.0) * (pr[0] - pl[0]) / rrho / rc2 / fmid;
    pmid = ppl * (pl[0] + pref) + pmr * (pr[0] + pref) - 2.0 * ppl * pmr * rrho * fmid * amid * (uurr - uull);
    if (zmid > 0.0) { zmpl1 = zmid; zmmr1 = 0.0; } else { zmmr1 = zmid; zmpl1 = 0.0; }
  }
  T ml = zmpl1 * amid * L.rho, mr = zmmr1 * amid * Rs.rho;
  fx[0] = (ml + mr) * dl;
  fx[1] = (ml * pl[1] + mr * pr[1] + pmid * nx) * dl;
  fx[2] = (ml * pl[2] + mr * pr[2] + pmid * ny) * dl;
  fx[3] = (ml * pl[3] + mr * pr[3] + pmid * nz) * dl;
  fx[4] = (ml * hl + mr * hr) * dl;
  for (int k = 5; k < npv; ++k) fx[k] = (ml * pl[k] + mr * pr[k]) * dl;
}


// FP64 face flux: the Roe-average EOS (only its sound speed is used,
// src/flux_module.f90:237,319,461,588), then the flux
template <bool MX = false>
__device__ inline void inviscid_flux(const Par& c, const double* n, const FaceState& L, const FaceState& Rs,
                                     const double* sdst_in, double* fx, unsigned long long* fb) {
  const int npv = c.npv;
  double dl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  if (dl == 0.0) {
    for (int k = 0; k < npv; ++k) fx[k] = 0.0;
    return;
  }
  double ravg[NPVM];
  roe_state<double>(npv, L, Rs, ravg);
  double rdv[NDV];
  deteos_simple<MX>(c.fluid, ravg[0] + c.pref, ravg[4], ravg[5], ravg[6], rdv, fb, ravg[5] != 0.0);
  inviscid_flux_core<double>(c, n, L, Rs, sdst_in, ravg, rdv[5], c.uref * c.uref, fx);
}

// ------------------------------------------------------------------ SST source
// k-omega SST production, destruction and cross diffusion of one cell (kwsst + calbigf +
// no_des, src/turbsource_module.f90:269-414) from the cell gradients gr[q][e] of
// (u, v, w, k, omega), the cell's k, omega, density, viscosity, eddy viscosity and wall
// distance.  r7, r8 are the residual contributions; the rest feeds the implicit
// coefficients.  Templated for the adjoint.
template <class T>
struct SstOut { T r7, r8, prod, dest, div, pkw, bigf, talpha, tbeta, strain; };

// the largest of the cell's grid spacings vol / (mean face area) per direction, from its
// six face vectors (the LES length of the DES variants)
template <class F>
__device__ __forceinline__ double grid_hmax(const F (*fa)[3], double vol) {
  double h = 0.0;
  for (int d = 0; d < 3; ++d) {
    const double a1 = ::sqrt((double)fa[2 * d][0] * fa[2 * d][0] + (double)fa[2 * d][1] * fa[2 * d][1] +
                             (double)fa[2 * d][2] * fa[2 * d][2]);
    const double a2 = ::sqrt((double)fa[2 * d + 1][0] * fa[2 * d + 1][0] + (double)fa[2 * d + 1][1] * fa[2 * d + 1][1] +
                             (double)fa[2 * d + 1][2] * fa[2 * d + 1][2]);
    h = ::fmax(h, vol / (0.5 * (a1 + a2)));
  }
  return h;
}

// calturblength (src/turbsource_module.f90:406-576): the length scale of the k destruction
// -- no_des (ides 0), sst_des (1), sst_ddes (2), sst_iddes (3), sst_s_iddes (4).  hmax: the
// largest grid spacing (metrics only); mu, mut the laminar and eddy viscosities.
template <class T>
__device__ __forceinline__ T sst_length(int ides, T kk, T oo, T bigf, T strain, T vort, double hmax, double y5,
                                        T mu, T mut) {
  const T tl_rans = sqrt(kk) / T(9.0) / oo * T(100.0);
  if (ides == 0) return tl_rans;
  if (ides == 1) return fmin(tl_rans, T(0.61 * hmax));
  const T cdes = T(0.78) * bigf + T(0.61) * (T(1.0) - bigf);
  const T den = T(0.41 * 0.41 * y5 * y5) * sqrt(T(0.5) * (strain + vort));
  if (ides == 2) {
    const T x = T(20.0) * ((mu + mut) / den);
    const T fd = T(1.0) - tanh(x * x * x);
    return tl_rans - fd * fmax(T(0.0), tl_rans - cdes * T(hmax));
  }
  const T tl_les = cdes * T(::fmin(0.15 * ::fmax(y5, hmax), hmax));
  const double alpha = 0.25 - y5 / hmax;
  const double fb = ::fmin(2.0 * ::exp(-9.0 * alpha * alpha), 1.0);
  const T rdt = mut / den, xt = T(20.0) * rdt;
  const T fdt = T(1.0) - tanh(xt * xt * xt);
  const T fd = fmax(T(1.0) - fdt, T(fb));
  if (ides == 4) return fd * tl_rans + (T(1.0) - fd) * tl_les;
  const T xl = T(25.0) * (mu / den), xl2 = xl * xl, xl4 = xl2 * xl2;
  const T fl = tanh(xl4 * xl4 * xl2);
  const T x3 = T(3.4969) * rdt;
  const T ft = tanh(x3 * x3 * x3);
  const T fe2 = T(1.0) - fmax(ft, fl);
  const double fe1 = (alpha >= 0.0) ? 2.0 * ::exp(-11.09 * alpha * alpha) : 2.0 * ::exp(-9.0 * alpha * alpha);
  const T fe = fe2 * T(::fmax(fe1 - 1.0, 0.0));
  return fd * (T(1.0) + fe) * tl_rans + (T(1.0) - fd) * tl_les;
}

// out-of-line copies for the residual kernels: the DES path keeps its code and registers
// off the RANS path
static __device__ __noinline__ double sst_length_d(int ides, double kk, double oo, double bigf, double strain, double vort,
                                            double hmax, double y5, double mu, double mut) {
  return sst_length<double>(ides, kk, oo, bigf, strain, vort, hmax, y5, mu, mut);
}
static __device__ __noinline__ float sst_length_f(int ides, float kk, float oo, float bigf, float strain, float vort,
                                           double hmax, double y5, float mu, float mut) {
  return sst_length<float>(ides, kk, oo, bigf, strain, vort, hmax, y5, mu, mut);
}

template <class T>
__device__ __forceinline__ SstOut<T> sst_source(const T (*gr)[3], T kk, T oo, T rho, T mu, T mut, double y5,
                                                double vol, int ides = 0, double hmax = 0.0) {
  const double c23 = 2.0 / 3.0, c59 = 5.0 / 9.0;
  SstOut<T> o;
  T dudx = gr[0][0], dudy = gr[0][1], dudz = gr[0][2];
  T dvdx = gr[1][0], dvdy = gr[1][1], dvdz = gr[1][2];
  T dwdx = gr[2][0], dwdy = gr[2][1], dwdz = gr[2][2];
  o.strain = 2.0 * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + sq(dudy + dvdx) + sq(dudz + dwdx) + sq(dvdz + dwdy);
  o.div = dudx + dvdy + dwdz;
  T prod = mut * (o.strain - c23 * o.div * o.div) - c23 * rho * kk * o.div;
  o.prod = fmin(prod, 0.9 * rho * kk * oo);
  o.pkw = gr[3][0] * gr[4][0] + gr[3][1] * gr[4][1] + gr[3][2] * gr[4][2];
  T cdkw = fmax(1.712 * rho / oo * o.pkw, T(1.0e-10));
  T term1 = sqrt(kk) / (0.09 * oo * y5);
  T term2 = 500.0 * mu / rho / (oo * y5 * y5);
  T term3 = (3.424 * rho * kk) / (cdkw * y5 * y5);
  T arg1 = fmin(fmax(term1, term2), term3);
  T a2 = arg1 * arg1;
  o.bigf = tanh(a2 * a2);
  o.talpha = o.bigf * c59 + (1.0 - o.bigf) * 0.44;
  o.tbeta = o.bigf * 0.075 + (1.0 - o.bigf) * 0.0828;
  T tl = sqrt(kk) / 9.0 / oo * 100.0;
  if (ides != 0) {
    const T vort = sq(dudy - dvdx) + sq(dudz - dwdx) + sq(dvdz - dwdy);
    if constexpr (std::is_same<T, double>::value) tl = sst_length_d(ides, kk, oo, o.bigf, o.strain, vort, hmax, y5, mu, mut);
    else tl = sst_length<T>(ides, kk, oo, o.bigf, o.strain, vort, hmax, y5, mu, mut);
  }
  o.dest = rho * pow(kk, 1.5) / tl;
  o.r7 = (o.prod - o.dest) * vol;
  o.r8 = (o.talpha * rho * (1.0 / mut) * o.prod - o.tbeta * rho * oo * oo + 1.712 * (1.0 - o.bigf) * rho * (1.0 / oo) * o.pkw) * vol;
  return o;
}

// k-epsilon source (t_kepsilon kepsilon, src/turbsource_module.f90:170-267): the production
// limited to 30 rho eps, the low-Re damping fe1, fe2 and the 2 mu |grad sqrt k|^2 terms, and
// the 2x2 implicit Jacobian itt with the reference's eigen-sign limiting.  gr: gradients
// of u, v, w; gsk: gradient of sqrt(k) (from the square roots of the face averages).
template <class T>
__device__ __forceinline__ void ke_source(const T (*gr)[3], const T* gsk, T kk, T ee, T rho, T mu, T mut, double vol,
                                          T* r, T* itt) {
  const double c23 = 2.0 / 3.0;
  const T dudx = gr[0][0], dudy = gr[0][1], dudz = gr[0][2];
  const T dvdx = gr[1][0], dvdy = gr[1][1], dvdz = gr[1][2];
  const T dwdx = gr[2][0], dwdy = gr[2][1], dwdz = gr[2][2];
  const T kkyy = gsk[0] * gsk[0] + gsk[1] * gsk[1] + gsk[2] * gsk[2];
  const T div = dudx + dvdy + dwdz;
  T prod = mut * (2.0 * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + sq(dudy + dvdx) + sq(dudz + dwdx) + sq(dvdz + dwdy) -
                  c23 * div * div) - c23 * rho * kk * div;
  const T re_t = rho * kk * kk / ee / mu;
  const T fe1 = 1.0 - exp(-sq(re_t / 40.0));
  const T fe2 = 1.0 - 2.0 / 9.0 * exp(-sq(re_t / 6.0));
  prod = fmin(prod, 30.0 * rho * ee);
  const T ki = 1.0 / kk, oi = 1.0 / ee;
  r[0] = (prod - rho * ee - 2.0 * mu * kkyy) * vol;
  r[1] = (1.5 * fe1 * prod * ee - 1.9 * fe2 * rho * ee * ee + 2.9556 * mu * ee * kkyy) * ki * vol;
  const T dpdk = 2.0 * prod * ki + c23 * rho * div;
  const T dpdo = -((prod + c23 * rho * kk * div) * oi);
  itt[0] = dpdk;
  itt[1] = dpdo - rho;
  itt[2] = (1.9 * fe2 * rho * ee * ee - 2.9556 * mu * ee * kkyy) * (ki * ki);
  itt[3] = (1.5 * fe1 * dpdo * ee + 1.5 * fe1 * prod - 3.8 * fe2 * rho * ee + 2.9556 * mu * kkyy) * ki;
  const T tr = itt[0] + itt[3], de = itt[0] * itt[3] - itt[1] * itt[2];
  const T sd = sqrt(fmax(0.25 * tr * tr - de, T(0.0)));
  const T l1 = copysign(T(1.0), 0.5 * tr + sd), l2 = copysign(T(1.0), 0.5 * tr - sd);
  const T f1 = (1.0 - 0.5 * (1.0 - l1)) - 0.5 * (1.0 - l1), f2 = (1.0 - 0.5 * (1.0 - l2)) - 0.5 * (1.0 - l2);
  itt[0] = itt[0] * f1; itt[1] = itt[1] * f1; itt[2] = itt[2] * f2; itt[3] = itt[3] * f2;
}

// k-epsilon eddy viscosity with its low-Re damping (t_eddy_ke kepsilon,
// src/eddy_module.f90: re_t, re_e from the wall distance y)
__device__ __forceinline__ double ke_eddy(double rho, double kk, double ee, double mu, double y) {
  const double re_t = rho * kk * kk / ee / mu;
  const double re_e = rho * ::pow(mu / rho * ee, 0.25) * y / mu;
  const double f_mu = (1.0 + 3.0 / ::pow(re_t, 3.0 / 4.0)) * (1.0 + 80.0 * ::exp(-re_e)) *
                      sq(1.0 - ::exp(-re_e / 43.0 - re_e * re_e / 330.0));
  return 0.09 * rho * kk * kk / ee * f_mu;
}

// ------------------------------------------------------------------ viscous flux
// Face viscous flux (vsflux_laminar / vsflux_turbulent, src/vsflux_module.f90:182-425)
// from the face gradients g[x|y|z][q] of (u, v, w, T, k, omega) and their face averages
// cc[q]; vis, con, emut, tcon are the face-averaged transport coefficients, rho the face
// density, ydns the face wall distance.  Templated for the adjoint.
template <class T>
__device__ __forceinline__ void vsflux_core(const Par& c, const double* nx, const T* gx, const T* gy, const T* gz,
                                            const T* cc, T vis, T con, T emut, T tcon, T rho, double ydns, T* fv) {
  const bool turb = (c.iturb >= -1);
  const double c23 = 2.0 / 3.0;
  T mu = turb ? (vis + emut) : vis;
  T div = gx[0] + gy[1] + gz[2];
  T txx = mu * (2.0 * gx[0] - c23 * div), tyy = mu * (2.0 * gy[1] - c23 * div), tzz = mu * (2.0 * gz[2] - c23 * div);
  T txy = mu * (gy[0] + gx[1]), txz = mu * (gz[0] + gx[2]), tyz = mu * (gz[1] + gy[2]);
  T kc = turb ? (con + tcon) : con;
  T uc = cc[0], vc = cc[1], wc = cc[2];
  fv[0] = T(0.0);
  fv[1] = txx * nx[0] + txy * nx[1] + txz * nx[2];
  fv[2] = txy * nx[0] + tyy * nx[1] + tyz * nx[2];
  fv[3] = txz * nx[0] + tyz * nx[1] + tzz * nx[2];
  fv[4] = nx[0] * (uc * txx + vc * txy + wc * txz + kc * gx[3]) + nx[1] * (uc * txy + vc * tyy + wc * tyz + kc * gy[3]) +
          nx[2] * (uc * txz + vc * tyz + wc * tzz + kc * gz[3]);
  fv[5] = T(0.0);
  fv[6] = T(0.0);
  if (turb && c.iturb == -1) {
    // k-epsilon: F1 = 0 with sigma_k = 1, sigma_eps = 1.3 (src/vsflux_module.f90:69-75,427-435)
    fv[7] = (vis + emut * 1.0) * (gx[4] * nx[0] + gy[4] * nx[1] + gz[4] * nx[2]);
    fv[8] = (vis + emut * (1.0 / 1.3)) * (gx[5] * nx[0] + gy[5] * nx[1] + gz[5] * nx[2]);
  } else if (turb) {
    T pkw = gx[4] * gx[5] + gy[4] * gy[5] + gz[4] * gz[5];
    T kf = cc[4], of = cc[5];
    T cdkw = fmax(1.712 * rho / of * pkw, T(1.0e-10));
    T term1 = sqrt(kf) / (0.09 * of * ydns);
    T term2 = 500.0 * vis / rho / (of * ydns * ydns);
    T term3 = (3.424 * rho * kf) / (cdkw * ydns * ydns);
    T arg1 = fmin(fmax(term1, term2), term3);
    T a2 = arg1 * arg1;
    T bigf = tanh(a2 * a2);
    T tdk = bigf * 0.85 + (1.0 - bigf) * 1.0;
    T tdo = bigf * 0.5 + (1.0 - bigf) * 0.856;
    fv[7] = (vis + emut * tdk) * (gx[4] * nx[0] + gy[4] * nx[1] + gz[4] * nx[2]);
    fv[8] = (vis + emut * tdo) * (gx[5] * nx[0] + gy[5] * nx[1] + gz[5] * nx[2]);
  }
}

// face gradient of one variable from its 18-cell stencil x (normal difference plus the
// 1/16-weighted transverse sums, src/vsflux_module.f90:200-230); ev, tv are the averaged
// transverse face vectors, vol the inverse mean volume
template <class T>
__device__ __forceinline__ void face_gradient(const T* x, const double* nx, const double* ev, const double* tv,
                                              double vol, T& gx, T& gy, T& gz, T& cc) {
  T dn = x[9] - x[8];
  T de = 0.0625 * (-x[0] - x[1] + x[4] + x[5] + 2.0 * (-x[6] - x[7] + x[10] + x[11]) - x[12] - x[13] + x[16] + x[17]);
  T dt = 0.0625 * (-x[0] - x[1] + x[12] + x[13] + 2.0 * (-x[2] - x[3] + x[14] + x[15]) - x[4] - x[5] + x[16] + x[17]);
  gx = (dn * nx[0] + de * ev[0] + dt * tv[0]) * vol;
  gy = (dn * nx[1] + de * ev[1] + dt * tv[1]) * vol;
  gz = (dn * nx[2] + de * ev[2] + dt * tv[2]) * vol;
  cc = 0.5 * (x[8] + x[9]);
}

// ------------------------------------------------------------------ cavitation
template <class T>
struct CavOutT { T r_c, r_v, icav[4]; };
using CavOut = CavOutT<double>;

// Mass-transfer rates r_c, r_v (times the volume) and the implicit coefficients icav of the
// five cavitation models; the free-stream speed uref and the coefficients c_v, c_c are
// arguments so that the adjoint can differentiate with respect to them.
template <class T>
__device__ inline CavOutT<T> cavsource_t(const Par& c, const T* pv2, const T* dv, double vol, T uref, T cvc,
                                         T ccc, const double* sat = nullptr) {
  // sat (optional): the saturation pressure p_sat(T) and temperature T_sat(P) evaluated in
  // FP64 by the caller (the mixed form's FP32 source keeps them FP64)
  CavOutT<T> o;
  o.r_c = T(T(0.0)); o.r_v = T(T(0.0));
  for (int q = 0; q < 4; ++q) o.icav[q] = T(T(0.0));
  if (pv2[4] >= T(647.096)) return o;
  const T dp_ref = T(2.0) / (T(c.rhoref) * uref * uref);
  const T t_ref = uref / T(c.l_chord);
  const T P = pv2[0] + T(c.pref);
  const T clamp_c = c.fix_cav_clamp ? pv2[5] : pv2[4];
  const T clamp_v = c.fix_cav_clamp ? (T(1.0) - pv2[5] - pv2[6]) : (T(1.0) - pv2[4] - pv2[5]);
  const T yl = T(1.0) - pv2[5] - pv2[6];
  T r_c, r_v;
  if (c.ncav == 1) {  // Merkle
    T pww = sat ? T(sat[0]) : h2o_pww(pv2[4]);
    T rho1 = T(1.0) / dv[0];
    T kc = ccc * dv[0] * dp_ref * t_ref, kv = cvc * dv[0] * dp_ref * t_ref;
    T dpc = fmax(P - pww, T(0.0)), dpv = fmax(pww - P, T(0.0));
    r_c = fmin(ccc * dv[0] * pv2[5] * dpc * dp_ref * t_ref, dv[0] * clamp_c);
    r_v = fmin(cvc * dv[0] * yl * dpv * dp_ref * t_ref, dv[0] * clamp_v);
    o.r_c = r_c * vol; o.r_v = r_v * vol;
    if (r_c != T(0.0)) {
      o.icav[0] = -(r_c * dv[6] * rho1) - kc * pv2[5];
      o.icav[1] = -(r_c * dv[7] * rho1);
      o.icav[2] = -(r_c * dv[8] * rho1) - kc * dpc;
      o.icav[3] = -(r_c * dv[9] * rho1);
    }
    if (r_v != T(0.0)) {
      o.icav[0] = r_v * dv[6] * rho1 - kv * yl;
      o.icav[1] = r_v * dv[7] * rho1;
      o.icav[2] = r_v * dv[8] * rho1 - kv * dpv;
      o.icav[3] = r_v * dv[9] * rho1 - kv * dpv;
    }
  } else if (c.ncav == 2) {  // Kunz
    T pww = sat ? T(sat[0]) : h2o_pww(pv2[4]);
    T rho1 = T(1.0) / dv[0];
    T av = dv[0] * pv2[5] / dv[3], ag = dv[0] * pv2[6] / dv[4], al = T(1.0) - av - ag;
    T dpv = fmax(pww - P, T(0.0));
    r_c = fmin(ccc * dv[3] * av * sq(al + ag) * t_ref, dv[0] * clamp_c);
    r_v = fmin(cvc * dv[0] * yl * dpv * dp_ref * t_ref, dv[0] * clamp_v);
    o.r_c = r_c * vol; o.r_v = r_v * vol;
    T av1 = T(1.0) - T(4.0) * av + T(3.0) * av * av;
    o.icav[0] = -(ccc * t_ref * (dv[6] * pv2[5] * av1 + T(2.0) * av * av * dv[14] * (al + ag)));
    o.icav[1] = -(ccc * t_ref * (dv[7] * pv2[5] * av1 + T(2.0) * av * av * dv[15] * (al + ag)));
    o.icav[2] = -(ccc * t_ref * (dv[8] * pv2[5] + dv[0]) * av1);
    o.icav[3] = -(ccc * t_ref * dv[9] * pv2[5] * av1);
    if (r_v != T(0.0)) {
      T kv = cvc * dv[0] * dp_ref * t_ref;
      o.icav[0] = r_v * dv[6] * rho1 - kv * yl;
      o.icav[1] = r_v * dv[7] * rho1;
      o.icav[2] = r_v * dv[8] * rho1 - kv * dpv;
      o.icav[3] = r_v * dv[9] * rho1 - kv * dpv;
    }
  } else if (c.ncav == 3) {  // Singhal
    T pww = sat ? T(sat[0]) : h2o_pww(pv2[4]);
    T sigma = h2o_sigma(pv2[4]);
    T rho1 = T(1.0) / dv[2], rho2 = T(1.0) / dv[3];
    T cc = ccc * uref / sigma * dv[2] * dv[3], cv = cvc * uref / sigma * dv[2] * dv[3];
    r_c = fmin(cc * sqrt(T(2.0) / T(3.0) * fmax(P - pww, T(0.0)) * rho1) * pv2[5], dv[0] * clamp_c);
    r_v = fmin(cv * sqrt(T(2.0) / T(3.0) * fmax(pww - P, T(0.0)) * rho1) * yl, dv[0] * clamp_v);
    o.r_c = r_c * vol; o.r_v = r_v * vol;
    if (r_c != T(0.0)) {
      o.icav[0] = -(r_c * (dv[14] * rho2 + T(0.5) * dv[16] * rho1)) - T(0.5) * cc * sqrt(T(2.0) / T(3.0) * rho1) * pv2[5] * pow(P - pww, -T(0.5));
      o.icav[1] = -(r_c * (dv[15] * rho2 + T(0.5) * dv[17] * rho1));
      o.icav[2] = -(cc * sqrt(T(2.0) / T(3.0) * fmax(P - pww, T(0.0)) * rho1));
      o.icav[3] = T(0.0);
    }
    if (r_v != T(0.0)) {
      o.icav[0] = r_v * (dv[14] * rho2 + T(0.5) * dv[16] * rho1) - T(0.5) * cv * sqrt(T(2.0) / T(3.0) * rho1) * yl * pow(pww - P, -T(0.5));
      o.icav[1] = r_v * (dv[15] * rho2 + T(0.5) * dv[17] * rho1);
      o.icav[2] = -(cv * sqrt(T(2.0) / T(3.0) * fmax(pww - P, T(0.0)) * rho1));
      o.icav[3] = o.icav[2];
    }
  } else if (c.ncav == 4) {  // Schnerr-Sauer
    const double pi = 3.14159265358979323846, eta = 1.0e13;
    T pww = sat ? T(sat[0]) : h2o_pww(pv2[4]);
    T rho1 = T(1.0) / dv[0], rho3 = T(1.0) / dv[2], rho4 = T(1.0) / dv[3];
    T k0 = T(3.0 * pow(4.0 * pi * eta / 3.0, 1.0 / 3.0) * sqrt(2.0 / 3.0));
    T base = k0 * dv[0] * pow(dv[3], T(1.0) / T(3.0)) * pow(dv[2], -T(5.0) / T(6.0)) * pow(yl, T(4.0) / T(3.0));
    r_c = fmin(ccc * base * pow(pv2[5], T(2.0) / T(3.0)) * sqrt(fmax(P - pww, T(0.0))), dv[0] * clamp_c);
    r_v = fmin(cvc * base * pow(pv2[5] + pv2[6], T(2.0) / T(3.0)) * sqrt(fmax(pww - P, T(0.0))), dv[0] * clamp_v);
    o.r_c = r_c * vol; o.r_v = r_v * vol;
    if (r_c != T(0.0)) {
      o.icav[0] = -(r_c * (dv[6] * rho1 + dv[14] * rho4 / T(3.0) - T(5.0) * dv[16] * rho3 / T(6.0) + T(0.5) / (P - pww)));
      o.icav[1] = -(r_c * (dv[7] * rho1 + dv[15] * rho4 / T(3.0) - T(5.0) * dv[17] * rho3 / T(6.0)));
      o.icav[2] = -(r_c * (dv[8] * rho1 + T(2.0) / (T(3.0) * pv2[5]) - T(4.0) / (T(3.0) * yl)));
      o.icav[3] = -(r_c * (dv[9] * rho1 - T(4.0) / (T(3.0) * yl)));
    }
    if (r_v != T(0.0)) {
      o.icav[0] = r_v * (dv[6] * rho1 + dv[14] * rho4 / T(3.0) - T(5.0) * dv[16] * rho3 / T(6.0) - T(0.5) / (pww - P));
      o.icav[1] = r_v * (dv[7] * rho1 + dv[15] * rho4 / T(3.0) - T(5.0) * dv[17] * rho3 / T(6.0));
      o.icav[2] = r_v * (dv[8] * rho1 + T(2.0) / (T(3.0) * (pv2[5] + pv2[6])) - T(4.0) / (T(3.0) * yl));
      o.icav[3] = r_v * (dv[9] * rho1 + T(2.0) / (T(3.0) * (pv2[5] + pv2[6])) - T(4.0) / (T(3.0) * yl));
    }
  } else {  // Lee
    T tww = sat ? T(sat[1]) : h2o_tww(P);
    T rho1 = T(1.0) / dv[0];
    r_c = fmin(ccc * dv[0] * pv2[5] * fmax(tww - pv2[4], T(0.0)) / tww, dv[0] * clamp_c);
    r_v = fmin(cvc * dv[0] * yl * fmax(pv2[4] - tww, T(0.0)) / tww, dv[0] * clamp_v);
    o.r_c = r_c * vol; o.r_v = r_v * vol;
    if (r_c != T(0.0)) {
      o.icav[0] = -(r_c * dv[6] * rho1);
      o.icav[1] = -(r_c * dv[7] * rho1) + ccc * dv[0] * pv2[5] / tww;
      o.icav[2] = -(r_c * dv[8] * rho1) - ccc * dv[0] * fmax(tww - pv2[4], T(0.0)) / tww;
      o.icav[3] = -(r_c * dv[9] * rho1);
    }
    if (r_v != T(0.0)) {
      o.icav[0] = r_v * dv[6] * rho1;
      o.icav[1] = r_v * dv[7] * rho1 + cvc * dv[0] * yl / tww;
      o.icav[2] = r_v * dv[8] * rho1 - cvc * dv[0] * fmax(pv2[4] - tww, T(0.0)) / tww;
      o.icav[3] = r_v * dv[9] * rho1 - cvc * dv[0] * fmax(pv2[4] - tww, T(0.0)) / tww;
    }
  }
  T lam = copysign(1.0, o.icav[2]);
  T f = (T(1.0) - T(0.5) * (T(1.0) - lam)) - T(0.5) * (T(1.0) - lam);
  for (int q = 0; q < 4; ++q) o.icav[q] *= f;
  return o;
}

__device__ inline CavOut cavsource(const Par& c, const double* pv2, const double* dv, double vol) {
  return cavsource_t<double>(c, pv2, dv, vol, c.uref, c.c_v, c.c_c);
}

// ------------------------------------------------------------------ diagonal operator
__device__ __forceinline__ double eigenvis_of(const Par& c, const double* dv, const double* tv) {
  if (c.iturb == -3) return 0.0;
  double den = dv[7] + dv[11] * dv[6] * dv[0] - dv[10] * dv[7] * dv[0];
  if (c.iturb == -2) return fmax(dv[6] * tv[1] / den, 4.0 / 3.0 * tv[0] / dv[0]);
  return fmax(dv[6] * (tv[1] + dv[11] * tv[2] / 0.9) / den, 4.0 / 3.0 * (tv[0] + tv[2]) / dv[0]);
}

// flowonly_ex / flowturball_ex (src/lhs_module.f90:247-344): the diagonal solve of the
// explicit schemes -- lhs%getx without spectral radii, viscous shift or source couplings,
// scaled by a = dt / vol
__device__ __forceinline__ void getx_explicit(const Par& c, const double* pv, const double* dv, const double* res,
                                              double dt, double vol, double* x) {
  const double a = dt / vol;
  const double bb = (c.nsteady == 1) ? 1.0 : 0.75;
  const double b = (c.nsteady >= 1) ? (double)c.nsteady * bb * vol / c.dt_phy * a : 0.0;
  const double b1 = 1.0 + b;
  const double i_b1 = 1.0 / (b1 * dv[0]);
  const double uv2 = pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3];
  const double isnd = 1.0 / sndp2_of<double>(c, dv[5], uv2), idv5 = 1.0 / dv[5];
  const double ss = dv[0] * dv[11] * (isnd + b * idv5);
  const double rr = isnd - idv5 + b1 * dv[6];
  const double hst = dv[1] + 0.5 * uv2 - uv2;
  const double cross1 = dv[12] * dv[7] - dv[11] * dv[8];
  const double cross2 = dv[13] * dv[7] - dv[11] * dv[9];
  const double dhdp1 = 1.0 - dv[10] * dv[0];
  const double ssy1 = dv[12] * dv[0] * rr + b1 * dv[8] * dhdp1;
  const double ssy2 = dv[13] * dv[0] * rr + b1 * dv[9] * dhdp1;
  const double ssh = dv[0] * rr * hst - b1 * dhdp1 * dv[0];
  const double aaa2 = dv[7] * hst + dv[11] * dv[0] - cross2 * pv[6];
  const double uuu = res[1] * pv[1] + res[2] * pv[2] + res[3] * pv[3] - res[4];
  const double coeff2 = res[0] * aaa2 + dv[7] * uuu + cross2 * res[6];
  const double coeff3 = res[0] * (ssh - ssy2 * pv[6]) + dv[0] * rr * uuu + res[6] * ssy2;
  const double mm = 1.0 / ss;
  x[0] = (coeff2 + cross1 * res[5] - cross1 * pv[5] * res[0]) * mm;
  x[1] = (res[1] - res[0] * pv[1]) * i_b1;
  x[2] = (res[2] - res[0] * pv[2]) * i_b1;
  x[3] = (res[3] - res[0] * pv[3]) * i_b1;
  x[4] = -(coeff3 - ssy1 * pv[5] * res[0] + res[5] * ssy1) * mm * i_b1;
  for (int v = 5; v < c.npv; ++v) x[v] = (res[v] - res[0] * pv[v]) * i_b1;
  for (int v = 0; v < c.npv; ++v) x[v] *= a;
}

// everything of lhs%getx that does not depend on the right-hand side (R = float: the mixed
// form's sweeps apply it to the neighbours' FP32 contribution)
template <class R>
struct DiagT {
  R a, b1, i_b1, ss, rr, cross, cross1, cross2, ssy1, ssy2, ssh, aaa1, aaa2, mm, c[4], tt, t[4];
};
using Diag = DiagT<double>;

// evis = eigenvis_of(c, dv, tv), which the caller also needs
// lam_fs (optional): the spectral radius lamda and the face-vector sum fs formed by the
// caller (the mixed form takes them in FP32: they only size the block)
template <class R>
__device__ __forceinline__ void diag_prepare_t(const Par& c, const R* pv, const R* dv, R evis,
                                               const R* fc /* cx1,cx2,ex1,ex2,tx1,tx2 x3 */, R vol, R dt,
                                               const R* icav, const R* itt, DiagT<R>& D,
                                               const float* lam_fs = nullptr) {
  // (the reference's repeated quotients are formed once: one reciprocal of c2, of the
  // preconditioned c2 and of the volume; the FP64 pipe is the scarce unit of a GB300)
  R uv2 = pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3];
  R sndp2 = sndp2_of<R>(c, dv[5], uv2);
  const R idv5 = R(1) / dv[5], isnd = R(1) / sndp2;
  const R qr = sndp2 * idv5, qh = R(0.5) * (R(1) + qr), qd = sq(R(1) - qr);
  const R cappa = R(1.05);
  R lamda = R(0), fs = R(0);
  if (lam_fs) { lamda = (R)lam_fs[0]; fs = (R)lam_fs[1]; }
  for (int d = 0; d < 3 && !lam_fs; ++d) {
    R ox = R(0.5) * (fc[6 * d + 0] + fc[6 * d + 3]);
    R oy = R(0.5) * (fc[6 * d + 1] + fc[6 * d + 4]);
    R oz = R(0.5) * (fc[6 * d + 2] + fc[6 * d + 5]);
    R ds = ox * ox + oy * oy + oz * oz;
    R u = ox * pv[1] + oy * pv[2] + oz * pv[3];
    R up = qh * u;
    R dd = R(0.5) * sqrt(u * u * qd + R(4) * sndp2 * ds);
    lamda += cappa * (fabs(up) + dd);
    fs += ds;  // 0.25*(f1+f2)^2 summed over the components
  }
  const R ivol = R(1) / vol;
  R ev = evis * fs;
  R bb = (c.nsteady == 1) ? R(1) : R(0.75);
  R a = R(1) / (vol / dt + lamda);
  R unst = (c.nsteady >= 1) ? (R)c.nsteady * bb * vol / (R)c.dt_phy : R(0);
  R b = (unst + R(2) * ev * ivol) * a;
  for (int q = 0; q < 4; ++q) { D.c[q] = icav[q] * vol * a; D.t[q] = itt[q] * vol * a; }
  D.a = a;
  D.b1 = R(1) + b;
  D.i_b1 = R(1) / (D.b1 * dv[0]);
  D.ss = dv[0] * dv[11] * (isnd + b * idv5);
  D.rr = isnd - idv5 + D.b1 * dv[6];
  R hst = dv[1] + R(0.5) * uv2 - uv2;
  D.cross = dv[13] * dv[8] - dv[12] * dv[9];
  D.cross1 = dv[12] * dv[7] - dv[11] * dv[8];
  D.cross2 = dv[13] * dv[7] - dv[11] * dv[9];
  R dhdp1 = R(1) - dv[10] * dv[0];
  D.ssy1 = dv[12] * dv[0] * D.rr + D.b1 * dv[8] * dhdp1;
  D.ssy2 = dv[13] * dv[0] * D.rr + D.b1 * dv[9] * dhdp1;
  D.ssh = dv[0] * D.rr * hst - D.b1 * dhdp1 * dv[0];
  D.aaa1 = dv[8] * hst + dv[12] * dv[0] - D.cross * pv[6];
  D.aaa2 = dv[7] * hst + dv[11] * dv[0] - D.cross2 * pv[6];
  D.mm = R(1) / (D.b1 * dv[0] * (D.ss + D.c[0] * D.cross1) - D.c[1] * D.ssy1 + D.c[2] * D.ss);
  D.tt = R(1) / (D.t[1] * D.t[2] - (D.t[0] + D.b1 * dv[0]) * (D.t[3] + D.b1 * dv[0]));
}
__device__ __forceinline__ void diag_prepare(const Par& c, const double* pv, const double* dv, double evis,
                                             const double* fc, double vol, double dt, const double* icav,
                                             const double* itt, Diag& D, const float* lam_fs = nullptr) {
  diag_prepare_t<double>(c, pv, dv, evis, fc, vol, dt, icav, itt, D, lam_fs);
}

// lhs%eigen (src/lhs_module.f90:459-496) in FP32: the spectral radius of the cell and the
// sum of its squared mean face vectors, from FP32 state and face vectors
__device__ __forceinline__ void diag_spectral_f(const Par& c, const float* pv, float c2, const float* fc,
                                                float* lam_fs) {
  const float uv2 = pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3];
  const float sndp2 = sndp2_of<float>(c, c2, uv2);
  const float qr = sndp2 / c2, qh = 0.5f * (1.0f + qr), qd = (1.0f - qr) * (1.0f - qr);
  float lamda = 0.0f, fs = 0.0f;
  for (int d = 0; d < 3; ++d) {
    const float ox = 0.5f * (fc[6 * d + 0] + fc[6 * d + 3]);
    const float oy = 0.5f * (fc[6 * d + 1] + fc[6 * d + 4]);
    const float oz = 0.5f * (fc[6 * d + 2] + fc[6 * d + 5]);
    const float ds = ox * ox + oy * oy + oz * oz;
    const float u = ox * pv[1] + oy * pv[2] + oz * pv[3];
    lamda += 1.05f * (fabsf(qh * u) + 0.5f * sqrtf(u * u * qd + 4.0f * sndp2 * ds));
    fs += ds;
  }
  lam_fs[0] = lamda;
  lam_fs[1] = fs;
}

// x = D^-1 res (lhs%getx)
template <class R>
__device__ __forceinline__ void diag_solve_t(const Par& c, const DiagT<R>& D, const R* pv, const R* dv, const R* res,
                                             R* x) {
  const R* C4 = D.c;
  R uuu = res[1] * pv[1] + res[2] * pv[2] + res[3] * pv[3] - res[4];
  R coeff1 = res[0] * D.aaa1 + dv[8] * uuu + D.cross * res[6];
  R coeff2 = res[0] * D.aaa2 + dv[7] * uuu + D.cross2 * res[6];
  R coeff3 = res[0] * (D.ssh - D.ssy2 * pv[6]) + dv[0] * D.rr * uuu + res[6] * D.ssy2;
  R r6 = res[6] - res[0] * pv[6];
  x[0] = (C4[3] * D.cross1 * (res[0] * pv[6] - res[6]) - C4[1] * coeff1 + C4[2] * coeff2 +
          dv[0] * D.b1 * (coeff2 + D.cross1 * res[5] - D.cross1 * pv[5] * res[0])) * D.mm;
  x[1] = (res[1] - res[0] * pv[1]) * D.i_b1;
  x[2] = (res[2] - res[0] * pv[2]) * D.i_b1;
  x[3] = (res[3] - res[0] * pv[3]) * D.i_b1;
  x[4] = (C4[3] * D.i_b1 * D.ssy1 * r6 + C4[0] * coeff1 - C4[2] * D.i_b1 * coeff3 -
          (coeff3 - D.ssy1 * pv[5] * res[0] + res[5] * D.ssy1)) * D.mm;
  x[5] = (D.ss * (res[5] - res[0] * pv[5]) - C4[3] * D.ss * D.i_b1 * r6 - C4[0] * coeff2 + C4[1] * D.i_b1 * coeff3) * D.mm;
  x[6] = r6 * D.i_b1;
  if (c.npv > 7) {
    R bd = D.b1 * dv[0];
    R r7 = res[7] - res[0] * pv[7], r8 = res[8] - res[0] * pv[8];
    x[7] = (r8 * D.t[1] - (bd + D.t[3]) * r7) * D.tt;
    x[8] = (r7 * D.t[2] - (bd + D.t[0]) * r8) * D.tt;
  }
  for (int n = 0; n < c.npv; ++n) x[n] *= D.a;
}
__device__ __forceinline__ void diag_solve(const Par& c, const Diag& D, const double* pv, const double* dv,
                                           const double* res, double* x) {
  diag_solve_t<double>(c, D, pv, dv, res, x);
}

// the Diag fields as an array (the sweep record's diagonal part)
constexpr int PREP_DIAG = 23;

template <class R>
__device__ __forceinline__ void diag_to_array(const DiagT<R>& D, R* o) {
  o[0] = D.a; o[1] = D.b1; o[2] = D.i_b1; o[3] = D.ss; o[4] = D.rr; o[5] = D.cross; o[6] = D.cross1;
  o[7] = D.cross2; o[8] = D.ssy1; o[9] = D.ssy2; o[10] = D.ssh; o[11] = D.aaa1; o[12] = D.aaa2; o[13] = D.mm;
  for (int q = 0; q < 4; ++q) { o[14 + q] = D.c[q]; o[19 + q] = D.t[q]; }
  o[18] = D.tt;
}
template <class R>
__device__ __forceinline__ void diag_from_array(const double* o, DiagT<R>& D) {
  D.a = (R)o[0]; D.b1 = (R)o[1]; D.i_b1 = (R)o[2]; D.ss = (R)o[3]; D.rr = (R)o[4]; D.cross = (R)o[5];
  D.cross1 = (R)o[6]; D.cross2 = (R)o[7]; D.ssy1 = (R)o[8]; D.ssy2 = (R)o[9]; D.ssh = (R)o[10]; D.aaa1 = (R)o[11];
  D.aaa2 = (R)o[12]; D.mm = (R)o[13];
  for (int q = 0; q < 4; ++q) { D.c[q] = (R)o[14 + q]; D.t[q] = (R)o[19 + q]; }
  D.tt = (R)o[18];
}

// spectral radius of the split Jacobian for one face: 1.05 (|u'| + d)
template <class R>
__device__ __forceinline__ R face_spectral(const Par& c, const R* nx, const R* pv, const R* dv) {
  R ds = nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2];
  R u = nx[0] * pv[1] + nx[1] * pv[2] + nx[2] * pv[3];
  R sndp2 = sndp2_of<R>(c, dv[5], pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3]);
  R up = R(0.5) * (R(1.0) + sndp2 / dv[5]) * u;
  R d = R(0.5) * sqrt(u * u * sq(R(1.0) - sndp2 / dv[5]) + R(4.0) * sndp2 * ds);
  return R(1.05) * (fabs(up) + d);
}

// acc += sign_acc * 0.5 * A dq with the precomputed spectral radius `spec`, beta and
// evv = 2 eigenvis / vol of the neighbour (same algebra as jac_apply); R = float is the
// mixed form's neighbour product
template <class R>
__device__ __forceinline__ void jac_apply_pre(int npv, const R* nx, const R* pv, const R* dv, R spec, R beta, R evv,
                                              R sign, const R* dq, R* acc) {
  R ds = nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2];
  R u = nx[0] * pv[1] + nx[1] * pv[2] + nx[2] * pv[3];
  R lamda = sign * spec;
  R vis = sign * evv * ds;
  R uuu = u + lamda + vis;
  R lv = lamda + vis;
  R r0 = (u * dv[6] + lamda * beta + vis * dv[6]) * dq[0] + nx[0] * dv[0] * dq[1] + nx[1] * dv[0] * dq[2] +
         nx[2] * dv[0] * dq[3] + (u * dv[7] + lv * dv[7]) * dq[4] + (u * dv[8] + lv * dv[8]) * dq[5] +
         (u * dv[9] + lv * dv[9]) * dq[6];
  R ru = dv[0] * uuu;
  R h = dv[1] + R(0.5) * (pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3]);
  R s = R(0.5) * sign;  // forward: +A+ ; backward: -A- (sign = -1 for both factors)
  acc[0] += s * r0;
  acc[1] += s * (pv[1] * r0 + nx[0] * dq[0] + ru * dq[1]);
  acc[2] += s * (pv[2] * r0 + nx[1] * dq[0] + ru * dq[2]);
  acc[3] += s * (pv[3] * r0 + nx[2] * dq[0] + ru * dq[3]);
  acc[4] += s * (ru * (dv[10] * dq[0] + pv[1] * dq[1] + pv[2] * dq[2] + pv[3] * dq[3] + dv[11] * dq[4] +
                       dv[12] * dq[5] + dv[13] * dq[6]) + h * r0 - lv * dq[0]);
  acc[5] += s * (pv[5] * r0 + ru * dq[5]);
  acc[6] += s * (pv[6] * r0 + ru * dq[6]);
  if (npv > 7) {
    acc[7] += s * (pv[7] * r0 + ru * dq[7]);
    acc[8] += s * (pv[8] * r0 + ru * dq[8]);
  }
}

// acc += sign_acc * A(sign) dq for the neighbour cell state (pv, dv, tv, vol) across face nx
__device__ __forceinline__ void jac_apply(const Par& c, const double* nx, double vol, const double* pv,
                                          const double* dv, const double* tv, double sign, const double* dq,
                                          double* acc, double sign_acc) {
  const double cappa = 1.05;
  double ds = nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2];
  double u = nx[0] * pv[1] + nx[1] * pv[2] + nx[2] * pv[3];
  double sndp2 = sndp2_of<double>(c, dv[5], pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3]);
  double up = 0.5 * (1.0 + sndp2 / dv[5]) * u;
  double d = 0.5 * sqrt(u * u * sq(1.0 - sndp2 / dv[5]) + 4.0 * sndp2 * ds);
  double lamda = sign * cappa * (fabs(up) + d);
  double vis = sign * 2.0 * eigenvis_of(c, dv, tv) * ds / vol;
  double beta = 1.0 / sndp2 - 1.0 / dv[5] + dv[6];
  double uuu = u + lamda + vis;
  double lv = lamda + vis;
  // row 1: a1..a7 (+ g, ge shifts)
  double r0 = (u * dv[6] + lamda * beta + vis * dv[6]) * dq[0] + nx[0] * dv[0] * dq[1] + nx[1] * dv[0] * dq[2] +
              nx[2] * dv[0] * dq[3] + (u * dv[7] + lv * dv[7]) * dq[4] + (u * dv[8] + lv * dv[8]) * dq[5] +
              (u * dv[9] + lv * dv[9]) * dq[6];
  double ru = dv[0] * uuu;
  double h = dv[1] + 0.5 * (pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3]);
  double y[NPVM];
  y[0] = r0;
  y[1] = pv[1] * r0 + nx[0] * dq[0] + ru * dq[1];
  y[2] = pv[2] * r0 + nx[1] * dq[0] + ru * dq[2];
  y[3] = pv[3] * r0 + nx[2] * dq[0] + ru * dq[3];
  y[4] = ru * (dv[10] * dq[0] + pv[1] * dq[1] + pv[2] * dq[2] + pv[3] * dq[3] + dv[11] * dq[4] + dv[12] * dq[5] +
               dv[13] * dq[6]) + h * r0 - lv * dq[0];
  y[5] = pv[5] * r0 + ru * dq[5];
  y[6] = pv[6] * r0 + ru * dq[6];
  if (c.npv > 7) {
    y[7] = pv[7] * r0 + ru * dq[7];
    y[8] = pv[8] * r0 + ru * dq[8];
  }
  double s = 0.5 * sign_acc;
  for (int n = 0; n < c.npv; ++n) acc[n] += s * y[n];
}

}  // namespace cfd
