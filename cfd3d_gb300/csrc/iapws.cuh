// iapws.cuh -- IAPWS-IF97 water/vapour property evaluation on the device.
//
// Replaces the per-phase routines of the reference EOS (src/eos_module.f90):
//   iapws97_l  (:1331-1374)  region 1, 34 terms
//   iapws97_v  (:1376-1461)  region 2 ideal (9) + residual (43), or the metastable-vapour
//                            set (9 + 13) when p > p_sat(T)
//   *_prop     (:1463-1659)  IAPWS viscosity / conductivity with the critical term off
//   h2o_pww    (:2266-2279)  saturation pressure, h2o_tww (:2340-2354), h2o_sigma (:2430-2439)
//   ideal / stiffened (:1236-1329)
//
// GB300 design: every exponent of the Gibbs sums is a compile-time constant (the term
// table is a constexpr array expanded by a fold expression), so each power x^I y^J is a
// short chain of multiplications shared by common subexpressions instead of the
// reference's runtime integer power per term.  The code is templated on the arithmetic
// type so the mixed form can evaluate the same sums in another precision.
//
// The reference multiplies by four literals written without a kind suffix, i.e.
// single-precision constants (src/eos_module.f90:1367,1370,1371,1457); they are kept.
#pragma once
#include <utility>

namespace cfd {

struct IJN { int i, j; double n; };

// IF97 region 1: (I, J, n)  -- the published coefficient table
constexpr IJN kR1[34] = {
    {0, -2, 0.14632971213167e0},   {0, -1, -0.84548187169114e0},  {0, 0, -0.37563603672040e1},
    {0, 1, 0.33855169168385e1},    {0, 2, -0.95791963387872e0},   {0, 3, 0.15772038513228e0},
    {0, 4, -0.16616417199501e-1},  {0, 5, 0.81214629983568e-3},   {1, -9, 0.28319080123804e-3},
    {1, -7, -0.60706301565874e-3}, {1, -1, -0.18990068218419e-1}, {1, 0, -0.32529748770505e-1},
    {1, 1, -0.21841717175414e-1},  {1, 3, -0.52838357969930e-4},  {2, -3, -0.47184321073267e-3},
    {2, 0, -0.30001780793026e-3},  {2, 1, 0.47661393906987e-4},   {2, 3, -0.44141845330846e-5},
    {2, 17, -0.72694996297594e-15}, {3, -4, -0.31679644845054e-4}, {3, 0, -0.28270797985312e-5},
    {3, 6, -0.85205128120103e-9},  {4, -5, -0.22425281908000e-5},  {4, -2, -0.65171222895601e-6},
    {4, 10, -0.14341729937924e-12}, {5, -8, -0.40516996860117e-6}, {8, -11, -0.12734301741641e-8},
    {8, -6, -0.17424871230634e-9}, {21, -29, -0.68762131295531e-18}, {23, -31, 0.14478307828521e-19},
    {29, -38, 0.26335781662795e-22}, {30, -39, -0.11947622640071e-22}, {31, -40, 0.18228094581404e-23},
    {32, -41, -0.93537087292458e-25}};

// IF97 region 2 ideal-gas part (J, n) as (0, J, n); the metastable set differs in n0, n1
constexpr IJN kR2I[9] = {{0, 0, -0.96927686500217e1}, {0, 1, 0.10086655968018e2},
                         {0, -5, -0.56087911283020e-2}, {0, -4, 0.71452738081455e-1},
                         {0, -3, -0.40710498223928e0}, {0, -2, 0.14240819171444e1},
                         {0, -1, -0.43839511319450e1}, {0, 2, -0.28408632460772e0},
                         {0, 3, 0.21268463753307e-1}};
constexpr IJN kR2MI[9] = {{0, 0, -0.96937268393049e1}, {0, 1, 0.10087275970006e2},
                          {0, -5, -0.56087911283020e-2}, {0, -4, 0.71452738081455e-1},
                          {0, -3, -0.40710498223928e0}, {0, -2, 0.14240819171444e1},
                          {0, -1, -0.43839511319450e1}, {0, 2, -0.28408632460772e0},
                          {0, 3, 0.21268463753307e-1}};
// IF97 region 2 residual part (I, J, n)
constexpr IJN kR2R[43] = {
    {1, 0, -0.17731742473213e-2},  {1, 1, -0.17834862292358e-1},  {1, 2, -0.45996013696365e-1},
    {1, 3, -0.57581259083432e-1},  {1, 6, -0.50325278727930e-1},  {2, 1, -0.33032641670203e-4},
    {2, 2, -0.18948987516315e-3},  {2, 4, -0.39392777243355e-2},  {2, 7, -0.43797295650573e-1},
    {2, 36, -0.26674547914087e-4}, {3, 0, 0.20481737692309e-7},   {3, 1, 0.43870667284435e-6},
    {3, 3, -0.32277677238570e-4},  {3, 6, -0.15033924542148e-2},  {3, 35, -0.40668253562649e-1},
    {4, 1, -0.78847309559367e-9},  {4, 2, 0.12790717852285e-7},   {4, 3, 0.48225372718507e-6},
    {5, 7, 0.22922076337661e-5},   {6, 3, -0.16714766451061e-10}, {6, 16, -0.21171472321355e-2},
    {6, 35, -0.23895741934104e2},  {7, 0, -0.59059564324270e-17}, {7, 11, -0.12621808899101e-5},
    {7, 25, -0.38946842435739e-1}, {8, 8, 0.11256211360459e-10},  {8, 36, -0.82311340897998e1},
    {9, 13, 0.19809712802088e-7},  {10, 4, 0.10406965210174e-18}, {10, 10, -0.10234747095929e-12},
    {10, 14, -0.10018179379511e-8}, {16, 29, -0.80882908646985e-10}, {16, 50, 0.10693031879409e0},
    {18, 57, -0.33662250574171e0}, {20, 20, 0.89185845355421e-24}, {20, 35, 0.30629316876232e-12},
    {20, 48, -0.42002467698208e-5}, {21, 21, -0.59056029685639e-25}, {22, 53, 0.37826947613457e-5},
    {23, 39, -0.12768608934681e-14}, {24, 26, 0.73087610595061e-28}, {24, 40, 0.55414715350778e-16},
    {24, 58, -0.94369707241210e-6}};
// metastable-vapour residual part (I, J, n)
constexpr IJN kR2MR[13] = {
    {1, 0, -0.73362260186506e-2}, {1, 2, -0.88223831943146e-1}, {1, 5, -0.72334555213245e-1},
    {1, 11, -0.40813178534455e-2}, {2, 1, 0.20097803380207e-2}, {2, 7, -0.53045921898642e-1},
    {2, 16, -0.76190409086970e-2}, {3, 4, -0.63498037657313e-2}, {3, 16, -0.86043093028588e-1},
    {4, 7, 0.75321581522770e-2},  {4, 10, -0.79238375446139e-2}, {5, 9, -0.22888160778447e-3},
    {5, 10, -0.26456501482810e-2}};

// IAPWS transport correlations: mu0/lambda0 denominators and the rho-T double series
__constant__ double kVisH[4] = {1.0, 0.978197, 0.579829, -0.202354};
__constant__ double kConL[4] = {1.0, 6.978267, 2.599096, -0.998254};
__constant__ double kVisHH[6][7] = {
    {0.5132047, 0.2151778, -0.2818107, 0.1778064, -0.0417661, 0.0, 0.0},
    {0.3205656, 0.7317883, -1.070786, 0.460504, 0.0, -0.01578386, 0.0},
    {0.0, 1.241044, -1.263184, 0.2340379, 0.0, 0.0, 0.0},
    {0.0, 1.476783, 0.0, -0.4924179, 0.1600435, 0.0, -0.003629481},
    {-0.7782567, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {0.1885447, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}};
__constant__ double kConLL[5][6] = {
    {1.3293046, -0.40452437, 0.24409490, 0.018660751, -0.12961068, 0.044809953},
    {1.7018363, -2.2156845, 1.6511057, -0.76736002, 0.37283344, -0.11203160},
    {5.2246158, -10.124111, 4.9874687, -0.27297694, -0.43083393, 0.13333849},
    {8.7127675, -9.5000611, 4.3786606, -0.91783782, 0.0, 0.0},
    {-1.8525999, 0.93404690, 0.0, 0.0, 0.0, 0.0}};

// ---- compile-time powers ----------------------------------------------------------
template <int N, class T>
__device__ __forceinline__ T cpow(T x, T xi) {
  if constexpr (N == 0) return T(1.0);
  else if constexpr (N < 0) return cpow<-N>(xi, x);
  else if constexpr (N == 1) return x;
  else {
    T h = cpow<N / 2>(x, xi);
    if constexpr (N % 2) return h * h * x;
    else return h * h;
  }
}

// Gibbs-sum accumulator: g_x = dg/dx, g_xx, g_y, g_yy, g_xy of g = sum n x^I y^J
template <class T>
struct GAcc { T x, xx, y, yy, xy; };

template <class T, const IJN* TAB, size_t K, bool FULL>
__device__ __forceinline__ void gterm(T x, T xi, T y, T yi, GAcc<T>& a) {
  constexpr int I = TAB[K].i;
  constexpr int J = TAB[K].j;
  constexpr double n = TAB[K].n;
  // t = n x^I y^J ; derivatives through the reference's recurrences g1..g5
  T t = T(n) * cpow<I>(x, xi) * cpow<J>(y, yi);
  if constexpr (I != 0) {
    T tx = T(double(I)) * t * xi;
    a.x += tx;
    if constexpr (FULL && I != 1) a.xx += T(double(I - 1)) * tx * xi;
    if constexpr (FULL && J != 0) a.xy += T(double(J)) * tx * yi;
  }
  if constexpr (J != 0) {
    T ty = T(double(J)) * t * yi;
    a.y += ty;
    if constexpr (FULL && J != 1) a.yy += T(double(J - 1)) * ty * yi;
  }
}

// Scalar types that evaluate the Gibbs sums by parts (the adjoint's dual numbers, which
// specialise this trait): the sums and their derivatives are accumulated in plain FP64 and
// the dual results formed once, instead of carrying the derivatives through every term.
template <class T>
struct GibbsByParts { static constexpr bool value = false; };

template <class T, const IJN* TAB, bool FULL = true, size_t... K>
__device__ __forceinline__ void gsum(T x, T xi, T y, T yi, GAcc<T>& a, std::index_sequence<K...>) {
  if constexpr (GibbsByParts<T>::value) {
    GibbsByParts<T>::template sum<TAB, K...>(x, xi, y, yi, a);
  } else {
    (gterm<T, TAB, K, FULL>(x, xi, y, yi, a), ...);
  }
}

template <class T>
struct Phase { T rho, h, drdp, drdt, dhdp, dhdt; };

// IF97 saturation pressure
template <class T>
__device__ __forceinline__ T h2o_pww(T t) {
  T tt = fmin(fmax(t, T(273.15)), T(647.096));
  T theta = tt - T(0.23855557567849) / (tt - T(0.65017534844798e3));
  T a = theta * theta + T(0.11670521452767e4) * theta - T(0.72421316703206e6);
  T b = -(T(0.17073846940092e2) * (theta * theta)) + T(0.12020824702470e5) * theta - T(0.32325550322333e7);
  T c = T(0.14915108613530e2) * (theta * theta) - T(0.48232657361591e4) * theta + T(0.40511340542057e6);
  T q = T(2.0) * c / (-b + sqrt(b * b - T(4.0) * a * c));
  T q2 = q * q;
  return T(1.0e6) * (q2 * q2);
}

// p > p_sat(T) -- the metastable-branch test of the vapour phase -- decided as the FP64
// comparison decides it: the FP32 saturation pressure first (its relative error stays
// below 7e-6 over 273-647 K), the FP64 one only where p lies within 1e-4 of it.  (An FP64
// saturation pressure is a division, a square root and a quotient on the FP64 pipe.)
__device__ __forceinline__ bool above_psat(double p, double t) {
  const float psf = h2o_pww<float>((float)t), pf = (float)p;
  if (fabsf(pf - psf) > 1.0e-4f * psf) return pf > psf;
  return p > h2o_pww<double>(t);
}

template <class T>
__device__ __forceinline__ T h2o_tww(T p) {
  T beta = pow(p / T(1.0e6), T(0.25));
  T e = beta * beta - T(0.17073846940092e2) * beta + T(0.14915108613530e2);
  T f = T(0.11670521452767e4) * (beta * beta) + T(0.12020824702470e5) * beta - T(0.48232657361591e4);
  T g = -(T(0.72421316703206e6) * (beta * beta)) - T(0.32325550322333e7) * beta + T(0.40511340542057e6);
  T d = T(2.0) * g / (-f - sqrt(f * f - T(4.0) * e * g));
  T s = T(0.65017534844798e3) + d;
  return T(0.5) * (T(0.65017534844798e3) + d - sqrt(s * s - T(4.0) * (T(-0.23855557567849) + T(0.65017534844798e3) * d)));
}

template <class T>
__device__ __forceinline__ T h2o_sigma(T t) {
  T t2 = t * t, t3 = t2 * t, t4 = t2 * t2, t5 = t4 * t;
  return T(0.0881130429998226) + T(0.0000616475914044782) * t - T(4.4860167748009e-7) * t2 +
         T(2.53682468718936e-10) * t3 - T(2.62005668908913e-13) * t4 + T(2.97878955533757e-16) * t5;
}

// region 1 (liquid); FULL = false evaluates only rho and h
template <class T, bool FULL = true>
__device__ __forceinline__ void iapws_l(T p, T t, Phase<T>& e) {
  T pi = p * T(0.00000006049607);
  T tau = T(1386.0) / t;
  T x = T(7.1) - pi, xi = T(1.0) / x;
  T y = tau - T(1.222), yi = T(1.0) / y;
  GAcc<T> a = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
  gsum<T, kR1, FULL>(x, xi, y, yi, a, std::make_index_sequence<34>{});
  // d/dpi = -d/dx
  T gp = -a.x, gpp = a.xx, gt = a.y, gtt = a.yy, gpt = -a.xy;
  T gp1 = T(1.0) / gp;
  e.rho = T((double)25.841246054191803727f) * tau * gp1;
  e.h = T(639675.036) * gt;
  if constexpr (!FULL) return;
  e.drdp = -(gpp * T(1.5632937721834122e-6) * tau * (gp1 * gp1));
  e.drdt = -(e.rho * T(7.215007215007215e-4) * tau) + T((double)0.01864447767257706f) * gpt * (tau * tau * tau) * (gp1 * gp1);
  e.dhdp = T((double)0.03869782431941923775f) * gpt;
  e.dhdt = -(T(461.526) * (tau * tau) * gtt);
}

// region 2 / metastable vapour; `meta` = p > p_sat(T) selects the metastable set
template <class T, bool FULL = true>
__device__ __forceinline__ void iapws_v_meta(T p, T t, bool meta, Phase<T>& e) {
  T pi = p * T(1e-6);
  T tau = T(540.0) / t;
  T pi1 = T(1.0e6) / p;
  T taui = T(1.0) / tau;
  T y = tau - T(0.5), yi = T(1.0) / y;
  GAcc<T> id = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
  GAcc<T> rs = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
  if (meta) {
    gsum<T, kR2MI, FULL>(pi, pi1, tau, taui, id, std::make_index_sequence<9>{});
    gsum<T, kR2MR, FULL>(pi, pi1, y, yi, rs, std::make_index_sequence<13>{});
  } else {
    gsum<T, kR2I, FULL>(pi, pi1, tau, taui, id, std::make_index_sequence<9>{});
    gsum<T, kR2R, FULL>(pi, pi1, y, yi, rs, std::make_index_sequence<43>{});
  }
  T g0p = pi1, g0pp = -(pi1 * pi1);
  T gp = g0p + rs.x, gpp = g0pp + rs.xx, gt = id.y + rs.y, gtt = id.yy + rs.yy, gpt = rs.xy;
  T gp1 = T(1.0) / gp;
  e.rho = T(4.01245401527075799) * tau * gp1;
  e.h = T(249224.04) * gt;
  if constexpr (!FULL) return;
  e.drdp = -(gpp * T(4.01245401527075799e-6) * tau * (gp1 * gp1));
  e.drdt = -(e.rho * T((double)0.00185185185185185185f) * tau) +
           T((double)0.0074304703986495518f) * gpt * (tau * tau * tau) * (gp1 * gp1);
  e.dhdp = T(0.24922404) * gpt;
  e.dhdt = -(T(461.526) * (tau * tau) * gtt);
}


template <class T>
__device__ __forceinline__ void ideal_gas(T p, T t, Phase<T>& e) {
  const T r1 = T(0.00348383500557);
  T tau = T(1.0) / t;
  e.rho = p * r1 * tau;
  e.h = T(1004.64) * t;
  e.drdp = r1 * tau;
  e.drdt = -(p * r1 * (tau * tau));
  e.dhdp = T(0.0);
  e.dhdt = T(1004.64);
}

template <class T>
__device__ __forceinline__ void stiffened(T p, T t, Phase<T>& e) {
  const T r1 = T(0.00037160906726);
  T tau = T(1.0) / t;
  e.rho = (p + T(8.5e8)) * r1 * tau;
  e.h = T(4186.0) * t - T(917822.36);
  e.drdp = r1 * tau;
  e.drdt = -((p + T(8.5e8)) * r1 * (tau * tau));
  e.dhdp = T(0.0);
  e.dhdt = T(4186.0);
}

template <class T>
__device__ __forceinline__ T ideal_vis(T t) {
  return T(1.716e-5) * pow(t / T(273.11), T(1.5)) * T(383.67) / (t + T(110.56));
}
template <class T>
__device__ __forceinline__ T stiffened_vis(T t) {
  T temp = fmax(T(273.0), t);
  T r = T(273.0) / temp;
  return T(1.788e-3) * exp(T(-1.704) - T(5.306 * 273.0) / temp + T(7.003) * (r * r));
}

// IAPWS viscosity and conductivity (critical enhancement off, as in the reference)
template <class T>
__device__ __forceinline__ void iapws_transport(T t, T rho, T& vis, T& cond) {
  T tt = t * T(0.00154495032985);
  T rr = fmax(T(1.0e-3), fmin(T(1332.4), rho)) * T(0.00314699949333);
  T tt1 = T(647.27) / t;
  T a = tt1 - T(1.0), b = rr - T(1.0);
  T st = sqrt(tt);
  T mu0 = st / (T(kVisH[0]) + T(kVisH[1]) * tt1 + T(kVisH[2]) * (tt1 * tt1) + T(kVisH[3]) * (tt1 * tt1 * tt1));
  T mu1 = T(0.0);
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    T row = T(0.0);
#pragma unroll
    for (int j = 6; j >= 0; --j) row = row * b + T(kVisHH[i][j]);
    mu1 = mu1 * a + row;
  }
  vis = T(55.071e-6) * mu0 * exp(rr * mu1);
  T lam0 = st / (T(kConL[0]) + T(kConL[1]) * tt1 + T(kConL[2]) * (tt1 * tt1) + T(kConL[3]) * (tt1 * tt1 * tt1));
  T lam1 = T(0.0);
#pragma unroll
  for (int i = 4; i >= 0; --i) {
    T row = T(0.0);
#pragma unroll
    for (int j = 5; j >= 0; --j) row = row * b + T(kConLL[i][j]);
    lam1 = lam1 * a + row;
  }
  cond = T(0.4945) * (lam0 * exp(rr * lam1));
}

}  // namespace cfd
