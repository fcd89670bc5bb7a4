// flux_mixed.cu -- face fluxes of the mixed-precision form (CFD3D_MIXED).
//
//   k_shadow          FP32 gauge shadow pvf of every padded cell, after the boundary program,
//                     and the cell's EOS state as the base of face-state expansions (lqf)
//   k_recon_mx<DIR>   per face: MUSCL / MLP on pvf, clips, face-state rho and h (FP64
//                     mixture of phases from df64 IF97 sums, or for a vapour-free state
//                     near its cell the liquid by first-order expansion), written to the
//                     face record frec
//   k_flux_mx<DIR>    per face: FP32 Roe-average sound speed, inviscid flux with FP64
//                     leading-order terms; stores F - Phi.n dl in FP32
//   k_visc_mx<DIR>    per face: the FP32 viscous flux
// Splitting reconstruction + EOS from the flux keeps each kernel's code within the
// instruction cache (the expanded df64 Gibbs sums are large) and its registers low.
// Same faces, stencils and formulas as the FP64 form (flux.cu); the precision choices are
// listed in mixed.cuh.
#include "engine.cuh"
#include "mixed.cuh"

namespace cfd {

// whether padded cell g is an interior cell of its block (padded index (i + 1) + ni ((j + 1)
// + nj (k + 1)) from the block's first cell, interior i = 2 .. imax and so on)
__device__ __forceinline__ bool padded_interior(const DevPtr& d, long long g) {
  const BlockGeom& B = d.blk[find_block_cell(d.blk, d.nblk, g)];
  const long long l = g - B.off, r = l / B.ni;
  const int li = (int)(l - r * B.ni), lj = (int)(r % B.nj), lk = (int)(r / B.nj);
  return li >= 3 && li <= B.imax + 1 && lj >= 3 && lj <= B.jmax + 1 && lk >= 3 && lk <= B.kmax + 1;
}

// Per padded cell: the FP32 gauge shadow, and (interior cells) its EOS state as the base of
// the face states' expansion.  The kernel is mostly casts of FP64 state to FP32: they run on
// the integer pipes (to_f32, to_f64), and the liquid's 1/rho in FP32, to spare the FP64
// pipe.  With y1 = 0 the mixture holds only liquid and gas, so the liquid's 1/rho and h
// follow from dv: 1/rho_l = 1/dv(3), h_l = h - y2 (h_g - h_l), and its derivatives
// d(1/rho_l)/d(p, T) = -drho_l/d(p, T) / rho_l^2, dh_l/dp = dh/dp / (1 - y2) (the gas's h
// does not depend on p) and dh_l/dT = (dh/dT - y2 cp_g) / (1 - y2).  The mixture's rho -
// rhoref and h - href are formed in FP64 and stored in FP32, as the face records keep them.
__global__ void __launch_bounds__(256) k_shadow(DevPtr d, Par c, long long g0, long long g1) {
  const long long n = d.ncell;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int npv = c.npv;
  const double off[NPVM] = {0.0, c.uref_vec[0], c.uref_vec[1], c.uref_vec[2], c.tref, 0.0, 0.0, 0.0, 0.0};
  for (long long g = g0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; g < g1; g += stride) {
    float sh[NPVM];
#pragma unroll
    for (int v = 0; v < NPVM; ++v) {
      if (v < npv) {
        sh[v] = to_f32(d.pv[v * n + g] - off[v]);
        d.pvf[v * n + g] = sh[v];
      }
    }
    // the expansion base only at interior cells: a face state's base is always one (its own
    // side's cell, or at a block face the cell across it)
    if (!padded_interior(d, g)) continue;
    float q[NLQ];
#pragma unroll
    for (int m = 0; m < NLQ; ++m) q[m] = 0.0f;
    const double y1 = d.pv[5 * n + g], rl = d.dv[2 * n + g];
    if (c.fluid == 2 && y1 == 0.0 && rl > 0.0) {
      const double y2 = d.pv[6 * n + g], rho = d.dv[g], h = d.dv[n + g];
      const float ilf = 1.0f / to_f32(rl), iyl = 1.0f / (1.0f - to_f32(y2));
      q[LQ_VP] = -to_f32(d.dv[16 * n + g]) * ilf * ilf;
      q[LQ_VT] = -to_f32(d.dv[17 * n + g]) * ilf * ilf;
      q[LQ_HP] = to_f32(d.dv[10 * n + g]) * iyl;
      q[LQ_HT] = (to_f32(d.dv[11 * n + g]) - to_f32(y2) * 1004.64f) * iyl;
      q[LQ_RP] = to_f32(d.pv[g] - to_f64(sh[0]));
      q[LQ_RT] = to_f32((d.pv[4 * n + g] - c.tref) - to_f64(sh[4]));
      q[LQ_RDEV] = to_f32(rho - c.rhoref);
      q[LQ_HDEV] = to_f32(h - c.href);
      q[LQ_RHO] = to_f32(rho);
      q[LQ_VL] = ilf;
      q[LQ_HLG] = -to_f32(d.dv[13 * n + g]);   // h_l - h_g = -(dh/dy2)
    }
#pragma unroll
    for (int m = 0; m < NLQ; ++m) d.lqf[m * n + g] = q[m];
  }
}

// A vapour-free face state (gauge shadow x: y1 = 0) by first-order expansion about its base
// cell b (shadow xb), in FP32 throughout: the liquid's 1/rho and h are expanded in (p, T),
// the gas's are exact (ideal gas), and the mixture's change from the base,
//   dv = (1 - y2) dv_l + dy2 (v_g - v_l) + y2_b dv_g,   drho = -rho^2 dv / (1 + rho dv),
//   dh = (1 - y2) dh_l + dy2 (h_g - h_l) + y2_b cp_g dT,
// is added to the base's rho - rhoref and h - href, which is what the face record keeps.
// The expansion's error stays below that record's FP32 rounding when |dp| <= 2e4 Pa and
// |dT| <= 0.02 K (the second derivatives of IF97 region 1 near 300 K: d2rho/dp2 ~ rho kappa^2,
// d2rho/dT2 ~ -0.01 kg/m^3/K^2, d2h/dp2 ~ -v kappa, dcp/dT ~ -0.3 J/kg/K^2).  Returns false
// -- the caller evaluates the IF97 sums -- when the base carries vapour or the state is
// farther away.
__device__ __forceinline__ bool liquid_expand(const DevPtr& d, const Par& c, long long b, const float* x,
                                              float xb0, float xb4, float xb6, float& rdev, float& hdev) {
  const long long n = d.ncell;
  const float rho = d.lqf[LQ_RHO * n + b];
  if (rho == 0.0f) return false;
  const float dp = (x[0] - xb0) - d.lqf[LQ_RP * n + b];
  const float dt = (x[4] - xb4) - d.lqf[LQ_RT * n + b];
  if (!(fabsf(dp) <= 2.0e4f && fabsf(dt) <= 0.02f)) return false;
  const float dvl = d.lqf[LQ_VP * n + b] * dp + d.lqf[LQ_VT * n + b] * dt;
  const float dhl = d.lqf[LQ_HP * n + b] * dp + d.lqf[LQ_HT * n + b] * dt;
  // the gas: 1/rho_g = T / (p r1), h_g = cp_g T; base state from its shadow and roundings
  const float r1 = 0.00348383500557f, cpg = 1004.64f;
  const float pb = (float)c.pref + xb0 + d.lqf[LQ_RP * n + b];
  const float tb = (float)c.tref + xb4 + d.lqf[LQ_RT * n + b];
  const float pf = pb + dp, tf = tb + dt;
  const float vgf = tf / (pf * r1);
  const float dvg = (dt * pb - tb * dp) / (pf * pb * r1);
  const float y2b = xb6, y2f = x[6], dy2 = y2f - y2b;
  const float dv = (1.0f - y2f) * dvl + dy2 * (vgf - d.lqf[LQ_VL * n + b]) + y2b * dvg;
  rdev = d.lqf[LQ_RDEV * n + b] - rho * rho * dv / (1.0f + rho * dv);
  const float hgl = -d.lqf[LQ_HLG * n + b] + cpg * dt;   // h_g(face) - h_l(base)
  hdev = d.lqf[LQ_HDEV * n + b] + ((1.0f - y2f) * dhl + dy2 * hgl + y2b * cpg * dt);
  return true;
}

// face of direction DIR for thread t: left cell g, the stencil strides, and whether the
// left and right cells are interior cells
struct FaceIdx {
  long long g, sn, s1, s2;
  bool ok, lin, rin;
};
template <int DIR>
__device__ __forceinline__ FaceIdx face_of(const DevPtr& d, long long t) {
  FaceIdx f{};
  int b = 0;
  while (b + 1 < d.nblk && t >= d.blk[b + 1].face_off[DIR]) ++b;
  const BlockGeom& B = d.blk[b];
  long long loc = t - B.face_off[DIR];
  int fi_, fj, fk;
  if (DIR == 0) { fi_ = B.imax; fj = B.jmax - 1; fk = B.kmax - 1; }
  else if (DIR == 1) { fi_ = B.imax - 1; fj = B.jmax; fk = B.kmax - 1; }
  else { fi_ = B.imax - 1; fj = B.jmax - 1; fk = B.kmax; }
  f.ok = !(loc < 0 || loc >= (long long)fi_ * fj * fk);
  if (!f.ok) return f;
  int i = (int)(loc % fi_) + (DIR == 0 ? 1 : 2);
  long long r = loc / fi_;
  int j = (int)(r % fj) + (DIR == 1 ? 1 : 2);
  int k = (int)(r / fj) + (DIR == 2 ? 1 : 2);
  const long long si = 1, sj = B.ni, sk = (long long)B.ni * B.nj;
  f.g = B.off + (i + 1) + sj * (j + 1) + sk * (k + 1);
  const int fn = (DIR == 0) ? i : (DIR == 1 ? j : k), nmax = (DIR == 0) ? B.imax : (DIR == 1 ? B.jmax : B.kmax);
  f.lin = fn >= 2;
  f.rin = fn + 1 <= nmax;
  if (DIR == 0) { f.sn = si; f.s1 = sj; f.s2 = sk; }
  else if (DIR == 1) { f.sn = sj; f.s1 = sk; f.s2 = si; }
  else { f.sn = sk; f.s1 = si; f.s2 = sj; }
  return f;
}

// The MUSCL / MLP reconstruction of the j (DIR 1) or k (DIR 2) faces by columns of cells:
// thread (v, i, t) walks the faces of its column along the face normal and keeps the reduced
// stencil of muscl_reduced in registers -- per plane of cells the centre, the two transverse
// differences and the 3 x 3 minimum and maximum -- so each step loads the one new 3 x 3 plane
// instead of the face's 38 cells, and the planes' minima serve the four faces that read them.
// The warp runs along i, so every plane load is a coalesced row.  Writes the face states,
// before the clips, into frec; k_recon_mx<DIR, true> clips them and forms the face EOS.
template <int DIR>
__global__ void __launch_bounds__(128) k_muscl_march(DevPtr d, Par c, long long c0, long long c1) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x, ncol = c1 - c0;
  const int v = (int)(t / ncol);
  if (v >= c.npv) return;
  const long long col = c0 + (t - (long long)v * ncol);
  int b = 0;
  while (b + 1 < d.nblk && col >= d.blk[b + 1].col_off[DIR]) ++b;
  const BlockGeom& B = d.blk[b];
  const long long loc = col - B.col_off[DIR];
  const int i = (int)(loc % (B.imax - 1)) + 2;
  const int o = (int)(loc / (B.imax - 1)) + 2;   // k (DIR 1) or j (DIR 2) of the column
  const long long n = d.ncell, sj = B.ni, sk = (long long)B.ni * B.nj;
  // normal, first and second transverse strides, as stencil_cell numbers the stencil
  const long long sn = DIR == 1 ? sj : sk, s1 = DIR == 1 ? sk : 1, s2 = DIR == 1 ? 1 : sj;
  const int nmax = DIR == 1 ? B.jmax : B.kmax;   // faces 1..nmax; face m has left cell m
  const long long gm1 = B.off + (i + 1) + (DIR == 1 ? sk : sj) * (o + 1);   // the column's cell at m = -1
  const float* P = d.pvf + (long long)v * n;
  float* FL = d.frec + (long long)v * n;
  float* FR = d.frec + (long long)(FREC_SIDE + v) * n;
  const bool mlp = c.nmuscl == 2;
  // slots 0..5: the planes m - 2 .. m + 3 of face m
  float cc[6], dt[6], dr[6], mn[6], mx[6];
  auto load = [&](int slot, int m) {
    const long long gc = gm1 + sn * (m + 1);
    cc[slot] = P[gc];
    if (mlp) {
      float a[3][3];   // [t1 + 1][t2 + 1]
#pragma unroll
      for (int p1 = 0; p1 < 3; ++p1)
#pragma unroll
        for (int p2 = 0; p2 < 3; ++p2) a[p1][p2] = P[gc + (p1 - 1) * s1 + (p2 - 1) * s2];
      dt[slot] = a[2][1] - a[0][1];
      dr[slot] = a[1][2] - a[1][0];
      float lo = a[0][0], hi = a[0][0];
#pragma unroll
      for (int p1 = 0; p1 < 3; ++p1)
#pragma unroll
        for (int p2 = 0; p2 < 3; ++p2) { lo = fminf(lo, a[p1][p2]); hi = fmaxf(hi, a[p1][p2]); }
      mn[slot] = lo; mx[slot] = hi;
    }
  };
#pragma unroll
  for (int q = 0; q < 5; ++q) load(q, q - 1);
  // the plane a face needs last (m + 3) is fetched one face ahead, so that its loads are in
  // flight while the face before it is formed
  float pre[9];   // [3 (t1 + 1) + (t2 + 1)]
  auto fetch = [&](int m) {
    const long long gc = gm1 + sn * (m + 1);
    if (mlp) {
#pragma unroll
      for (int p1 = 0; p1 < 3; ++p1)
#pragma unroll
        for (int p2 = 0; p2 < 3; ++p2) pre[3 * p1 + p2] = P[gc + (p1 - 1) * s1 + (p2 - 1) * s2];
    } else {
      pre[4] = P[gc];
    }
  };
  fetch(4);
  for (int m = 1; m <= nmax; ++m) {
    cc[5] = pre[4];
    if (mlp) {
      dt[5] = pre[7] - pre[1];
      dr[5] = pre[5] - pre[3];
      float lo = pre[0], hi = pre[0];
#pragma unroll
      for (int q = 1; q < 9; ++q) { lo = fminf(lo, pre[q]); hi = fmaxf(hi, pre[q]); }
      mn[5] = lo; mx[5] = hi;
    }
    if (m < nmax) fetch(m + 4);
    const float mnr[4] = {mn[1], mn[2], mn[3], mn[4]}, mxr[4] = {mx[1], mx[2], mx[3], mx[4]};
    float xl, xr;
    muscl_reduced(c, cc[0], cc[1], cc[2], cc[3], cc[4], cc[5], dt[2], dr[2], dt[3], dr[3], mnr, mxr, xl, xr);
    const long long gf = gm1 + sn * (m + 1);
    FL[gf] = xl;
    FR[gf] = xr;
#pragma unroll
    for (int q = 0; q < 5; ++q) { cc[q] = cc[q + 1]; dt[q] = dt[q + 1]; dr[q] = dr[q + 1]; mn[q] = mn[q + 1]; mx[q] = mx[q + 1]; }
  }
}

// Second order (nmuscl > 0): with MARCH the face states come from k_muscl_march (frec,
// before the clips), otherwise from the face's 38-cell stencil; first order: the face states
// are the cells' own.  (The per-variable loops run over the compile-time bound, guarded by
// npv, so that the arrays stay in registers.)
template <int DIR, bool MARCH = false>
// (the column-fed instantiations at 4 CTAs of 256 threads per SM, the stencil one at 3:
// 0.55 and 0.65 ms faster than at the compiler's choice of 2)
__global__ void __launch_bounds__(256, MARCH ? 4 : 3) k_recon_mx(DevPtr d, Par c, long long t0, long long t1) {
  const long long t = t0 + blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= t1) return;
  const FaceIdx f = face_of<DIR>(d, t);
  if (!f.ok) return;
  const long long n = d.ncell, g = f.g, gr = g + f.sn;
  const int npv = c.npv;
  const float* P = d.pvf;
  float gl[NPVM], gR[NPVM];
  float rdl, hdl, rdr, hdr;   // face rho - rhoref, h - href
  float cl = 0.0f, cr = 0.0f;
  if (c.nmuscl > 0) {
    float c9[NPVM], c10[NPVM];
#pragma unroll
    for (int v = 0; v < NPVM; ++v) gl[v] = gR[v] = c9[v] = c10[v] = 0.0f;
    if (MARCH) {
#pragma unroll
      for (int v = 0; v < NPVM; ++v) {
        if (v >= npv) continue;
        gl[v] = d.frec[v * n + g]; gR[v] = d.frec[(FREC_SIDE + v) * n + g];
        c9[v] = P[v * n + g]; c10[v] = P[v * n + gr];
      }
    } else {
      // one rolled loop over the variables (a 38-cell stencil and the limiter each: unrolled
      // nine times the kernel outgrows the instruction cache); its results reach the
      // register arrays by predicated selects
#pragma unroll 1
      for (int v = 0; v < npv; ++v) {
        float x[38];
#pragma unroll
        for (int l = 0; l < 38; ++l) x[l] = P[v * n + stencil_cell(l, g, f.sn, f.s1, f.s2)];
        float xl, xr;
        muscl_var<float>(c, x, xl, xr);
#pragma unroll
        for (int u = 0; u < NPVM; ++u)
          if (u == v) { gl[u] = xl; gR[u] = xr; c9[u] = x[8]; c10[u] = x[9]; }
      }
    }
    muscl_clip_mx(c, c9, c10, gl, gR);
    // a vapour-free face state by expansion about an interior cell -- its own side's, or at
    // a block face, where that cell is a ghost, the cell across the face; any other state by
    // the IF97 sums (FP64 mixture).  (Without the second base, the boundary faces of the i
    // direction, two in every warp's row of faces, would send their warps through the sums.)
    const float bl0 = f.lin ? c9[0] : c10[0], bl4 = f.lin ? c9[4] : c10[4], bl6 = f.lin ? c9[6] : c10[6];
    const float br0 = f.rin ? c10[0] : c9[0], br4 = f.rin ? c10[4] : c9[4], br6 = f.rin ? c10[6] : c9[6];
    if (!(gl[5] == 0.0f && liquid_expand(d, c, f.lin ? g : gr, gl, bl0, bl4, bl6, rdl, hdl))) {
      double rho, h;
      eos_rho_h<true>(c.fluid, c.pref + (double)gl[0], c.tref + (double)gl[4], gl[5], gl[6], rho, h);
      rdl = (float)(rho - c.rhoref);
      hdl = (float)(h - c.href);
    }
    if (!(gR[5] == 0.0f && liquid_expand(d, c, f.rin ? gr : g, gR, br0, br4, br6, rdr, hdr))) {
      double rho, h;
      eos_rho_h<true>(c.fluid, c.pref + (double)gR[0], c.tref + (double)gR[4], gR[5], gR[6], rho, h);
      rdr = (float)(rho - c.rhoref);
      hdr = (float)(h - c.href);
    }
    if (c.nscheme == 2 || c.nscheme == 3) {
      cl = eos_c2_f(c.fluid, (float)c.pref + gl[0], (float)c.tref + gl[4], gl[5], gl[6], &d.sc->snd2_fallbacks);
      cr = eos_c2_f(c.fluid, (float)c.pref + gR[0], (float)c.tref + gR[4], gR[5], gR[6], &d.sc->snd2_fallbacks);
    }
  } else {
#pragma unroll
    for (int v = 0; v < NPVM; ++v) {
      gl[v] = gR[v] = 0.0f;
      if (v < npv) { gl[v] = P[v * n + g]; gR[v] = P[v * n + gr]; }
    }
    rdl = (float)(d.dv[g] - c.rhoref); hdl = (float)(d.dv[n + g] - c.href); cl = (float)d.dv[5 * n + g];
    rdr = (float)(d.dv[gr] - c.rhoref); hdr = (float)(d.dv[n + gr] - c.href); cr = (float)d.dv[5 * n + gr];
  }
  float* F = d.frec;
#pragma unroll
  for (int v = 0; v < NPVM; ++v)
    if (v < npv) { F[v * n + g] = gl[v]; F[(FREC_SIDE + v) * n + g] = gR[v]; }
  F[NPVM * n + g] = rdl;
  F[(NPVM + 1) * n + g] = hdl;
  F[(NPVM + 2) * n + g] = cl;
  F[(FREC_SIDE + NPVM) * n + g] = rdr;
  F[(FREC_SIDE + NPVM + 1) * n + g] = hdr;
  F[(FREC_SIDE + NPVM + 2) * n + g] = cr;
}

template <int DIR>
// (3 CTAs of 256 threads per SM: measured 1 ms faster over the three directions than the
// compiler's own 2 on the 14.2 M-cell case, the few spills cost less than the warps gain)
__global__ void __launch_bounds__(256, 3) k_flux_mx(DevPtr d, Par c, long long t0, long long t1) {
  const long long t = t0 + blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= t1) return;
  const FaceIdx f = face_of<DIR>(d, t);
  if (!f.ok) return;
  const long long n = d.ncell, g = f.g;
  const long long sn = f.sn, s1 = f.s1, s2 = f.s2;
  const int npv = c.npv;
  const float* P = d.pvf;
  const int fplane = (DIR == 0) ? GM_CX : (DIR == 1 ? GM_EX : GM_TX);
  df64 nv[3];
  for (int q = 0; q < 3; ++q) nv[q] = df64(d.gmf[(fplane + q) * n + g], d.gmlo[(fplane + q) * n + g]);
  FaceMx L, R;
  {
    const float* F = d.frec;
#pragma unroll
    for (int v = 0; v < NPVM; ++v) {
      L.g[v] = R.g[v] = 0.0f;
      if (v < npv) { L.g[v] = F[v * n + g]; R.g[v] = F[(FREC_SIDE + v) * n + g]; }
    }
    const df64 rref = dfp(c.rhoref2), href = dfp(c.href2);
    L.rho = rref + dff(F[NPVM * n + g]);
    L.h = href + dff(F[(NPVM + 1) * n + g]);
    L.c2 = F[(NPVM + 2) * n + g];
    R.rho = rref + dff(F[(FREC_SIDE + NPVM) * n + g]);
    R.h = href + dff(F[(FREC_SIDE + NPVM + 1) * n + g]);
    R.c2 = F[(FREC_SIDE + NPVM + 2) * n + g];
    for (int q = 0; q < 3; ++q) { L.u[q] = dfp(c.U2[q]) + dff(L.g[1 + q]); R.u[q] = dfp(c.U2[q]) + dff(R.g[1 + q]); }
  }
  // Roe-average state (sqrt(rho) weights; p and T arithmetic means) and its FP32 sound speed
  float ravg_u[3], ravg_s[NPVM];
  float rc2 = 0.0f;
  {
    float srl = sqrtf(tof(L.rho)), srr = sqrtf(tof(R.rho));
    float rd = 1.0f / (srl + srr);
    for (int q = 0; q < 3; ++q) ravg_u[q] = c.U2[q][0] + (srl * L.g[1 + q] + srr * R.g[1 + q]) * rd;
    for (int q = 0; q < NPVM; ++q) ravg_s[q] = 0.0f;
#pragma unroll
    for (int q = 5; q < NPVM; ++q)
      if (q < npv) ravg_s[q] = (srl * L.g[q] + srr * R.g[q]) * rd;
    if (nv[0].hi != 0.0f || nv[1].hi != 0.0f || nv[2].hi != 0.0f) {
      // the FP32 sound speed of the Roe average: FP32 state
      const float pa = (float)c.pref + 0.5f * (L.g[0] + R.g[0]);
      const float ta = (float)c.tref + 0.5f * (L.g[4] + R.g[4]);
      rc2 = eos_c2_f(c.fluid, pa, ta, ravg_s[5], ravg_s[6], &d.sc->snd2_fallbacks);
    }
  }
  float sdst[18];
  if (c.nscheme == 2 || c.nscheme == 3) {
#pragma unroll
    for (int l = 0; l < 18; ++l) sdst[l] = P[stencil_cell(l, g, sn, s1, s2)];
  }
  float fx[NPVM];
  inviscid_flux_mx(c, nv, L, R, sdst, rc2, ravg_u, ravg_s, fx);
  float* fo = d.fi32 + (long long)DIR * npv * n;
#pragma unroll
  for (int v = 0; v < NPVM; ++v)
    if (v < npv) fo[v * n + g] = fx[v];
}

// The viscous flux of the DIR faces in FP32 (vsflux_laminar / vsflux_turbulent,
// src/vsflux_module.f90:182-425): a kernel of its own, so that its 18-cell gradient stencils
// run at 4 CTAs of 256 threads per SM (64 registers) rather than under the inviscid flux's
// df64 register budget.  Writes fv32.
template <int DIR>
__global__ void __launch_bounds__(256, 4) k_visc_mx(DevPtr d, Par c, long long t0, long long t1) {
  const long long t = t0 + blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= t1) return;
  const FaceIdx f = face_of<DIR>(d, t);
  if (!f.ok) return;
  const long long n = d.ncell, g = f.g, gr = g + f.sn;
  const long long sn = f.sn, s1 = f.s1, s2 = f.s2;
  const int npv = c.npv;
  const float* P = d.pvf;
  const int fplane = (DIR == 0) ? GM_CX : (DIR == 1 ? GM_EX : GM_TX);
  const bool turb = (c.iturb >= -1);
  const int ep = (DIR == 0) ? GM_EX : (DIR == 1 ? GM_TX : GM_CX);
  const int tp = (DIR == 0) ? GM_TX : (DIR == 1 ? GM_CX : GM_EX);
  // metrics from their FP32 copy
  const float* GF = d.gmf;
  float nx[3] = {GF[(fplane + 0) * n + g], GF[(fplane + 1) * n + g], GF[(fplane + 2) * n + g]};
  float ev[3], tvv[3];
  for (int q = 0; q < 3; ++q) {
    const float* E1 = GF + (ep + q) * n;
    ev[q] = 0.25f * (E1[g - s1] + E1[g - s1 + sn] + E1[g] + E1[g + sn]);
    const float* T1 = GF + (tp + q) * n;
    tvv[q] = 0.25f * (T1[g - s2] + T1[g - s2 + sn] + T1[g] + T1[g + sn]);
  }
  float vol = 2.0f / (GF[GM_GRD * n + g] + GF[GM_GRD * n + gr]);
  float tvl[3] = {0, 0, 0}, tvr[3] = {0, 0, 0};
#pragma unroll
  for (int q = 0; q < 3; ++q)
    if (q < c.ntv) { tvl[q] = (float)d.tv[q * n + g]; tvr[q] = (float)d.tv[q * n + gr]; }
  float vis = 0.5f * (tvl[0] + tvr[0]);
  float con = 0.5f * (tvl[1] + tvr[1]);
  float emut = 0.0f, tcon = 0.0f;
  if (turb) {
    emut = 0.5f * (tvl[2] + tvr[2]);
    tcon = 0.5f * (tvl[2] * (float)d.dv[11 * n + g] + tvr[2] * (float)d.dv[11 * n + gr]) / 0.9f;
  }
  const int vars[6] = {1, 2, 3, 4, 7, 8};
  float gx[6], gy[6], gz[6], cc[6];
  const int nvv = turb ? 6 : 4;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    gx[q] = gy[q] = gz[q] = cc[q] = 0.0f;
    if (q >= nvv) continue;
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
  // face-average velocities are full values: the shadow holds u - U
  float uc = cc[0] + (float)c.uref_vec[0], vc = cc[1] + (float)c.uref_vec[1], wc = cc[2] + (float)c.uref_vec[2];
  float fv[NPVM];
  fv[0] = 0.0f;
  fv[1] = txx * nx[0] + txy * nx[1] + txz * nx[2];
  fv[2] = txy * nx[0] + tyy * nx[1] + tyz * nx[2];
  fv[3] = txz * nx[0] + tyz * nx[1] + tzz * nx[2];
  fv[4] = nx[0] * (uc * txx + vc * txy + wc * txz + kc * gx[3]) + nx[1] * (uc * txy + vc * tyy + wc * tyz + kc * gy[3]) +
          nx[2] * (uc * txz + vc * tyz + wc * tzz + kc * gz[3]);
  fv[5] = 0.0f;
  fv[6] = 0.0f;
  if (turb && c.iturb == -1) {
    // k-epsilon: F1 = 0, sigma_k = 1, sigma_eps = 1.3
    fv[7] = (vis + emut) * (gx[4] * nx[0] + gy[4] * nx[1] + gz[4] * nx[2]);
    fv[8] = (vis + emut * (1.0f / 1.3f)) * (gx[5] * nx[0] + gy[5] * nx[1] + gz[5] * nx[2]);
  } else if (turb) {
    float pkw = gx[4] * gx[5] + gy[4] * gy[5] + gz[4] * gz[5];
    float rho = (float)(0.5 * (d.dv[g] + d.dv[gr]));
    float ydns = 0.5f * (GF[(GM_GRD + 4) * n + g] + GF[(GM_GRD + 4) * n + gr]);
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
#pragma unroll
  for (int v = 0; v < NPVM; ++v)
    if (v < npv) fvo[v * n + g] = fv[v];
}

// the face stage of blocks [b0, b1): their padded cells, faces and columns are contiguous
// ranges of the flat numberings
void launch_face_flux_mixed(const Engine& E, cudaStream_t s, int b0, int b1) {
  const int T = E.tpb_face;
  const int nb = (int)E.blk.size();
  auto nblk = [T](long long n) { return (unsigned)std::max<long long>((n + T - 1) / T, 1); };
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long g0 = E.blk[b0].off, g1 = (b1 < nb) ? E.blk[b1].off : E.ncell;
  long long f0[3], f1[3], c0[3], c1[3];
  for (int q = 0; q < 3; ++q) {
    f0[q] = E.blk[b0].face_off[q]; f1[q] = (b1 < nb) ? E.blk[b1].face_off[q] : E.nface[q];
    c0[q] = E.blk[b0].col_off[q]; c1[q] = (b1 < nb) ? E.blk[b1].col_off[q] : E.ncol[q];
  }
  const long long share = (long long)(b1 - b0) * std::max(nsm, 1) * 8 / std::max(nb, 1);
  k_shadow<<<(unsigned)std::max<long long>(share, 1), 256, 0, s>>>(E.d, E.par, g0, g1);
  // the i faces from their 38-cell stencils, the j and k faces by columns (k_muscl_march)
  // under MUSCL; then the clips and the face EOS
  const bool march = E.par.nmuscl > 0, visc = E.par.iturb != -3;
  auto cols = [&](int q) { return (unsigned)(((c1[q] - c0[q]) * E.par.npv + 127) / 128); };
  k_recon_mx<0><<<nblk(f1[0] - f0[0]), T, 0, s>>>(E.d, E.par, f0[0], f1[0]);
  k_flux_mx<0><<<nblk(f1[0] - f0[0]), T, 0, s>>>(E.d, E.par, f0[0], f1[0]);
  if (visc) k_visc_mx<0><<<nblk(f1[0] - f0[0]), T, 0, s>>>(E.d, E.par, f0[0], f1[0]);
  if (march) k_muscl_march<1><<<cols(1), 128, 0, s>>>(E.d, E.par, c0[1], c1[1]);
  if (march) k_recon_mx<1, true><<<nblk(f1[1] - f0[1]), T, 0, s>>>(E.d, E.par, f0[1], f1[1]);
  else k_recon_mx<1><<<nblk(f1[1] - f0[1]), T, 0, s>>>(E.d, E.par, f0[1], f1[1]);
  k_flux_mx<1><<<nblk(f1[1] - f0[1]), T, 0, s>>>(E.d, E.par, f0[1], f1[1]);
  if (visc) k_visc_mx<1><<<nblk(f1[1] - f0[1]), T, 0, s>>>(E.d, E.par, f0[1], f1[1]);
  if (march) k_muscl_march<2><<<cols(2), 128, 0, s>>>(E.d, E.par, c0[2], c1[2]);
  if (march) k_recon_mx<2, true><<<nblk(f1[2] - f0[2]), T, 0, s>>>(E.d, E.par, f0[2], f1[2]);
  else k_recon_mx<2><<<nblk(f1[2] - f0[2]), T, 0, s>>>(E.d, E.par, f0[2], f1[2]);
  k_flux_mx<2><<<nblk(f1[2] - f0[2]), T, 0, s>>>(E.d, E.par, f0[2], f1[2]);
  if (visc) k_visc_mx<2><<<nblk(f1[2] - f0[2]), T, 0, s>>>(E.d, E.par, f0[2], f1[2]);
}

}  // namespace cfd
