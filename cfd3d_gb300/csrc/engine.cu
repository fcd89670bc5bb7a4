// engine.cu -- kernels of one LU-SGS pseudo-iteration and the C ABI (include/cfd3d.h).
//
// One iteration (the reference's `lusgs`, src/update_module.f90:455-733, plus the
// residual of src/residual_module.f90:110-186) is a fixed sequence of launches on the
// handle's stream, captured once into a CUDA graph and replayed:
//
//   k_timestep            local time step + global minimum   (timestep_module.f90:127-212)
//   k_ghost x3            boundary program: faces+halos, edges, corners (bc_module.f90:1235-1396)
//   k_face_flux x3        inviscid + viscous face fluxes per direction (rhs_module.f90:282-538)
//   k_rhs                 flux differences + cavitation / SST / dual-time sources (:540-642)
//   k_sweep (fwd) x S     forward LU-SGS sweep, one launch per hyperplane i+j+k = s
//   k_sweep (bwd) x S     backward sweep                          (update_module.f90:486-670)
//   k_update              pv += dq, clipping, EOS with transport, residual partial sums (:672-700)
//   k_eddy                SST eddy viscosity                      (:701-732)
//   k_finish              residual norms, max location, solution time
//
// All blocks of a multi-block case advance together in every launch; the LU-SGS
// operator stays block-local (dq outside a block is zero), as in the reference.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstddef>
#include <cstring>
#include <cuda.h>
#include <fcntl.h>
#include <mutex>
#include <new>
#include <type_traits>
#include <unistd.h>
#include <vector>
#include "engine.cuh"
#include "mixed.cuh"

namespace cfd {

struct Cell {
  double pv[NPVM], dv[NDV], tv[3];
};

__device__ __forceinline__ void load_cell(const DevPtr& d, const Par& c, long long g, Cell& x) {
  const long long n = d.ncell;
  for (int v = 0; v < c.npv; ++v) x.pv[v] = d.pv[v * n + g];
  for (int v = 0; v < NDV; ++v) x.dv[v] = d.dv[v * n + g];
  x.tv[0] = x.tv[1] = x.tv[2] = 0.0;
  for (int v = 0; v < c.ntv; ++v) x.tv[v] = d.tv[v * n + g];
}
__device__ __forceinline__ void store_cell(const DevPtr& d, const Par& c, long long g, const Cell& x) {
  const long long n = d.ncell;
  for (int v = 0; v < c.npv; ++v) d.pv[v * n + g] = x.pv[v];
  for (int v = 0; v < NDV; ++v) d.dv[v * n + g] = x.dv[v];
  for (int v = 0; v < c.ntv; ++v) d.tv[v * n + g] = x.tv[v];
}

// ------------------------------------------------------------------ pointwise EOS
__global__ void k_eos_points(int fluid, int with_prop, long long n, const double* __restrict__ p,
                             const double* __restrict__ t, const double* __restrict__ y1,
                             const double* __restrict__ y2, double* __restrict__ dv, double* __restrict__ tv,
                             unsigned long long* fb) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  double d[NDV], tt[2] = {0.0, 0.0};
  deteos(fluid, with_prop, p[q], t[q], y1[q], y2[q], d, tt, fb);
  for (int v = 0; v < NDV; ++v) dv[NDV * q + v] = d[v];
  if (tv) { tv[2 * q] = tt[0]; tv[2 * q + 1] = tt[1]; }
}

// ------------------------------------------------------------------ initial state
// set_others (src/initial_module.f90:707-771) on the uploaded interior pv
// One block's uploaded primitives (AoS staging a, every padded cell) into pv, for the cells
// whose values differ from the device's: dv and tv(1:2) of such an interior cell follow by
// the update's EOS, as k_init(fresh = 0) forms them, and pv_changed records the change for
// the eddy viscosity.  A cell whose uploaded pv equals the device's bit for bit keeps the dv
// and tv that are already the EOS of that pv.
template <bool MX>
__global__ void k_take_pv(const double* __restrict__ a, BlockGeom B, DevPtr d, Par c) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= (long long)B.ni * B.nj * B.nk) return;
  const long long n = d.ncell, g = B.off + q;
  double pv[NPVM];
  bool same = true;
  for (int v = 0; v < c.npv; ++v) {
    pv[v] = a[q * c.npv + v];
    same = same && (__double_as_longlong(pv[v]) == __double_as_longlong(d.pv[v * n + g]));
  }
  if (same) return;
  for (int v = 0; v < c.npv; ++v) d.pv[v * n + g] = pv[v];
  d.sc->pv_changed = 1;
  const int i = (int)(q % B.ni) - 1, j = (int)((q / B.ni) % B.nj) - 1, k = (int)(q / ((long long)B.ni * B.nj)) - 1;
  if (i < 2 || j < 2 || k < 2 || i > B.imax || j > B.jmax || k > B.kmax) return;
  double dv[NDV], tv[3] = {0.0, 0.0, 0.0};
  if (MX) deteos_split(c.fluid, c.with_prop, pv[0] + c.pref, pv[4], pv[5], pv[6], dv, tv, &d.sc->snd2_fallbacks);
  else deteos<false>(c.fluid, c.with_prop, pv[0] + c.pref, pv[4], pv[5], pv[6], dv, tv, &d.sc->snd2_fallbacks);
  for (int v = 0; v < NDV; ++v) d.dv[v * n + g] = dv[v];
  for (int v = 0; v < c.ntv && v < 2; ++v) d.tv[v * n + g] = tv[v];
}

template <bool MX>
// fresh = 0 (cfd3d_upload_primitives): dv and tv(1:2) only; the eddy viscosity follows
// from k_eddy and the history and rates are the caller's
__global__ void k_init(DevPtr d, Par c, int b, int fresh) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const BlockGeom& B = d.blk[b];
  if (t >= (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1)) return;
  int i, j, k;
  long long g = interior_cell(B, t, i, j, k);
  const long long n = d.ncell;
  double pv[NPVM], dv[NDV], tv[3] = {0.0, 0.0, 0.0};
  for (int v = 0; v < c.npv; ++v) pv[v] = d.pv[v * n + g];
  if (MX) deteos_split(c.fluid, c.with_prop, pv[0] + c.pref, pv[4], pv[5], pv[6], dv, tv, &d.sc->snd2_fallbacks);
  else deteos<false>(c.fluid, c.with_prop, pv[0] + c.pref, pv[4], pv[5], pv[6], dv, tv, &d.sc->snd2_fallbacks);
  for (int v = 0; v < NDV; ++v) d.dv[v * n + g] = dv[v];
  if (!fresh) {
    for (int v = 0; v < c.ntv && v < 2; ++v) d.tv[v * n + g] = tv[v];
    return;
  }
  if (c.iturb >= -1) tv[2] = c.emutref;
  for (int v = 0; v < c.ntv; ++v) d.tv[v * n + g] = tv[v];
  if (c.nqq) {
    double q[NPVM];
    q[0] = dv[0]; q[1] = dv[0] * pv[1]; q[2] = dv[0] * pv[2]; q[3] = dv[0] * pv[3];
    q[4] = dv[0] * (dv[1] + 0.5 * (pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3])) - pv[0] - c.pref;
    for (int v = 5; v < c.npv; ++v) q[v] = dv[0] * pv[v];
    for (int v = 0; v < c.npv; ++v) { d.qq[v * n + g] = q[v]; d.qq[(c.npv + v) * n + g] = q[v]; }
  }
  if (c.ncav) { d.rcav[g] = 0.0; d.rcav[n + g] = 0.0; }
}

// BDF history shift (solve%unsteadyupdate, src/solve_module.f90:155-183)
__global__ void k_unsteady_shift(DevPtr d, Par c) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= d.nint) return;
  int b = find_block_interior(d.blk, d.nblk, t), i, j, k;
  long long g = interior_cell(d.blk[b], t - d.blk[b].int_off, i, j, k);
  const long long n = d.ncell;
  double pv[NPVM];
  for (int v = 0; v < c.npv; ++v) pv[v] = d.pv[v * n + g];
  double r = d.dv[g], h = d.dv[n + g];
  for (int v = 0; v < c.npv; ++v) d.qq[(c.npv + v) * n + g] = d.qq[v * n + g];
  d.qq[g] = r;
  d.qq[n + g] = r * pv[1];
  d.qq[2 * n + g] = r * pv[2];
  d.qq[3 * n + g] = r * pv[3];
  d.qq[4 * n + g] = r * (h + 0.5 * (pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3])) - pv[0] - c.pref;
  for (int v = 5; v < c.npv; ++v) d.qq[v * n + g] = r * pv[v];
}

// ------------------------------------------------------------------ local time step
// the viscous eigenvalue term of eigenvis_of in FP32 (the mixed form's time step)
__device__ __forceinline__ float eigenvis_f(const Par& c, const float* dv, const float* tv) {
  if (c.iturb == -3) return 0.0f;
  const float den = dv[7] + dv[11] * dv[6] * dv[0] - dv[10] * dv[7] * dv[0];
  if (c.iturb == -2) return fmaxf(dv[6] * tv[1] / den, (4.0f / 3.0f) * tv[0] / dv[0]);
  return fmaxf(dv[6] * (tv[1] + dv[11] * tv[2] * (1.0f / 0.9f)) / den, (4.0f / 3.0f) * (tv[0] + tv[2]) / dv[0]);
}

// MX: the local time step only scales the implicit operator -- FP32 on the FP32 metrics
template <bool MX>
__global__ void k_timestep(DevPtr d, Par c) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double dtv = 1.0e10;
  if (t < d.nint) {
    int b = find_block_interior(d.blk, d.nblk, t), i, j, k;
    const BlockGeom& B = d.blk[b];
    long long g = interior_cell(B, t - B.int_off, i, j, k);
    if (c.local == -1) {
      dtv = c.cfl;
    } else if (MX) {
      const long long n = d.ncell, sj = B.ni, sk = (long long)B.ni * B.nj;
      const float u = (float)d.pv[n + g], v = (float)d.pv[2 * n + g], w = (float)d.pv[3 * n + g];
      float dvf[12], tvf[3] = {0.0f, 0.0f, 0.0f};
      for (int q = 0; q < 12; ++q) dvf[q] = (float)d.dv[q * n + g];
      for (int q = 0; q < c.ntv; ++q) tvf[q] = (float)d.tv[q * n + g];
      const float* G = d.gmf;
      const float vol = G[GM_GRD * n + g];
      float cs[3][3];
      for (int q = 0; q < 3; ++q) {
        cs[0][q] = 0.5f * (G[(GM_CX + q) * n + g - 1] + G[(GM_CX + q) * n + g]);
        cs[1][q] = 0.5f * (G[(GM_EX + q) * n + g - sj] + G[(GM_EX + q) * n + g]);
        cs[2][q] = 0.5f * (G[(GM_TX + q) * n + g - sk] + G[(GM_TX + q) * n + g]);
      }
      const float sndp2 = sndp2_of<float>(c, dvf[5], u * u + v * v + w * w);
      const float qf = sndp2 / dvf[5];
      float eig = 0.0f, ss = 0.0f;
      for (int q = 0; q < 3; ++q) {
        const float uc = fabsf(cs[q][0] * u + cs[q][1] * v + cs[q][2] * w);
        const float s2 = cs[q][0] * cs[q][0] + cs[q][1] * cs[q][1] + cs[q][2] * cs[q][2];
        const float up = uc * (1.0f + qf);
        const float dd = sqrtf(uc * uc * (1.0f - qf) * (1.0f - qf) + 4.0f * sndp2 * s2);
        eig += 0.5f * (up + dd);
        ss += s2;
      }
      const float ev = eigenvis_f(c, dvf, tvf) * ss / vol;
      dtv = (double)((float)c.cfl * vol / (eig + 4.0f * ev));
    } else {
      const long long n = d.ncell, sj = B.ni, sk = (long long)B.ni * B.nj;
      double u = d.pv[n + g], v = d.pv[2 * n + g], w = d.pv[3 * n + g];
      double dv[NDV];
      for (int q = 0; q < NDV; ++q) dv[q] = d.dv[q * n + g];
      double tv[3] = {0.0, 0.0, 0.0};
      for (int q = 0; q < c.ntv; ++q) tv[q] = d.tv[q * n + g];
      double vol = d.gm[GM_GRD * n + g];
      double cs[3][3];
      for (int q = 0; q < 3; ++q) {
        cs[0][q] = 0.5 * (d.gm[(GM_CX + q) * n + g - 1] + d.gm[(GM_CX + q) * n + g]);
        cs[1][q] = 0.5 * (d.gm[(GM_EX + q) * n + g - sj] + d.gm[(GM_EX + q) * n + g]);
        cs[2][q] = 0.5 * (d.gm[(GM_TX + q) * n + g - sk] + d.gm[(GM_TX + q) * n + g]);
      }
      double sndp2 = sndp2_of<double>(c, dv[5], u * u + v * v + w * w);
      double qf = sndp2 / dv[5];
      double eig = 0.0, ss = 0.0;
      for (int q = 0; q < 3; ++q) {
        double uc = fabs(cs[q][0] * u + cs[q][1] * v + cs[q][2] * w);
        double s = cs[q][0] * cs[q][0] + cs[q][1] * cs[q][1] + cs[q][2] * cs[q][2];
        double up = uc * (1.0 + qf);
        double dd = sqrt(uc * uc * (1.0 - qf) * (1.0 - qf) + 4.0 * sndp2 * s);
        eig += 0.5 * (up + dd);
        ss += s;
      }
      double ev = eigenvis_of(c, dv, tv) * ss / vol;
      dtv = c.cfl * vol / (eig + 4.0 * ev);
    }
    d.dt[g] = dtv;
  }
  // block minimum -> one atomic per CTA (positive doubles order like their bit patterns)
  for (int o = 16; o > 0; o >>= 1) dtv = fmin(dtv, __shfl_xor_sync(0xffffffffu, dtv, o));
  __shared__ double wmin[32];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = dtv;
  __syncthreads();
  if (threadIdx.x < 32) {
    double m = (threadIdx.x < (blockDim.x >> 5)) ? wmin[threadIdx.x] : 1.0e10;
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) atomicMin(&d.sc->dtmin_bits, (unsigned long long)__double_as_longlong(m));
  }
}

// ------------------------------------------------------------------ boundary program
// ---- total-pressure inlet (bctotalpressurein, src/bc_module.f90:3299-3514) ------------
// newt (:4305-4387) for x = (p, T): f1 = p_t - p (T_t / T)^(g / (g - 1)),
// f2 = h_t - (h(p, T) + |u|^2 / 2) (funcv :4408-4422), with fdjac's forward differences
// (:4424-4447), the backtracking line search lnsrch (:4449-4526) and ludcmp / lubksb
// (:4528-4622) on the 2 x 2 system -- as written, including that newt evaluates its fvec
// once (lnsrch evaluates into a local copy), so its tests and Jacobian reuse that first one.
struct TpProblem { double pt, tt, ht, y1, y2, uu, gam; int fluid; };
__device__ void tp_funcv(const TpProblem& P, const double* x, double* f) {
  double dv[NDV];
  deteos_simple<false>(P.fluid, x[0], x[1], P.y1, P.y2, dv, nullptr);
  f[0] = P.pt - x[0] * pow(P.tt / x[1], P.gam / (P.gam - 1.0));
  f[1] = P.ht - (dv[1] + 0.5 * P.uu);
}
__device__ double tp_fmin(const TpProblem& P, const double* x, double* f) {
  tp_funcv(P, x, f);
  return 0.5 * (f[0] * f[0] + f[1] * f[1]);
}
__device__ void tp_ludcmp(double (*a)[2], int* indx) {
  double vv[2];
  for (int i = 0; i < 2; ++i) vv[i] = 1.0 / fmax(fabs(a[i][0]), fabs(a[i][1]));
  for (int j = 0; j < 2; ++j) {
    for (int i = 0; i < j; ++i) {
      double sum = a[i][j];
      for (int k = 0; k < i; ++k) sum -= a[i][k] * a[k][j];
      a[i][j] = sum;
    }
    double aamax = 0.0;
    int imax = j;
    for (int i = j; i < 2; ++i) {
      double sum = a[i][j];
      for (int k = 0; k < j; ++k) sum -= a[i][k] * a[k][j];
      a[i][j] = sum;
      const double dum = vv[i] * fabs(sum);
      if (dum >= aamax) { imax = i; aamax = dum; }
    }
    if (j != imax) {
      for (int k = 0; k < 2; ++k) { const double dum = a[imax][k]; a[imax][k] = a[j][k]; a[j][k] = dum; }
      vv[imax] = vv[j];
    }
    indx[j] = imax;
    if (a[j][j] == 0.0) a[j][j] = 1.0e-20;
    if (j != 1) {
      const double dum = 1.0 / a[j][j];
      for (int i = j + 1; i < 2; ++i) a[i][j] *= dum;
    }
  }
}
__device__ void tp_lubksb(const double (*a)[2], const int* indx, double* b) {
  int ii = -1;
  for (int i = 0; i < 2; ++i) {
    const int ll = indx[i];
    double sum = b[ll];
    b[ll] = b[i];
    if (ii >= 0) for (int j = ii; j < i; ++j) sum -= a[i][j] * b[j];
    else if (sum != 0.0) ii = i;
    b[i] = sum;
  }
  for (int i = 1; i >= 0; --i) {
    double sum = b[i];
    for (int j = i + 1; j < 2; ++j) sum -= a[i][j] * b[j];
    b[i] = sum / a[i][i];
  }
}
__device__ void tp_newt(const TpProblem& P, double* x) {
  const double tolf = 1.0e-4, tolmin = 1.0e-6, tolx = 1.0e-7, stpmx = 100.0, alf = 1.0e-4;
  double fvec[2], fjac[2][2], g[2], p[2], xold[2], ftmp[2];
  double f = tp_fmin(P, x, fvec);
  if (fmax(fabs(fvec[0]), fabs(fvec[1])) < 0.01 * tolf) return;
  const double stpmax = stpmx * fmax(sqrt(x[0] * x[0] + x[1] * x[1]), 2.0);
  for (int its = 0; its < 200; ++its) {
    for (int j = 0; j < 2; ++j) {   // fdjac
      double tmp[2] = {x[0], x[1]};
      double h = 1.0e-4 * fabs(tmp[j]);
      if (h == 0.0) h = 1.0e-4;
      tmp[j] = tmp[j] + h;
      h = tmp[j] - x[j];
      tp_funcv(P, tmp, ftmp);
      for (int i = 0; i < 2; ++i) fjac[i][j] = (ftmp[i] - fvec[i]) / h;
    }
    for (int i = 0; i < 2; ++i) g[i] = fjac[0][i] * fvec[0] + fjac[1][i] * fvec[1];
    xold[0] = x[0]; xold[1] = x[1];
    const double fold = f;
    p[0] = -fvec[0]; p[1] = -fvec[1];
    int indx[2];
    tp_ludcmp(fjac, indx);
    tp_lubksb(fjac, indx, p);
    // lnsrch
    bool check = false;
    {
      const double sum = sqrt(p[0] * p[0] + p[1] * p[1]);
      if (sum > stpmax) { p[0] *= stpmax / sum; p[1] *= stpmax / sum; }
      const double slope = g[0] * p[0] + g[1] * p[1];
      const double test = fmax(fabs(p[0]) / fmax(fabs(xold[0]), 1.0), fabs(p[1]) / fmax(fabs(xold[1]), 1.0));
      const double alamin = tolx / test;
      double alam = 1.0, alam2 = 0.0, f2 = 0.0, fold2 = 0.0, tmplam = 0.0;
      for (int ls = 0; ls < 1000; ++ls) {   // (bounded: alam falls by 10x per pass at least)
        x[0] = xold[0] + alam * p[0];
        x[1] = xold[1] + alam * p[1];
        double fl[2];
        f = tp_fmin(P, x, fl);
        if (alam < alamin) { x[0] = xold[0]; x[1] = xold[1]; check = true; break; }
        if (f <= fold + alf * alam * slope) break;
        if (alam == 1.0) {
          tmplam = -slope / (2.0 * (f - fold - slope));
        } else {
          const double rhs1 = f - fold - alam * slope, rhs2 = f2 - fold2 - alam2 * slope;
          const double a = (rhs1 / (alam * alam) - rhs2 / (alam2 * alam2)) / (alam - alam2);
          const double b = (-alam2 * rhs1 / (alam * alam) + alam * rhs2 / (alam2 * alam2)) / (alam - alam2);
          if (a == 0.0) tmplam = -slope / (2.0 * b);
          else {
            const double disc = b * b - 3.0 * a * slope;
            if (disc < 0.0) tmplam = 0.5 * alam;
            else if (b <= 0.0) tmplam = (-b + sqrt(disc)) / (3.0 * a);
            else tmplam = -slope / (b + sqrt(disc));
          }
          if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
        }
        alam2 = alam;
        f2 = f;
        fold2 = fold;
        alam = fmax(tmplam, 0.1 * alam);
      }
    }
    if (fmax(fabs(fvec[0]), fabs(fvec[1])) < tolf) return;
    if (check) return;   // (the reference's test here only sets its check flag)
    const double tx = fmax(fabs(x[0] - xold[0]) / fmax(fabs(x[0]), 1.0), fabs(x[1] - xold[1]) / fmax(fabs(x[1]), 1.0));
    if (tx < tolx) return;
  }
}

// the grid velocity omega x r of a boundary face: r the mean of the centroids of the
// boundary cell b and the ghost cell across the face (gridvel, e.g. src/bc_module.f90:3539-3559)
__device__ __forceinline__ void face_gridvel(const DevPtr& d, const Par& c, long long b, long long gc, double* gv) {
  const long long n = d.ncell;
  double r[3];
  for (int e = 0; e < 3; ++e) r[e] = 0.5 * (d.gm[(GM_GRD + 1 + e) * n + b] + d.gm[(GM_GRD + 1 + e) * n + gc]);
  grid_vel(c, r, gv);
}

// one CTA per pool of total-pressure patches (the n-th inlet of every block): the
// area-weighted boundary averages over the pool (the reference's reduction over its
// communicator), then the Newton solve by thread 0
__global__ void __launch_bounds__(128) k_totalp(DevPtr d, Par c) {
  const int pt = blockIdx.x;
  const long long n = d.ncell;
  __shared__ double sh[6][128];
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int e = d.tp_off[pt] + threadIdx.x; e < d.tp_off[pt + 1]; e += blockDim.x) {
    const int* E = d.tp_ent + 4 * e;
    double nx[3];
    face_vec(d, E[2], E[1], nx);
    const double dl = sqrt(nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2]);
    const long long b = E[0];
    double gv[3] = {0.0, 0.0, 0.0};
    if (c.rot) face_gridvel(d, c, b, E[3], gv);
    acc[0] += d.pv[b] * dl;
    for (int q = 0; q < 3; ++q) acc[1 + q] += (d.pv[(1 + q) * n + b] + gv[q]) * dl;
    acc[4] += d.pv[4 * n + b] * dl;
    acc[5] += dl;
  }
  for (int q = 0; q < 6; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < 6; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double area = sh[5][0];
  const double pa = sh[0][0] / area, ua = sh[1][0] / area, va = sh[2][0] / area, wa = sh[3][0] / area;
  const double ta = sh[4][0] / area;
  TpProblem P;
  P.pt = c.tp_pt; P.tt = c.tp_tt; P.ht = c.tp_ht; P.y1 = c.y1ref; P.y2 = c.y2ref;
  P.uu = ua * ua + va * va + wa * wa;
  P.gam = (1.0 - c.y2ref) * 1.33 + c.y2ref * 1.4;   // eos%getgamma_f (water), getgamma_g (ideal gas)
  P.fluid = c.fluid;
  double x[2] = {pa + c.pref, ta};
  tp_newt(P, x);
  d.tp_x[3 * pt] = x[0];
  d.tp_x[3 * pt + 1] = x[1];
  d.tp_x[3 * pt + 2] = P.uu;
}

// The EOS of a ghost state: FP64, or in the mixed form the update's split evaluation (rho
// and h from df64 IF97 sums, derivatives and transport properties in FP32).  What reads
// ghost cells there -- the FP32 viscous fluxes and SST terms, first-order face states' rho
// and h, the volume fraction -- needs no more, and the far-field faces' full FP64 sums were
// most of the boundary program's time.
__device__ __forceinline__ void ghost_eos(const DevPtr& d, const Par& c, double p, double t, double y1, double y2,
                                          double* dv, double* tv) {
  if (c.mixed) deteos_split(c.fluid, c.with_prop, p, t, y1, y2, dv, tv, &d.sc->snd2_fallbacks);
  else deteos(c.fluid, c.with_prop, p, t, y1, y2, dv, tv, &d.sc->snd2_fallbacks);
}

__global__ void k_ghost(DevPtr d, Par c, const GhostOp* __restrict__ ops, int nops) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nops) return;
  const GhostOp op = ops[q];
  const long long n = d.ncell;
  Cell x;
  switch (op.kind) {
    case G_COPY:
    case G_EXTRAP:
      load_cell(d, c, op.src, x);
      store_cell(d, c, op.dst, x);
      return;
    case G_WALL_VISCOUS:
      load_cell(d, c, op.src, x);
      x.pv[1] = -x.pv[1]; x.pv[2] = -x.pv[2]; x.pv[3] = -x.pv[3];
      store_cell(d, c, op.dst, x);
      return;
    case G_WALL_KW: {
      load_cell(d, c, op.src, x);
      double vis_b = d.tv[op.bnd], rho_b = d.dv[op.bnd], y5 = d.gm[(GM_GRD + 4) * n + op.bnd];
      double om = 1600.0 * vis_b / rho_b / (y5 * y5) - x.pv[8];
      x.pv[1] = -x.pv[1]; x.pv[2] = -x.pv[2]; x.pv[3] = -x.pv[3]; x.pv[7] = -x.pv[7]; x.pv[8] = om;
      x.tv[2] = -x.tv[2];
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_SYMMETRY: {
      load_cell(d, c, op.src, x);
      double nx[3];
      face_vec(d, op.fplane, op.fidx, nx);
      for (int v = 0; v < 3; ++v) nx[v] *= (double)op.fsign;
      double us = d.pv[n + op.bnd], vs = d.pv[2 * n + op.bnd], ws = d.pv[3 * n + op.bnd];
      double un = (us * nx[0] + vs * nx[1] + ws * nx[2]) / (nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2]);
      x.pv[1] = 2.0 * (us - nx[0] * un) - x.pv[1];
      x.pv[2] = 2.0 * (vs - nx[1] * un) - x.pv[2];
      x.pv[3] = 2.0 * (ws - nx[2] * un) - x.pv[3];
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_FARFIELD:
    case G_INFLOW_SUB:
    case G_OUTFLOW_SUB:
    case G_INFLOW_SUP: {
      load_cell(d, c, op.src, x);
      double nx[3];
      face_vec(d, op.fplane, op.fidx, nx);
      for (int v = 0; v < 3; ++v) nx[v] *= (double)op.fsign;
      double pb[NPVM];
      for (int v = 0; v < c.npv; ++v) pb[v] = d.pv[v * n + op.bnd];
      double rb = d.dv[op.bnd], c2b = d.dv[5 * n + op.bnd];
      double dl = 1.0 / sqrt(nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2]);
      // free-stream state bcinfo%pv with bcinfo%pressure = pref
      double bp[NPVM];
      bp[0] = c.pref; bp[1] = c.uref_vec[0]; bp[2] = c.uref_vec[1]; bp[3] = c.uref_vec[2];
      bp[4] = c.tref; bp[5] = c.y1ref; bp[6] = c.y2ref; bp[7] = c.kref; bp[8] = c.oref;
      double* pv = x.pv;
      farfield_pv<double>(c, nx, dl, pb, rb, c2b, bp, c.uref * c.uref, pv, ghost_ff_mode(op.kind));
      ghost_eos(d, c, pv[0] + bp[0], pv[4], pv[5], pv[6], x.dv, x.tv);
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_WALL_KE:
      // bcwallviscouske (src/bc_module.f90:2324-2366): u, v, w, k, eps and mu_t reflected
      load_cell(d, c, op.src, x);
      x.pv[1] = -x.pv[1]; x.pv[2] = -x.pv[2]; x.pv[3] = -x.pv[3]; x.pv[7] = -x.pv[7]; x.pv[8] = -x.pv[8];
      x.tv[2] = -x.tv[2];
      store_cell(d, c, op.dst, x);
      return;
    case G_TOTALP: {
      // bctotalpressurein's ghost (:3398-3505): p and T from the patch's Newton solve, the
      // normal inflow speed |u_avg|, y1, k, omega from the free stream -- and y2 reflected
      // twice, so the mirror's
      load_cell(d, c, op.src, x);
      const double* X = d.tp_x + 3 * op.pad;
      double nx[3];
      face_vec(d, op.fplane, op.fidx, nx);
      for (int v = 0; v < 3; ++v) nx[v] *= (double)op.fsign;
      const double dl = 1.0 / sqrt(nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2]);
      const double su = sqrt(X[2]);
      const double bp[NPVM] = {c.pref, 0.0, 0.0, 0.0, c.tp_tt, c.y1ref, c.y2ref, c.kref, c.oref};
      double gv[3] = {0.0, 0.0, 0.0};
      if (c.rot) face_gridvel(d, c, op.bnd, op.gcell, gv);
      double* pv = x.pv;
      pv[0] = 2.0 * (X[0] - c.pref) - pv[0];
      for (int q3 = 0; q3 < 3; ++q3) pv[1 + q3] = 2.0 * (-su * nx[q3] * dl - gv[q3]) - pv[1 + q3];
      pv[4] = 2.0 * X[1] - pv[4];
      for (int v = 5; v < c.npv; ++v) pv[v] = 2.0 * bp[v] - pv[v];
      pv[6] = 2.0 * bp[6] - pv[6];
      pv[5] = fmin(fmax(pv[5], 0.0), 1.0);
      pv[6] = fmin(fmax(pv[6], 0.0), 1.0);
      ghost_eos(d, c, pv[0] + c.pref, pv[4], pv[5], pv[6], x.dv, x.tv);
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_CRWALL:
    case G_CRWALL_KW: {
      // bccounterrotatingwallviscous (src/bc_module.f90:3516-3580) and its k-omega variant
      // (:3654-3731): u = -u_mirror - 2 gridvel; k-omega: k and mu_t reflected, omega the
      // mirror's, the reference's wall value being computed and then discarded
      load_cell(d, c, op.src, x);
      double gv[3] = {0.0, 0.0, 0.0};
      if (c.rot) face_gridvel(d, c, op.bnd, op.gcell, gv);
      for (int q3 = 0; q3 < 3; ++q3) x.pv[1 + q3] = -x.pv[1 + q3] - 2.0 * gv[q3];
      if (op.kind == G_CRWALL_KW) { x.pv[7] = -x.pv[7]; x.tv[2] = -x.tv[2]; }
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_CRWALL_INV: {
      // bccounterrotatingwallinviscid (:3733-3810): the symmetry reflection of the boundary
      // cell's velocity less the face's grid velocity
      load_cell(d, c, op.src, x);
      double nx[3];
      face_vec(d, op.fplane, op.fidx, nx);
      for (int v = 0; v < 3; ++v) nx[v] *= (double)op.fsign;
      double gv[3] = {0.0, 0.0, 0.0};
      if (c.rot) face_gridvel(d, c, op.bnd, op.gcell, gv);
      const double us = d.pv[n + op.bnd], vs = d.pv[2 * n + op.bnd], ws = d.pv[3 * n + op.bnd];
      const double un = (us * nx[0] + vs * nx[1] + ws * nx[2]) / (nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2]);
      x.pv[1] = 2.0 * (us - nx[0] * un - gv[0]) - x.pv[1];
      x.pv[2] = 2.0 * (vs - nx[1] * un - gv[1]) - x.pv[2];
      x.pv[3] = 2.0 * (ws - nx[2] * un - gv[2]) - x.pv[3];
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_HFWALL_KW: {
      // bcheatfluxwallviscouskw (src/bc_module.f90:4184-4273): u, v, w, k reflected, the
      // wall temperature from the heat flux through the boundary cell, the SST omega wall
      // value.  The routine's EOS call takes the mirror's state, so the ghost keeps the
      // mirror's dv and tv(1:2); tv(3) reflects.
      load_cell(d, c, op.src, x);
      const long long b = op.bnd;
      const double hf = heatflux_at(d.hft + op.pad, bc_time(d, c));
      const double yb = d.gm[(GM_GRD + 4) * n + b], mub = d.tv[b], kb = d.tv[n + b];
      const double ub = d.pv[n + b], vb = d.pv[2 * n + b], wb = d.pv[3 * n + b];
      x.pv[1] = -x.pv[1]; x.pv[2] = -x.pv[2]; x.pv[3] = -x.pv[3]; x.pv[7] = -x.pv[7];
      x.pv[4] = 2.0 * ((hf * yb + 0.5 * mub * (ub * ub + vb * vb + wb * wb)) / kb + d.pv[4 * n + b]) - x.pv[4];
      x.pv[8] = 1600.0 * mub / d.dv[b] / (yb * yb) - x.pv[8];
      x.tv[2] = -x.tv[2];
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_MASSFLOW_IN: {
      // bcmassflowratein (:3812-4012) with the rate 0 its construct sets: the inflow speed
      // m / (rho A) is 0, so u = 2 (0 - gridvel) - u_mirror; T, y1, y2, k, omega from the
      // free stream; the pressure stays the mirror's; EOS of the ghost state
      load_cell(d, c, op.src, x);
      const double bp[NPVM] = {c.pref, c.uref_vec[0], c.uref_vec[1], c.uref_vec[2], c.tref, c.y1ref, c.y2ref,
                               c.kref, c.oref};
      double gv[3] = {0.0, 0.0, 0.0};
      if (c.rot) face_gridvel(d, c, op.bnd, op.gcell, gv);
      double* pv = x.pv;
      for (int q3 = 1; q3 < 4; ++q3) pv[q3] = 2.0 * (0.0 - gv[q3 - 1]) - pv[q3];
      for (int v = 4; v < c.npv; ++v) pv[v] = 2.0 * bp[v] - pv[v];
      pv[5] = fmin(fmax(pv[5], 0.0), 1.0);
      pv[6] = fmin(fmax(pv[6], 0.0), 1.0);
      ghost_eos(d, c, pv[0] + bp[0], pv[4], pv[5], pv[6], x.dv, x.tv);
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_WALLWALL:
    case G_WALLWALL_KW4:
    case G_WALLWALL_KW8: {
      load_cell(d, c, op.src, x);
      double ppv[NPVM];
      for (int v = 0; v < c.npv; ++v) ppv[v] = -x.pv[v];
      for (int m = 0; m < 6; ++m) {
        if (op.nb[m] < 0) break;
        for (int v = 0; v < c.npv; ++v) ppv[v] -= d.pv[v * n + op.nb[m]];
      }
      x.pv[1] = ppv[1]; x.pv[2] = ppv[2]; x.pv[3] = ppv[3];
      if (op.kind == G_WALLWALL) {
        if (c.npv > 7) { x.pv[7] = ppv[7]; x.pv[8] = ppv[8]; }
      } else {
        double y5 = d.gm[(GM_GRD + 4) * n + op.src];
        double var = 800.0 * x.tv[0] / x.dv[0] / (y5 * y5);
        x.pv[7] = ppv[7];
        x.pv[8] = ((op.kind == G_WALLWALL_KW8) ? 8.0 : 4.0) * var + ppv[8];
      }
      store_cell(d, c, op.dst, x);
      return;
    }
    case G_NOWALL3:
    case G_NOWALL7: {
      double pv[NPVM], tv[3] = {0.0, 0.0, 0.0};
      for (int v = 0; v < c.npv; ++v) pv[v] = d.pv[v * n + op.src];
      for (int v = 0; v < c.ntv; ++v) tv[v] = d.tv[v * n + op.src];
      for (int m = 0; m < 6; ++m) {
        if (op.nb[m] < 0) break;
        for (int v = 0; v < c.npv; ++v) pv[v] += d.pv[v * n + op.nb[m]];
        for (int v = 0; v < c.ntv; ++v) tv[v] += d.tv[v * n + op.nb[m]];
      }
      double f = (op.kind == G_NOWALL7) ? 1.0 / 7.0 : 1.0 / 3.0;
      for (int v = 0; v < c.npv; ++v) x.pv[v] = f * pv[v];
      for (int v = 0; v < 3; ++v) x.tv[v] = f * tv[v];
      ghost_eos(d, c, x.pv[0] + c.pref, x.pv[4], x.pv[5], x.pv[6], x.dv, x.tv);
      store_cell(d, c, op.dst, x);
      return;
    }
    default:
      return;
  }
}

// the mixed form's free-stream closure of every interior cell, (Phi + pref I).sum(n dl)
// over its six faces, for k_rhs (the metrics do not change, so this runs once)
__global__ void k_closure(DevPtr d, Par c) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= d.nint) return;
  int b = find_block_interior(d.blk, d.nblk, t), i, j, k;
  const BlockGeom& B = d.blk[b];
  const long long g = interior_cell(B, t - B.int_off, i, j, k);
  const long long n = d.ncell, st[3] = {1, B.ni, (long long)B.ni * B.nj};
  const int planes[3] = {GM_CX, GM_EX, GM_TX};
  double sn[3];
  for (int e = 0; e < 3; ++e) {
    double s = 0.0;
    for (int q = 0; q < 3; ++q) {
      const double* G = d.gm + (planes[q] + e) * n;
      s += G[g] - G[g - st[q]];
    }
    sn[e] = s;
  }
  for (int v = 0; v < c.npv; ++v) {
    double r = c.phi[v][0] * sn[0] + c.phi[v][1] * sn[1] + c.phi[v][2] * sn[2];
    if (v >= 1 && v <= 3) r += c.pref * sn[v - 1];
    d.clo[v * n + g] = r;
  }
}

// ------------------------------------------------------------------ surface tension
// Products that are summed are rounded first (no multiply-add contraction), as the
// reference's evaluation order gives them, so that the interface threshold |vfg| = 0.04 and
// the curvature see the same values as the CPU restatement.
__device__ __forceinline__ double mr(double a, double b) { return __dmul_rn(a, b); }

// (block, i, j, k) of padded cell g
__device__ __forceinline__ int padded_ijk(const DevPtr& d, long long g, int& i, int& j, int& k) {
  const int b = find_block_cell(d.blk, d.nblk, g);
  const BlockGeom& B = d.blk[b];
  const long long r = g - B.off;
  i = (int)(r % B.ni) - 1;
  const long long r2 = r / B.ni;
  j = (int)(r2 % B.nj) - 1;
  k = (int)(r2 / B.nj) - 1;
  return b;
}

// calvfg (src/variable_module.f90:304-318): vf = rho (y1 / rho_v + y2 / rho_g), the volume
// fraction of vapour and gas, over the cells 0..imax+2 of each block
__global__ void k_vf(DevPtr d) {
  const long long n = d.ncell;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    const BlockGeom& B = d.blk[padded_ijk(d, g, i, j, k)];
    if (i < 0 || j < 0 || k < 0 || i > B.imax + 2 || j > B.jmax + 2 || k > B.kmax + 2) continue;
    d.vf[g] = d.dv[g] * (d.pv[5 * n + g] / d.dv[3 * n + g] + d.pv[6 * n + g] / d.dv[4 * n + g]);
  }
}

// calvfg / calgrad_gg (:320-377): the Green-Gauss gradient of vf over the cells 1..imax+1,
// the interior and the first ghost layer.  For the ghost layer the reference reads face
// vectors past the ends of its arrays (cx(0), cx(imax+1), ex(., 0, .), ex(., jmax+1, .),
// tx(., ., 0), tx(., ., kmax+1)), which hold no defined values; here such a face takes the
// vector of the nearest face of its row.
__global__ void k_vfg(DevPtr d) {
  const long long n = d.ncell;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    const BlockGeom& B = d.blk[padded_ijk(d, g, i, j, k)];
    if (i < 1 || j < 1 || k < 1 || i > B.imax + 1 || j > B.jmax + 1 || k > B.kmax + 1) continue;
    const long long sj = B.ni, sk = (long long)B.ni * B.nj;
    const double x[7] = {d.vf[g - 1], d.vf[g + 1], d.vf[g - sj], d.vf[g + sj], d.vf[g - sk], d.vf[g + sk], d.vf[g]};
    const long long f[6] = {g + (max(i - 1, 1) - i), g + (min(i, B.imax) - i), g + (max(j - 1, 1) - j) * sj,
                            g + (min(j, B.jmax) - j) * sj, g + (max(k - 1, 1) - k) * sk, g + (min(k, B.kmax) - k) * sk};
    const int pl[6] = {GM_CX, GM_CX, GM_EX, GM_EX, GM_TX, GM_TX};
    double gr[3] = {0.0, 0.0, 0.0};
    for (int l = 0; l < 6; ++l) {
      const double xm = 0.5 * (x[6] + x[l]);
      const double sg = (l % 2 == 0) ? -1.0 : 1.0;
      for (int e = 0; e < 3; ++e) gr[e] = gr[e] + mr(xm, sg * d.gm[(pl[l] + e) * n + f[l]]);
    }
    const double vol = d.gm[GM_GRD * n + g];
    for (int e = 0; e < 3; ++e) d.vfg[e * n + g] = gr[e] / vol;
  }
}

// setbc_vfg (src/bc_module.f90:1398-1804): across each 1-to-1 interface the donor's first
// ghost layer takes the block's first interior layer
__global__ void k_vfg_halo(DevPtr d) {
  const long long n = d.ncell;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= d.nvfg_halo) return;
  const long long src = d.vfg_halo[2 * q], dst = d.vfg_halo[2 * q + 1];
  for (int e = 0; e < 3; ++e) d.vfg[e * n + dst] = d.vfg[e * n + src];
}

// csfsource (src/csf_module.f90:97-175) of interior cell g as calrhs calls it
// (src/rhs_module.f90:607-635): vfg of the cell and its six neighbours, the outward face
// vectors -cx(i-1), cx(i), -ex(j-1), ex(j), -tx(k-1), tx(k).  Below |vfg| = 0.04 there is no
// interface and the source is zero.  The surface tension is the reference's constant
// 0.071684196047 N/m in every cell, so its tangential (Marangoni) part, made of its
// differences, is zero.  out: the five flow components of the source, times the volume.
__device__ void csf_cell(const DevPtr& d, long long g, long long sj, long long sk, double vol, const double* pvc,
                         double* out) {
  const long long n = d.ncell;
  for (int q = 0; q < 5; ++q) out[q] = 0.0;
  const long long nb[7] = {g - 1, g + 1, g - sj, g + sj, g - sk, g + sk, g};
  double v[7][3];
  for (int l = 0; l < 7; ++l)
    for (int e = 0; e < 3; ++e) v[l][e] = d.vfg[e * n + nb[l]];
  const double delta = sqrt(mr(v[6][0], v[6][0]) + mr(v[6][1], v[6][1]) + mr(v[6][2], v[6][2]));
  if (delta <= 0.04) return;
  const double sigma = 0.071684196047;
  double nv[7][3];
  for (int l = 0; l < 7; ++l) {
    const double dl = mr(v[l][0], v[l][0]) + mr(v[l][1], v[l][1]) + mr(v[l][2], v[l][2]);
    for (int e = 0; e < 3; ++e) nv[l][e] = (dl > 0.0) ? v[l][e] / sqrt(dl) : 0.0;
  }
  const long long f[6] = {g - 1, g, g - sj, g, g - sk, g};
  const int pl[6] = {GM_CX, GM_CX, GM_EX, GM_EX, GM_TX, GM_TX};
  double kappa = 0.0;
  for (int m = 0; m < 6; ++m) {
    const double sg = (m % 2 == 0) ? -1.0 : 1.0;
    for (int e = 0; e < 3; ++e) kappa = kappa + mr(0.5 * (nv[6][e] + nv[m][e]), sg * d.gm[(pl[m] + e) * n + f[m]]);
  }
  kappa = -kappa / vol;
  for (int e = 0; e < 3; ++e) out[1 + e] = sigma * kappa * v[6][e];
  out[4] = mr(out[1], pvc[1]) + mr(out[2], pvc[2]) + mr(out[3], pvc[3]);
  for (int q = 0; q < 5; ++q) out[q] = out[q] * vol;
}

// ------------------------------------------------------------------ residual + sources
// REC = false (the explicit schemes): the residual alone, without the sweep records (a
// separate instantiation, so that the LU-SGS kernel carries no branch for it)
// XS (extended sources): the SST destruction with the DES length scale of c.ides, the
// gravity and the surface-tension sources (a separate instantiation, so that the plain kernel carries none of their
// code)
template <bool MX, bool REC = true, bool XS = false>
// The mixed form at 4 CTAs of 256 threads per SM: its residual is latency-bound (the FP64
// pipe about a third busy), and the occupancy buys more than the registers' spills cost
// (measured: 10.8 ms at 1 CTA, 8.1 at 2, 7.4 at 3, 6.6 at 4 on the 14.2 M-cell case).  store_res: the residual, icav and itt planes are written (the residual query and
// the explicit schemes read them); the mixed form's LU-SGS iteration keeps them in
// registers, and only the sweep record and x0 carry them on.
__global__ void __launch_bounds__(256, MX ? 4 : 1) k_rhs(DevPtr d, Par c, long long t0, long long t1, int store_res) {
  long long t = t0 + blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= t1) return;
  const bool out = !(MX && REC) || store_res != 0;
  int b = find_block_interior(d.blk, d.nblk, t), i, j, k;
  const BlockGeom& B = d.blk[b];
  long long g = interior_cell(B, t - B.int_off, i, j, k);
  const long long n = d.ncell, sj = B.ni, sk = (long long)B.ni * B.nj;
  const int npv = c.npv;
  const bool vis = c.iturb != -3;
  const long long st[3] = {1, sj, sk};
  double res[NPVM];
  if (MX) {
    // the stored FP32 fluxes are deviations from the free-stream flux: their differences
    // and sums in FP32 carry rounding of the order of the storage's own (one conversion to
    // FP64 per variable instead of one per stored value)
#pragma unroll
    for (int v = 0; v < NPVM; ++v) {
      res[v] = 0.0;
      if (v >= npv) continue;
      float r = 0.0f;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float* F = d.fi32 + ((long long)q * npv + v) * n;
        r -= F[g] - F[g - st[q]];
        if (vis) {
          const float* V = d.fv32 + ((long long)q * npv + v) * n;
          r += V[g] - V[g - st[q]];
        }
      }
      res[v] = (double)r;
    }
  }
  for (int v = 0; v < npv && !MX; ++v) {
    double r = 0.0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double f1, f0;
      if (MX) {
        const float* F = d.fi32 + ((long long)q * npv + v) * n;
        f1 = F[g]; f0 = F[g - st[q]];
      } else {
        const double* F = d.fi + ((long long)q * npv + v) * n;
        f1 = F[g]; f0 = F[g - st[q]];
      }
      if (q == 0) r = -(f1 - f0);
      else r = r - (f1 - f0);
      if (vis) {
        double v1, v0;
        if (MX) {
          const float* V = d.fv32 + ((long long)q * npv + v) * n;
          v1 = V[g]; v0 = V[g - st[q]];
        } else {
          const double* V = d.fv + ((long long)q * npv + v) * n;
          v1 = V[g]; v0 = V[g - st[q]];
        }
        r = r + (v1 - v0);
      }
    }
    res[v] = r;
  }
  if (MX) {
    // the stored mixed-form fluxes are F - (Phi + pref I).n dl: the free-stream part comes
    // back through the cell's face-vector sum (zero up to the metrics' closure error),
    // formed once by k_closure
#pragma unroll
    for (int v = 0; v < NPVM; ++v)
      if (v < npv) res[v] -= d.clo[v * n + g];
  }
  double pv2[NPVM], dv[NDV];
#pragma unroll
  for (int v = 0; v < NPVM; ++v) pv2[v] = (v < npv) ? d.pv[v * n + g] : 0.0;
  for (int v = 0; v < NDV; ++v) dv[v] = d.dv[v * n + g];
  const double vol = d.gm[GM_GRD * n + g];
  // the FP64 sources first (the dual-time source, the extended sources): after them the
  // mixed form needs only the FP32 copies of the state
  if (c.nsteady >= 1) {
    double bb = (c.nsteady == 1) ? 1.0 : 0.75;
    const double vdt = vol / c.dt_phy;
    double fx[NPVM];
    fx[0] = dv[0];
    fx[1] = dv[0] * pv2[1]; fx[2] = dv[0] * pv2[2]; fx[3] = dv[0] * pv2[3];
    fx[4] = dv[0] * (dv[1] + 0.5 * (pv2[1] * pv2[1] + pv2[2] * pv2[2] + pv2[3] * pv2[3])) - (pv2[0] + c.pref);
#pragma unroll
    for (int v = 5; v < NPVM; ++v) fx[v] = dv[0] * pv2[v];
#pragma unroll
    for (int v = 0; v < NPVM; ++v) {
      if (v >= npv) continue;
      double q1 = d.qq[v * n + g], q2 = d.qq[(npv + v) * n + g];
      double s = (double)c.nsteady * (bb * fx[v] - q1) + 0.5 * ((double)c.nsteady - 1.0) * q2;
      res[v] = res[v] - s * vdt;
    }
  }
  if (XS && c.gravity) {
    // gravity%getgravitysource (src/gravity_module.f90:110-131) at the residual's time
    double a[3];
    gravity_at(d.grav, bc_time(d, c), a);
    const double rv = dv[0] * vol;
    for (int e = 0; e < 3; ++e) res[1 + e] = res[1 + e] + rv * a[e];
    res[4] = res[4] + rv * (a[0] * pv2[1] + a[1] * pv2[2] + a[2] * pv2[3]);
  }
  if (XS && c.rot) {
    // rotation%getrotationsource (src/rotation_module.f90:75-97), subtracted
    // (src/rhs_module.f90:600-605): rho vol (2 omega x u + omega x (omega x r))
    const double* w = c.omega;
    double r[3];
    for (int e = 0; e < 3; ++e) r[e] = d.gm[(GM_GRD + 1 + e) * n + g];
    const double cor[3] = {2.0 * (w[1] * pv2[3] - w[2] * pv2[2]), 2.0 * (w[2] * pv2[1] - w[0] * pv2[3]),
                           2.0 * (w[0] * pv2[2] - w[1] * pv2[1])};
    const double cen[3] = {w[0] * (w[1] * r[1] + w[2] * r[2]) - r[0] * (w[1] * w[1] + w[2] * w[2]),
                           w[1] * (w[0] * r[0] + w[2] * r[2]) - r[1] * (w[0] * w[0] + w[2] * w[2]),
                           w[2] * (w[0] * r[0] + w[1] * r[1]) - r[2] * (w[0] * w[0] + w[1] * w[1])};
    for (int e = 0; e < 3; ++e) res[1 + e] = res[1 + e] - dv[0] * vol * (cor[e] + cen[e]);
  }
  if (XS && c.csf) {
    double cs[5];
    csf_cell(d, g, sj, sk, vol, pv2, cs);
    for (int q = 0; q < 5; ++q) res[q] = res[q] + cs[q];
    for (int e = 0; e < 3; ++e) d.csf[e * n + g] = cs[1 + e];
  }
  // the mixed form's FP32 copies of the state, made once (its cavitation source, diagonal
  // block and tile record read them), and its sources' FP32 implicit coefficients, kept in
  // registers for the diagonal block
  float p2f[NPVM], dvf[NDV], tvf[3] = {0.0f, 0.0f, 0.0f};
  float icf[4] = {0.0f, 0.0f, 0.0f, 0.0f}, itf[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  if (MX) {
#pragma unroll
    for (int q = 0; q < NPVM; ++q) p2f[q] = (float)pv2[q];
#pragma unroll
    for (int q = 0; q < NDV; ++q) dvf[q] = (float)dv[q];
#pragma unroll
    for (int q = 0; q < 3; ++q)
      if (q < c.ntv) tvf[q] = (float)d.tv[q * n + g];
  }
  const float volf = MX ? d.gmf[GM_GRD * n + g] : 0.0f;
  if (c.ncav) {
    if (MX) {
      // FP32 source (its rates reach the residual to ~1e-7 of their size) with the
      // saturation pressure / temperature in FP64 (a df64 saturation pressure measured
      // slower here: its quotients and root cost more FP32 issue than the FP64 pipe frees)
      double sat[2] = {0.0, 0.0};
      if (pv2[4] < 647.096) {
        if (c.ncav == 5) sat[1] = h2o_tww(pv2[0] + c.pref);
        else sat[0] = h2o_pww(pv2[4]);
      }
      const CavOutT<float> o = cavsource_t<float>(c, p2f, dvf, vol, (float)c.uref, (float)c.c_v, (float)c.c_c, sat);
      res[5] = res[5] + (double)o.r_v - (double)o.r_c;
      for (int q = 0; q < 4; ++q) { if (out) d.icav[q * n + g] = o.icav[q]; icf[q] = o.icav[q]; }
      d.rcav[g] = o.r_c;
      d.rcav[n + g] = o.r_v;
    } else {
      CavOut o = cavsource(c, pv2, dv, vol);
      res[5] = res[5] + o.r_v - o.r_c;
      for (int q = 0; q < 4; ++q) d.icav[q * n + g] = o.icav[q];
      d.rcav[g] = o.r_c;
      d.rcav[n + g] = o.r_v;
    }
  }
  if (c.iturb == 0) {
    // cell-centred gradients of u, v, w, k, omega (turbsource kwsst, :269-383)
    const long long nbr[6] = {g - 1, g + 1, g - sj, g + sj, g - sk, g + sk};
    const int gv[5] = {1, 2, 3, 7, 8};
    const double c23 = 2.0 / 3.0;
    if (MX) {
      // FP32 on the gauge shadow: differences of u - U are exact where u's are not
      float faf[6][3];
      for (int q = 0; q < 3; ++q) {
        faf[0][q] = d.gmf[(GM_CX + q) * n + g - 1]; faf[1][q] = d.gmf[(GM_CX + q) * n + g];
        faf[2][q] = d.gmf[(GM_EX + q) * n + g - sj]; faf[3][q] = d.gmf[(GM_EX + q) * n + g];
        faf[4][q] = d.gmf[(GM_TX + q) * n + g - sk]; faf[5][q] = d.gmf[(GM_TX + q) * n + g];
      }
      float grf[5][3];
      const float ivf = 1.0f / volf;
      for (int q = 0; q < 5; ++q) {
        const float* P = d.pvf + gv[q] * n;
        const float c0 = P[g];
        float vv[6];
        for (int m = 0; m < 6; ++m) vv[m] = 0.5f * (P[nbr[m]] + c0);
        for (int e = 0; e < 3; ++e)
          grf[q][e] = (vv[1] * faf[1][e] + vv[3] * faf[3][e] + vv[5] * faf[5][e] -
                       vv[0] * faf[0][e] - vv[2] * faf[2][e] - vv[4] * faf[4][e]) * ivf;
      }
      const double hmax = (XS && c.ides) ? grid_hmax<float>(faf, vol) : 0.0;
      const float kf = p2f[7], of = p2f[8], rho = dvf[0];
      const SstOut<float> sf = sst_source_f(grf, kf, of, rho, tvf[0], tvf[2], d.gmf[(GM_GRD + 4) * n + g], volf,
                                            XS ? c.ides : 0, hmax);
      res[7] = res[7] + (double)sf.r7;
      res[8] = res[8] + (double)sf.r8;
      // the implicit coefficients and the omega bound of the update: FP32
      const float pf = sf.prod, df_ = sf.dest, dvf_ = sf.div, pkf = sf.pkw, bf = sf.bigf;
      const float taf = sf.talpha, tbf = sf.tbeta;
      d.ocut[g] = (double)sqrtf(sf.strain - (2.0f / 3.0f) * dvf_ * dvf_);
      const float ki = 1.0f / kf, oi = 1.0f / of, ei = 1.0f / tvf[2];
      const float dpdk = pf * ki;
      const float dpdo = -((pf + (2.0f / 3.0f) * rho * kf * dvf_) * oi);
      const float it0 = dpdk - df_ * ki, it1 = dpdo - df_ * oi, it2 = 0.0f;
      const float it3 = taf * rho * ei * dpdo + taf * rho * ei * pf * oi - 2.0f * tbf * rho * of -
                        1.712f * (1.0f - bf) * rho * oi * oi * pkf;
      // the signs of the block's eigenvalues 0.5 tr +- sqrt(0.25 tr^2 - det): with it2 = 0
      // these are max(it0, it3) and min(it0, it3).  Taken from those directly: in FP32 the
      // difference 0.5 tr - sqrt(..) cancels catastrophically next to walls, where omega
      // makes it3 ~ 1e12 against it0 ~ 1e4, and its sign comes out at random.
      const float l1 = copysignf(1.0f, fmaxf(it0, it3)), l2 = copysignf(1.0f, fminf(it0, it3));
      const float f1 = (1.0f - 0.5f * (1.0f - l1)) - 0.5f * (1.0f - l1);
      const float f2 = (1.0f - 0.5f * (1.0f - l2)) - 0.5f * (1.0f - l2);
      itf[0] = it0 * f1; itf[1] = it1 * f1; itf[2] = it2 * f2; itf[3] = it3 * f2;
      if (out) for (int q = 0; q < 4; ++q) d.itt[q * n + g] = itf[q];
    } else {
      double tv[3];
      for (int q = 0; q < 3; ++q) tv[q] = d.tv[q * n + g];
      const double kk = pv2[7], oo = pv2[8];
      const double y5 = d.gm[(GM_GRD + 4) * n + g];
      double fa[6][3];
      for (int q = 0; q < 3; ++q) {
        fa[0][q] = d.gm[(GM_CX + q) * n + g - 1]; fa[1][q] = d.gm[(GM_CX + q) * n + g];
        fa[2][q] = d.gm[(GM_EX + q) * n + g - sj]; fa[3][q] = d.gm[(GM_EX + q) * n + g];
        fa[4][q] = d.gm[(GM_TX + q) * n + g - sk]; fa[5][q] = d.gm[(GM_TX + q) * n + g];
      }
      double gr[5][3];
      double ivol = 1.0 / vol;
      for (int q = 0; q < 5; ++q) {
        const double* P = d.pv + gv[q] * n;
        double c0 = P[g];
        double v1 = 0.5 * (P[nbr[0]] + c0), v2 = 0.5 * (P[nbr[1]] + c0), v3 = 0.5 * (P[nbr[2]] + c0);
        double v4 = 0.5 * (P[nbr[3]] + c0), v5 = 0.5 * (P[nbr[4]] + c0), v6 = 0.5 * (P[nbr[5]] + c0);
        for (int e = 0; e < 3; ++e)
          gr[q][e] = (v2 * fa[1][e] + v4 * fa[3][e] + v6 * fa[5][e] - v1 * fa[0][e] - v3 * fa[2][e] - v5 * fa[4][e]) * ivol;
      }
      const double hmax = (XS && c.ides) ? grid_hmax<double>(fa, vol) : 0.0;
      const SstOut<double> so = sst_source<double>(gr, kk, oo, dv[0], tv[0], tv[2], y5, vol, XS ? c.ides : 0, hmax);
      res[7] = res[7] + so.r7;
      res[8] = res[8] + so.r8;
      const double prod = so.prod, dest = so.dest, div = so.div, pkw = so.pkw, bigf = so.bigf;
      const double talpha = so.talpha, tbeta = so.tbeta;
      d.ocut[g] = sqrt(so.strain - c23 * so.div * so.div);
      const double ki = 1.0 / kk, oi = 1.0 / oo, ei = 1.0 / tv[2];
      double dpdk = prod * ki;
      double dpdo = -((prod + c23 * dv[0] * kk * div) * oi);
      double it0 = dpdk - dest * ki, it1 = dpdo - dest * oi, it2 = 0.0;
      double it3 = talpha * dv[0] * ei * dpdo + talpha * dv[0] * ei * prod * oi - 2.0 * tbeta * dv[0] * oo -
                   1.712 * (1.0 - bigf) * dv[0] * oi * oi * pkw;
      double tr = it0 + it3, de = it0 * it3 - it1 * it2;
      double sd = sqrt(fmax(0.25 * tr * tr - de, 0.0));
      double l1 = copysign(1.0, 0.5 * tr + sd), l2 = copysign(1.0, 0.5 * tr - sd);
      double f1 = (1.0 - 0.5 * (1.0 - l1)) - 0.5 * (1.0 - l1);
      double f2 = (1.0 - 0.5 * (1.0 - l2)) - 0.5 * (1.0 - l2);
      d.itt[g] = it0 * f1; d.itt[n + g] = it1 * f1; d.itt[2 * n + g] = it2 * f2; d.itt[3 * n + g] = it3 * f2;
    }
  }
  if (c.iturb == -1) {
    // k-epsilon source (FP64 in both forms); no omega bound
    const long long nbr[6] = {g - 1, g + 1, g - sj, g + sj, g - sk, g + sk};
    double fa[6][3];
    for (int q = 0; q < 3; ++q) {
      fa[0][q] = d.gm[(GM_CX + q) * n + g - 1]; fa[1][q] = d.gm[(GM_CX + q) * n + g];
      fa[2][q] = d.gm[(GM_EX + q) * n + g - sj]; fa[3][q] = d.gm[(GM_EX + q) * n + g];
      fa[4][q] = d.gm[(GM_TX + q) * n + g - sk]; fa[5][q] = d.gm[(GM_TX + q) * n + g];
    }
    const double ivol = 1.0 / vol;
    double gr[3][3], gsk[3];
    for (int q = 0; q < 4; ++q) {
      const double* P = d.pv + (q < 3 ? 1 + q : 7) * n;
      const double c0 = P[g];
      double vv[6];
      for (int m = 0; m < 6; ++m) vv[m] = 0.5 * (P[nbr[m]] + c0);
      if (q == 3) for (int m = 0; m < 6; ++m) vv[m] = sqrt(vv[m]);
      double* o = (q < 3) ? gr[q] : gsk;
      for (int e = 0; e < 3; ++e)
        o[e] = (vv[1] * fa[1][e] + vv[3] * fa[3][e] + vv[5] * fa[5][e] - vv[0] * fa[0][e] - vv[2] * fa[2][e] -
                vv[4] * fa[4][e]) * ivol;
    }
    double rk[2], itk[4];
    ke_source<double>(gr, gsk, pv2[7], pv2[8], dv[0], d.tv[g], d.tv[2 * n + g], vol, rk, itk);
    res[7] = res[7] + rk[0];
    res[8] = res[8] + rk[1];
    for (int q = 0; q < 4; ++q) { if (out) d.itt[q * n + g] = itk[q]; itf[q] = (float)itk[q]; }
    d.ocut[g] = 0.0;
  }
#pragma unroll
  for (int v = 0; v < NPVM; ++v)
    if (out && v < npv) d.res[v * n + g] = res[v];
  if constexpr (!REC) return;   // the explicit schemes need no sweep records
  if (c.rot) {
    // the implicit operator's enthalpy is the rothalpy (lhs%getenthalpy, jac%getenthalpy):
    // the diagonal block below and the neighbours' products read it from the record's dv(2)
    double r[3];
    for (int e = 0; e < 3; ++e) r[e] = d.gm[(GM_GRD + 1 + e) * n + g];
    dv[1] = dv[1] - rot_q(c, r);
    if (MX) dvf[1] = (float)dv[1];
  }
  // ---- LU-SGS coefficients of this cell (diagonal block, spectral radii, beta, viscous
  // term), written with its state and residual as the cell's sweep record
  // face vectors cx1, cx2, ex1, ex2, tx1, tx2: FP64, or (mixed form) their FP32 copies
  double fc[18];
  float fcf[18];
  for (int q = 0; q < 3; ++q) {
    const long long o6[6] = {(GM_CX + q) * n + g - 1, (GM_CX + q) * n + g, (GM_EX + q) * n + g - sj,
                             (GM_EX + q) * n + g, (GM_TX + q) * n + g - sk, (GM_TX + q) * n + g};
    for (int m = 0; m < 6; ++m) {
      if (MX) fcf[3 * m + q] = d.gmf[o6[m]];
      else fc[3 * m + q] = d.gm[o6[m]];
    }
  }
  const int pvi[7] = {1, 2, 3, 5, 6, 7, 8};
  const int dvi[10] = {0, 1, 6, 7, 8, 9, 10, 11, 12, 13};
  if constexpr (MX) {
    // the diagonal block in FP32: it shapes the implicit operator only (the sweeps' FP32
    // corrections use it as well), and its closed-form inverse gives x0 below
    DiagT<float> Df;
    float lam_fs[2];
    diag_spectral_f(c, p2f, dvf[5], fcf, lam_fs);
    const float evf = eigenvis_f(c, dvf, tvf);
    diag_prepare_t<float>(c, p2f, dvf, evf, fcf, volf, (float)d.dt[g], icf, itf, Df, lam_fs);
    // the cell's tile record (FP32) and the forward sweep's own part x0 = D^-1 res, at its
    // tile slot: consecutive i are consecutive slots.  x0 is an FP32 solve of the FP64
    // residual (rounded once): an inexact step of the iteration, not of its fixed point.
    const long long sl = d.pos[g];
    float rf[NPVM], xf[NPVM];
#pragma unroll
    for (int v = 0; v < NPVM; ++v) { rf[v] = (v < npv) ? (float)res[v] : 0.0f; xf[v] = 0.0f; }
    diag_solve_t<float>(c, Df, p2f, dvf, rf, xf);
    float* R = d.trf + trf_at(sl, 0);
#pragma unroll
    for (int v = 0; v < NPVM; ++v)
      if (v < npv) { d.tq[tq_at(sl, v)] = xf[v]; R[(TR_X + v) * TILE_SLOTS] = xf[v]; }
#pragma unroll
    for (int q = 0; q < 7; ++q) R[(TR_PV + q) * TILE_SLOTS] = (pvi[q] < npv) ? p2f[pvi[q]] : 0.0f;
#pragma unroll
    for (int q = 0; q < 10; ++q) R[(TR_DV + q) * TILE_SLOTS] = dvf[dvi[q]];
    // (the sweeps form beta = rr - (b1 - 1) drho/dp from the block)
    R[TR_EVV * TILE_SLOTS] = 2.0f * evf / volf;
    {
      float od[PREP_DIAG];
      diag_to_array(Df, od);
#pragma unroll
      for (int q = 0; q < PREP_DIAG; ++q) R[(TR_DIAG + q) * TILE_SLOTS] = od[q];
    }
    // the spectral radii only scale the implicit operator: FP32
    for (int dir = 0; dir < 3; ++dir) {
      for (int e = 0; e < 3; ++e) {
        R[(TR_FACEP + 3 * dir + e) * TILE_SLOTS] = fcf[6 * dir + 3 + e];   // cx2, ex2, tx2
        R[(TR_FACEM + 3 * dir + e) * TILE_SLOTS] = fcf[6 * dir + e];       // cx1, ex1, tx1
      }
      R[(TR_SPECP + dir) * TILE_SLOTS] = face_spectral<float>(c, fcf + 3 * (2 * dir + 1), p2f, dvf);
      R[(TR_SPECM + dir) * TILE_SLOTS] = face_spectral<float>(c, fcf + 3 * (2 * dir), p2f, dvf);
    }
  } else {
    double tvc[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < 3; ++q)
      if (q < c.ntv) tvc[q] = d.tv[q * n + g];
    double ic[4] = {0, 0, 0, 0}, it4[4] = {0, 0, 0, 0};
    if (c.ncav) for (int q = 0; q < 4; ++q) ic[q] = d.icav[q * n + g];
    if (c.iturb >= -1) for (int q = 0; q < 4; ++q) it4[q] = d.itt[q * n + g];
    Diag D;
    const double evis = eigenvis_of(c, dv, tvc);
    diag_prepare(c, pv2, dv, evis, fc, vol, d.dt[g], ic, it4, D);
    double o[NREC];
    for (int q = 0; q < NREC; ++q) o[q] = 0.0;
    for (int q = 0; q < 7; ++q) o[REC_PV + q] = (pvi[q] < npv) ? pv2[pvi[q]] : 0.0;
    for (int q = 0; q < 10; ++q) o[REC_DV + q] = dv[dvi[q]];
    diag_to_array(D, o + REC_DIAG);
    for (int q = 0; q < 6; ++q) o[REC_SPEC + q] = face_spectral<double>(c, fc + 3 * q, pv2, dv);
    // beta = 1/sndp2 - 1/c2 + drho/dp = D.rr - (D.b1 - 1) drho/dp
    o[REC_BETA] = D.rr - (D.b1 - 1.0) * dv[6];
    o[REC_EVV] = 2.0 * evis / vol;
    for (int e = 0; e < 3; ++e) { o[REC_FACE + e] = fc[3 + e]; o[REC_FACE + 3 + e] = fc[9 + e]; o[REC_FACE + 6 + e] = fc[15 + e]; }
    for (int v = 0; v < npv; ++v) o[REC_RES + v] = res[v];
    const long long nint = d.nint, tp = d.pos[g];
    for (int q = 0; q < NREC; ++q) d.rec[q * nint + tp] = o[q];
  }
}

// ------------------------------------------------------------------ LU-SGS sweeps
// FP64 form: the sweeps work in the plane-major numbering t (setup_planes).  k_rhs writes
// what they read of each cell -- as itself (diagonal block, residual) and as a neighbour
// (state, split-Jacobian coefficients, + face vectors) -- as the cell's sweep record at t;
// each hyperplane launch then reads its own records and those of the previous (next) plane
// with coalesced loads.  dcv and dqs live at t as well; k_update reads dqs through pos[g].
// The mixed form sweeps by tiles (k_sweep_tile, below).

// a cell's pv / dv as the Jacobian and diagonal routines index them, from its record
template <class T>
__device__ __forceinline__ void rec_state(const T* R, long long nint, long long t, T* pv, T* dv) {
  pv[0] = T(0); pv[4] = T(0);
  pv[1] = R[(REC_PV + 0) * nint + t]; pv[2] = R[(REC_PV + 1) * nint + t]; pv[3] = R[(REC_PV + 2) * nint + t];
  pv[5] = R[(REC_PV + 3) * nint + t]; pv[6] = R[(REC_PV + 4) * nint + t];
  pv[7] = R[(REC_PV + 5) * nint + t]; pv[8] = R[(REC_PV + 6) * nint + t];
  dv[0] = R[(REC_DV + 0) * nint + t]; dv[1] = R[(REC_DV + 1) * nint + t];
  dv[2] = dv[3] = dv[4] = dv[5] = T(0);
#pragma unroll
  for (int q = 0; q < 8; ++q) dv[6 + q] = R[(REC_DV + 2 + q) * nint + t];
}

// the three lower (forward) or upper (backward) neighbours' products, added to acc
template <bool FWD, bool CG = false>
__device__ __forceinline__ void sweep_neighbours(const DevPtr& d, int npv, long long t, double* acc) {
  const long long nint = d.nint;
  const double* R = d.rec;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    // forward: lower neighbour through its + face; backward: upper neighbour through this
    // cell's + face.  Neighbours outside the block carry dq = 0.
    const int nb = FWD ? d.nbf[q * nint + t] : d.nbb[q * nint + t];
    if (nb < 0) continue;
    const long long fr = FWD ? nb : t;
    double nx[3], pv[NPVM], dv[14], dq[NPVM];
    for (int e = 0; e < 3; ++e) nx[e] = R[(REC_FACE + 3 * q + e) * nint + fr];
    rec_state<double>(R, nint, nb, pv, dv);
    // the dataflow sweep reads dq written during this launch by other CTAs: from L2 (CG)
    for (int v = 0; v < NPVM; ++v) dq[v] = (v < npv) ? (CG ? __ldcg(d.dqs + v * nint + nb) : d.dqs[v * nint + nb]) : 0.0;
    const double spec = R[(REC_SPEC + 2 * q + (FWD ? 1 : 0)) * nint + nb];
    const double beta = R[REC_BETA * nint + nb];
    const double evv = R[REC_EVV * nint + nb];
    jac_apply_pre<double>(npv, nx, pv, dv, spec, beta, evv, FWD ? 1.0 : -1.0, dq, acc);
  }
}

// one cell of a sweep: its three neighbours' products, the closed-form D^-1, dq
template <bool FWD, bool CG>
__device__ __forceinline__ void sweep_cell(const DevPtr& d, const Par& c, long long t) {
  const long long nint = d.nint;
  const double* R = d.rec;
  const int npv = c.npv;
  double pv[NPVM], dv[14], o[PREP_DIAG], acc[NPVM], x[NPVM];
  rec_state<double>(R, nint, t, pv, dv);
  for (int q = 0; q < PREP_DIAG; ++q) o[q] = R[(REC_DIAG + q) * nint + t];
  for (int v = 0; v < NPVM; ++v) { acc[v] = 0.0; x[v] = 0.0; }
  if (FWD) for (int v = 0; v < npv; ++v) acc[v] = R[(REC_RES + v) * nint + t];
  else for (int v = 0; v < npv; ++v) acc[v] = d.dcv[v * nint + t];
  sweep_neighbours<FWD, CG>(d, npv, t, acc);
  if (FWD) for (int v = 0; v < npv; ++v) d.dcv[v * nint + t] = acc[v];
  Diag D;
  diag_from_array(o, D);
  diag_solve(c, D, pv, dv, acc, x);
  for (int v = 0; v < npv; ++v) d.dqs[v * nint + t] = x[v];
}

// one launch per hyperplane
template <bool FWD>
__global__ void __launch_bounds__(64) k_sweep(DevPtr d, Par c, long long p0, long long p1) {
  const long long t = p0 + blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= p1) return;
  sweep_cell<FWD, false>(d, c, t);
}

// the dataflow sweeps' done flags: a release store by one thread after a barrier publishes
// what the barrier ordered before it (release is cumulative), an acquire load followed by a
// barrier makes it visible to the threads that passed the barrier
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// a bounded wait for a done flag: gives up (recording sweep_stall, which ends every other
// wait too) after `spin` polls
__device__ __forceinline__ void wait_flag(const DevPtr& d, const int* flag, long long spin) {
  long long it = 0;
  while (ld_acquire(flag) == 0) {
    ++it;
    if ((it & 63) == 0 && *(volatile int*)&d.sc->sweep_stall) break;
    if (it > spin) { atomicExch(&d.sc->sweep_stall, 1); break; }
    if (it > 8) __nanosleep(32);
  }
}

// what a dataflow sweep cell reads of one neighbour before its dq is known
struct SweepNb {
  int nb;
  double nx[3], pv[NPVM], dv[14], spec, beta, evv;
};

template <bool FWD>
__device__ __forceinline__ void sweep_nb_load(const DevPtr& d, long long t, int q, SweepNb& s) {
  const long long nint = d.nint;
  const double* R = d.rec;
  s.nb = FWD ? d.nbf[q * nint + t] : d.nbb[q * nint + t];
  if (s.nb < 0) return;
  const long long fr = FWD ? s.nb : t;
  for (int e = 0; e < 3; ++e) s.nx[e] = R[(REC_FACE + 3 * q + e) * nint + fr];
  rec_state<double>(R, nint, s.nb, s.pv, s.dv);
  s.spec = R[(REC_SPEC + 2 * q + (FWD ? 1 : 0)) * nint + s.nb];
  s.beta = R[REC_BETA * nint + s.nb];
  s.evv = R[REC_EVV * nint + s.nb];
}

template <bool FWD>
__device__ __forceinline__ void sweep_nb_apply(const DevPtr& d, int npv, const SweepNb& s, double* acc) {
  if (s.nb < 0) return;
  const long long nint = d.nint;
  double dq[NPVM];
  for (int v = 0; v < NPVM; ++v) dq[v] = (v < npv) ? __ldcg(d.dqs + v * nint + s.nb) : 0.0;
  jac_apply_pre<double>(npv, s.nx, s.pv, s.dv, s.spec, s.beta, s.evv, FWD ? 1.0 : -1.0, dq, acc);
}

// Dataflow sweep of the FP64 form: one persistent launch per sweep.  CTAs take chunks
// (runs of at most SW_CH cells of one plane) in plane order -- reversed for the backward
// sweep -- from a ticket counter.  A chunk's cells need the dq of their lower (upper)
// neighbours, which lie in a few chunks of the previous (next) plane.  Each cell first
// loads everything that does not depend on those dq (its own record, the neighbours'
// records); then the CTA waits for the needed chunks' done flags (one polling thread per
// flag), runs the hyperplane kernel's arithmetic and raises its own chunk's flag.  The
// needed chunks always hold earlier tickets, so the earliest unfinished chunk never waits
// and its CTA is running: the waits end.  Each wait is still bounded by `spin` polls; a
// wait that runs out records sweep_stall, which also ends every other wait, so the launch
// completes and the host reports CFD3D_ERR_TIMEOUT.  `withhold` >= 0 names a chunk whose
// flag is never raised (the stall test).
template <bool FWD>
__global__ void __launch_bounds__(SW_CH) k_sweep_df(DevPtr d, Par c, long long spin, int withhold) {
  __shared__ int s_q, s_lo[SW_CH / 32], s_hi[SW_CH / 32];
  const long long nint = d.nint;
  const int npv = c.npv;
  unsigned* ticket = d.tickets + (FWD ? 0 : 1);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_q = (int)atomicAdd(ticket, 1u);
    __syncthreads();
    const int q = s_q;
    if (q >= d.nchunk) return;
    const int ch = FWD ? q : d.nchunk - 1 - q;
    const long long t = d.chunk_t0[ch] + threadIdx.x;
    const bool live = t < d.chunk_t0[ch + 1];
    // ---- work that does not wait: own record, neighbour records, the needed chunks
    SweepNb nbs[3];
    double acc[NPVM], pv[NPVM], dv[14], o[PREP_DIAG];
    int lo = 0x7fffffff, hi = -1;
    if (live) {
      const double* R = d.rec;
      rec_state<double>(R, nint, t, pv, dv);
      for (int k = 0; k < PREP_DIAG; ++k) o[k] = R[(REC_DIAG + k) * nint + t];
      for (int v = 0; v < NPVM; ++v) acc[v] = 0.0;
      if (FWD) for (int v = 0; v < npv; ++v) acc[v] = R[(REC_RES + v) * nint + t];
      else for (int v = 0; v < npv; ++v) acc[v] = d.dcv[v * nint + t];
      for (int k = 0; k < 3; ++k) {
        sweep_nb_load<FWD>(d, t, k, nbs[k]);
        if (nbs[k].nb >= 0) {
          const int cn = d.chunk_of[nbs[k].nb];
          lo = min(lo, cn);
          hi = max(hi, cn);
        }
      }
    }
    for (int k = 16; k > 0; k >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, k));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, k));
    }
    if (lane == 0) { s_lo[wid] = lo; s_hi[wid] = hi; }
    __syncthreads();
    for (int w = 0; w < SW_CH / 32; ++w) { lo = min(lo, s_lo[w]); hi = max(hi, s_hi[w]); }
    // ---- wait: thread k polls chunks lo + k, lo + k + SW_CH, ... (none when no cell of
    // the chunk has a neighbour: then hi = -1 and lo is not a chunk index)
    for (int cn = (hi >= 0) ? lo + (int)threadIdx.x : 0; hi >= 0 && cn <= hi; cn += SW_CH) wait_flag(d, d.done + cn, spin);
    __syncthreads();
    if (live) {
      double x[NPVM];
      for (int k = 0; k < 3; ++k) sweep_nb_apply<FWD>(d, npv, nbs[k], acc);
      if (FWD) for (int v = 0; v < npv; ++v) d.dcv[v * nint + t] = acc[v];
      Diag D;
      diag_from_array(o, D);
      for (int v = 0; v < NPVM; ++v) x[v] = 0.0;
      diag_solve(c, D, pv, dv, acc, x);
      for (int v = 0; v < npv; ++v) d.dqs[v * nint + t] = x[v];
    }
    __syncthreads();
    if (threadIdx.x == 0 && ch != withhold) st_release(d.done + ch, 1);
  }
}

// ---- the mixed form's tile sweeps -----------------------------------------------------
// Since D^-1 is linear, a sweep's dq splits into the cell's own part and D^-1 applied to
// the neighbours' FP32 products:
//   forward   dq* = D^-1 (res + sum A+ dq*)  = x0 + y_f,   y_f = D^-1 (sum A+ dq*),   x0 = D^-1 res
//   backward  dq  = D^-1 (dcv - sum A- dq)   = dq* + y_b,  y_b = D^-1 (- sum A- dq)   (D^-1 dcv = dq*)
// k_rhs writes x0 (FP32) into tq and into the cell's tile record; the sweeps work in FP32
// alone -- the products take dq in FP32 -- and store their corrections y_f, y_b; the update
// forms dq = x0 + y_f + y_b and adds it to pv in FP64.  (On a GB300 each FP64 instruction
// holds a warp for tens of cycles: none stays on the sweeps' dependency chain.)  One warp sweeps one tile at a
// time (tiles from a ticket counter in tile-hyperplane order, reversed for the backward
// sweep): it stages the tile's records in shared memory with one bulk copy per array
// (cp.async.bulk, completion on an mbarrier), waits for the done flags of the (at most
// three) tiles it depends on, reads the contributions they left at its faces, and then
// walks the tile's hyperplanes: lane (lj, lk) holds cell (s - lj - lk, lj, lk) at step s.
// Each cell forms its products A.dq for its three downstream neighbours (its outgoing
// contributions) once its dq is known: the +i one stays in the lane for its next cell, the
// +j and +k ones move to lanes +1 and +TILE_J by shuffles, and those leaving the tile go to
// the downstream tile's entry block (tin).  So only FP32 arithmetic, shuffles and the done
// flags between tiles lie on the sweep's dependency chain.  The waits are bounded as in the
// FP64 form's dataflow sweep; `withhold` >= 0 names a tile whose flag is never raised (the
// stall test).
constexpr unsigned TILE_B32 = TS_FIELDS * TILE_SLOTS * 4;   // the FP32 fields one sweep reads
constexpr unsigned TILE_BIN = NPVM * TILE_IN * 4;           // the entering contributions
constexpr unsigned TILE_SMEM = TILE_B32 + TILE_BIN + 16;
static_assert(TILE_B32 % 16 == 0 && (TR_COMMON * TILE_SLOTS * 4) % 16 == 0, "bulk copies move multiples of 16 bytes");

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" : : "r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long* bar, unsigned bytes) {
  asm volatile("{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1; }"
               : : "r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
               : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               : : "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

template <bool FWD>
__global__ void __launch_bounds__(32) k_sweep_tile(DevPtr d, Par c, long long spin, int withhold) {
  extern __shared__ __align__(128) unsigned char smem[];
  float* S32 = reinterpret_cast<float*>(smem);
  float* SIN = reinterpret_cast<float*>(smem + TILE_B32);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + TILE_B32 + TILE_BIN);
  const int lane = threadIdx.x, npv = c.npv;
  const int lj = lane % TILE_J, lk = lane / TILE_J;
  const float sgn = FWD ? 1.0f : -1.0f;
  unsigned* ticket = d.tickets + (FWD ? 0 : 1);
  if (lane == 0) mbar_init(bar);
  __syncwarp();
  unsigned parity = 0;
  for (;;) {
    int q = 0;
    if (lane == 0) q = (int)atomicAdd(ticket, 1u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= d.ntile) break;
    const int tile = FWD ? q : d.ntile - 1 - q;
    const TileDesc T = d.tiles[tile];
    // ---- stage the tile's records (written by earlier launches): the common fields and
    // this sweep's faces and spectral radii
    if (lane == 0) {
      // the previous tile's shared-memory reads (generic proxy) before the bulk writes
      asm volatile("fence.proxy.async.shared::cta;" : : : "memory");
      mbar_expect(bar, TILE_B32);
      const float* rf = d.trf + (long long)tile * NTR * TILE_SLOTS;
      bulk_load(S32, rf, TR_COMMON * TILE_SLOTS * 4, bar);
      bulk_load(S32 + TR_COMMON * TILE_SLOTS, rf + (FWD ? TR_FACEP : TR_FACEM) * TILE_SLOTS, 12 * TILE_SLOTS * 4, bar);
    }
    // ---- the tiles this one depends on, then the contributions they left at its faces
    // (the tiles before and after, as scalars: no indexing into the descriptor)
    const int dep0 = FWD ? T.lo[0] : T.hi[0], dep1 = FWD ? T.lo[1] : T.hi[1], dep2 = FWD ? T.lo[2] : T.hi[2];
    const int nxt0 = FWD ? T.hi[0] : T.lo[0], nxt1 = FWD ? T.hi[1] : T.lo[1], nxt2 = FWD ? T.hi[2] : T.lo[2];
    {
      const int mine = (lane == 0) ? dep0 : (lane == 1) ? dep1 : (lane == 2) ? dep2 : -1;
      if (mine >= 0) wait_flag(d, d.done + mine, spin);
    }
    __syncwarp();
    {
      const float* in = d.tin + (long long)tile * NPVM * TILE_IN;
      for (int e = lane; e < NPVM * TILE_IN; e += 32) SIN[e] = __ldcg(in + e);
    }
    // ---- the staged records (the copy completes by itself: the wait is bounded only as a
    // guard, and on a timeout the tile's cells are skipped)
    bool staged = false;
    for (long long it = 0; it < (1ll << 26); ++it)
      if (mbar_test(bar, parity)) { staged = true; break; }
    parity ^= 1u;
    __syncwarp();
    if (!staged) atomicExch(&d.sc->sweep_stall, 1);
    // ---- the tile's hyperplanes
    const int ni = T.ni, nj = T.nj, nk = T.nk;
    const bool col = lj < nj && lk < nk && staged;
    // faces with a tile beyond them: the others (block faces) bring no contribution
    const bool hi_ = dep0 >= 0, hj_ = dep1 >= 0, hk_ = dep2 >= 0;
    // lane's sweep-local column coordinates (reversed in the backward sweep)
    const int pj = FWD ? lj : nj - 1 - lj, pk = FWD ? lk : nk - 1 - lk;
    float ci[NPVM], cj[NPVM], ck[NPVM];
#pragma unroll
    for (int v = 0; v < NPVM; ++v) ci[v] = cj[v] = ck[v] = 0.0f;
    const int nsteps = ni + nj + nk - 2;
    for (int s = 0; s < nsteps; ++s) {
      // the +j / +k contributions of the previous step from the neighbouring columns
      float rj[NPVM], rk[NPVM];
#pragma unroll
      for (int v = 0; v < NPVM; ++v) {
        rj[v] = FWD ? __shfl_up_sync(0xffffffffu, cj[v], 1) : __shfl_down_sync(0xffffffffu, cj[v], 1);
        rk[v] = FWD ? __shfl_up_sync(0xffffffffu, ck[v], TILE_J) : __shfl_down_sync(0xffffffffu, ck[v], TILE_J);
      }
      const int pi = s - pj - pk;   // sweep-local i of the lane's cell
      if (col && pi >= 0 && pi < ni) {
        const int li = FWD ? pi : ni - 1 - pi;
        const int sl = lane * TILE_LS + li;
        // entering contributions: from the tile's face, or from this tile's cells
        float acc[NPVM];
        const bool fi = pi == 0, fj = pj == 0, fk = pk == 0;
#pragma unroll
        for (int v = 0; v < NPVM; ++v) {
          const float a0 = fi ? (hi_ ? SIN[v * TILE_IN + lj + TILE_J * lk] : 0.0f) : ci[v];
          const float a1 = fj ? (hj_ ? SIN[v * TILE_IN + TILE_IN_J + TILE_I * lk + li] : 0.0f) : rj[v];
          const float a2 = fk ? (hk_ ? SIN[v * TILE_IN + TILE_IN_K + TILE_I * lj + li] : 0.0f) : rk[v];
          acc[v] = (a0 + a1) + a2;
        }
        // the cell's state and diagonal block (FP32), D^-1 acc, dq = own part + it
        float pv[NPVM], dv[14], od[PREP_DIAG];
        pv[0] = 0.0f; pv[4] = 0.0f;
        pv[1] = S32[(TR_PV + 0) * TILE_SLOTS + sl]; pv[2] = S32[(TR_PV + 1) * TILE_SLOTS + sl];
        pv[3] = S32[(TR_PV + 2) * TILE_SLOTS + sl]; pv[5] = S32[(TR_PV + 3) * TILE_SLOTS + sl];
        pv[6] = S32[(TR_PV + 4) * TILE_SLOTS + sl]; pv[7] = S32[(TR_PV + 5) * TILE_SLOTS + sl];
        pv[8] = S32[(TR_PV + 6) * TILE_SLOTS + sl];
        dv[0] = S32[(TR_DV + 0) * TILE_SLOTS + sl]; dv[1] = S32[(TR_DV + 1) * TILE_SLOTS + sl];
        dv[2] = dv[3] = dv[4] = dv[5] = 0.0f;
#pragma unroll
        for (int m = 0; m < 8; ++m) dv[6 + m] = S32[(TR_DV + 2 + m) * TILE_SLOTS + sl];
#pragma unroll
        for (int m = 0; m < PREP_DIAG; ++m) od[m] = S32[(TR_DIAG + m) * TILE_SLOTS + sl];
        DiagT<float> D;
        D.a = od[0]; D.b1 = od[1]; D.i_b1 = od[2]; D.ss = od[3]; D.rr = od[4]; D.cross = od[5];
        D.cross1 = od[6]; D.cross2 = od[7]; D.ssy1 = od[8]; D.ssy2 = od[9]; D.ssh = od[10];
        D.aaa1 = od[11]; D.aaa2 = od[12]; D.mm = od[13];
        for (int m = 0; m < 4; ++m) { D.c[m] = od[14 + m]; D.t[m] = od[19 + m]; }
        D.tt = od[18];
        float y[NPVM];
#pragma unroll
        for (int v = 0; v < NPVM; ++v) y[v] = 0.0f;
        diag_solve_t<float>(c, D, pv, dv, acc, y);
        // dq in FP32 for the products: own part + correction; the correction kept for the
        // update, and (forward) dq* as the backward sweep's own part
        float dqf[NPVM];
        const long long gq = (long long)tile * NPVM * TILE_SLOTS + sl;
        float* ty = FWD ? d.tyf : d.tyb;
        float* own = d.trf + ((long long)tile * NTR + TR_X) * TILE_SLOTS + sl;
#pragma unroll
        for (int v = 0; v < NPVM; ++v) {
          if (v < npv) {
            dqf[v] = S32[(TR_X + v) * TILE_SLOTS + sl] + y[v];
            ty[gq + (long long)v * TILE_SLOTS] = y[v];
            if (FWD) own[v * TILE_SLOTS] = dqf[v];
          } else {
            dqf[v] = 0.0f;
          }
        }
        // outgoing contributions: A+ dq through the cell's + faces (forward), -A- dq through
        // its - faces (backward), each from zero so that the receiver adds them in order
        const float beta = D.rr - (D.b1 - 1.0f) * dv[6], evv = S32[TR_EVV * TILE_SLOTS + sl];
        auto contribution = [&](int dir, float* o) {
          float nx[3];
#pragma unroll
          for (int e = 0; e < 3; ++e) nx[e] = S32[(TR_COMMON + 3 * dir + e) * TILE_SLOTS + sl];
          const float spec = S32[(TR_COMMON + 9 + dir) * TILE_SLOTS + sl];
#pragma unroll
          for (int v = 0; v < NPVM; ++v) o[v] = 0.0f;
          jac_apply_pre<float>(npv, nx, pv, dv, spec, beta, evv, sgn, dqf, o);
        };
        contribution(0, ci);
        contribution(1, cj);
        contribution(2, ck);
        // contributions that leave the tile: into the entry block of the tile beyond
        if (pi == ni - 1 && nxt0 >= 0) {
          float* dst = d.tin + (long long)nxt0 * NPVM * TILE_IN + lj + TILE_J * lk;
          for (int v = 0; v < NPVM; ++v) dst[v * TILE_IN] = ci[v];
        }
        if (pj == nj - 1 && nxt1 >= 0) {
          float* dst = d.tin + (long long)nxt1 * NPVM * TILE_IN + TILE_IN_J + TILE_I * lk + li;
          for (int v = 0; v < NPVM; ++v) dst[v * TILE_IN] = cj[v];
        }
        if (pk == nk - 1 && nxt2 >= 0) {
          float* dst = d.tin + (long long)nxt2 * NPVM * TILE_IN + TILE_IN_K + TILE_I * lj + li;
          for (int v = 0; v < NPVM; ++v) dst[v * TILE_IN] = ck[v];
        }
      } else {
#pragma unroll
        for (int v = 0; v < NPVM; ++v) cj[v] = ck[v] = 0.0f;
      }
    }
    // ---- publish the tile's contributions and dq
    __syncwarp();
    if (lane == 0 && tile != withhold) {
      __threadfence();
      st_release(d.done + tile, 1);
    }
  }
}

// ------------------------------------------------------------------ update + residual
// stage > 0: one stage of the explicit schemes instead of the LU-SGS update --
// eulerex (src/update_module.f90:214-322), pv += getx_ex(res), or stage m of rk3rd
// (:324-453), pv = a1 rk + a2 pv + a3 getx_ex(res), rk being the state before the
// iteration (kept in dqs at t by stage 1).  The residual norms measure the change over
// the whole iteration (they are final after the last stage).
template <bool MX, bool EX = false>
__global__ void __launch_bounds__(128, 3) k_update(DevPtr d, Par c, int stage) {
  // grid-stride over the interior cells: the grid is a fixed multiple of the SM count,
  // so the per-CTA partials (and the order they are summed in) do not depend on size
  const int npv = c.npv;
  double sq_[NPVM];
  for (int v = 0; v < NPVM; ++v) sq_[v] = 0.0;
  double dpmax = -1.0;
  long long dpidx = -1;
  int bad = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < d.nint; t += stride) {
    int b = find_block_interior(d.blk, d.nblk, t), i, j, k;
    long long g = interior_cell(d.blk[b], t - d.blk[b].int_off, i, j, k);
    const long long n = d.ncell;
    double old[NPVM], p[NPVM];
    if constexpr (!EX) {
      // the sweep's dq: at the cell's tile slot (mixed form) or plane-major position
      const long long pq = d.pos[g];
#pragma unroll
      for (int v = 0; v < NPVM; ++v) {
        old[v] = p[v] = 0.0;
        if (v >= npv) continue;
        old[v] = d.pv[v * n + g];
        if (MX) {
          // dq = x0 + y_f + y_b in FP32: each part is an FP32 result of the FP32 operator, so
          // an FP64 sum would add digits none of them carries
          const long long q = tq_at(pq, v);
          const float dqf = (d.tq[q] + d.tyf[q]) + d.tyb[q];
          p[v] = old[v] + (double)dqf;
        } else {
          p[v] = old[v] + d.dqs[v * d.nint + pq];
        }
      }
    } else {
      double cur[NPVM], dvc[NDV], r[NPVM], x[NPVM];
      for (int v = 0; v < npv; ++v) { cur[v] = d.pv[v * n + g]; r[v] = d.res[v * n + g]; }
      for (int v = 0; v < NDV; ++v) dvc[v] = d.dv[v * n + g];
      if (c.rot) {
        // the explicit diagonal's enthalpy is the rothalpy (lhs%getenthalpy)
        double rc[3];
        for (int e = 0; e < 3; ++e) rc[e] = d.gm[(GM_GRD + 1 + e) * n + g];
        dvc[1] = dvc[1] - rot_q(c, rc);
      }
      getx_explicit(c, cur, dvc, r, d.dt[g], d.gm[GM_GRD * n + g], x);
      const double a1[3] = {0.0, 0.75, 1.0 / 3.0}, a2[3] = {1.0, 0.25, 2.0 / 3.0};
      const bool rk3 = c.timemethod == 2;
      const double c1 = rk3 ? a1[stage - 1] : 0.0, c2 = rk3 ? a2[stage - 1] : 1.0;
      for (int v = 0; v < npv; ++v) {
        double* rk = d.dqs + v * d.nint + t;
        if (stage == 1) *rk = cur[v];
        old[v] = *rk;
        p[v] = c1 * old[v] + c2 * cur[v] + c2 * x[v];   // a3 = a2 in both schemes
      }
    }
#pragma unroll
    for (int v = 0; v < NPVM; ++v)
      if (v < npv && !finite_bits(p[v])) bad = 1;   // checked before the clips, which would hide a NaN (fmax/fmin)
    p[0] = fmax(-c.pref + 1.0e1, p[0]);
    p[5] = fmin(1.0, fmax(0.0, p[5]));
    p[6] = fmin(1.0, fmax(0.0, p[6]));
    if (c.iturb >= -1) {
      p[7] = fmax(p[7], 1.0e-16);
      p[8] = fmax(fmax(p[8], 1.0e-16), d.ocut[g]);
    }
    // the state, its change norms and the largest |dp| before the EOS, so that only the EOS's
    // inputs stay live across it
#pragma unroll
    for (int v = 0; v < NPVM; ++v) {
      if (v >= npv) continue;
      d.pv[v * n + g] = p[v];
      double df = fabs(old[v] - p[v]);
      sq_[v] += df * df;   // (the clips keep a finite p finite)
    }
    double dp = fabs(old[0] - p[0]);
    if (dp > dpmax) { dpmax = dp; dpidx = t; }   // t increases: ties keep the first cell
    const double pe = p[0] + c.pref, te = p[4], y1 = p[5], y2 = p[6];
    double dv[NDV], tv[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int v = 0; v < 3; ++v)
      if (v < c.ntv) tv[v] = d.tv[v * n + g];
    if (MX) deteos_split(c.fluid, c.with_prop, pe, te, y1, y2, dv, tv, &d.sc->snd2_fallbacks);
    else deteos<false>(c.fluid, c.with_prop, pe, te, y1, y2, dv, tv, &d.sc->snd2_fallbacks);
    for (int v = 0; v < NDV; ++v) {
      d.dv[v * n + g] = dv[v];
      if (!finite_bits(dv[v])) bad = 1;
    }
#pragma unroll
    for (int v = 0; v < 3; ++v)
      if (v < c.ntv) d.tv[v * n + g] = tv[v];
  }
  if (bad) atomicExch(&d.sc->nonfinite, 1);
  // per-CTA partial sums (deterministic order: warp shuffles then warps in order)
  __shared__ double sh[4][NPVM + 2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < NPVM; ++v) {
    if (v >= npv) continue;
    double s = sq_[v];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sh[w][v] = s;
  }
  for (int o = 16; o > 0; o >>= 1) {
    double om = __shfl_down_sync(0xffffffffu, dpmax, o);
    long long oi = __shfl_down_sync(0xffffffffu, dpidx, o);
    if (om > dpmax || (om == dpmax && oi >= 0 && (dpidx < 0 || oi < dpidx))) { dpmax = om; dpidx = oi; }
  }
  if (lane == 0) { sh[w][NPVM] = dpmax; sh[w][NPVM + 1] = __longlong_as_double(dpidx); }
  __syncthreads();
  if (threadIdx.x == 0) {
    double* out = d.partial + (long long)blockIdx.x * (NPVM + 2);
    double m = -1.0;
    long long mi = -1;
    for (int v = 0; v < npv; ++v) {
      double s = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += sh[q][v];
      out[v] = s;
    }
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      double om = sh[q][NPVM];
      long long oi = __double_as_longlong(sh[q][NPVM + 1]);
      if (om > m || (om == m && oi >= 0 && (mi < 0 || oi < mi))) { m = om; mi = oi; }
    }
    out[NPVM] = m;
    out[NPVM + 1] = __longlong_as_double(mi);
  }
}

// MX: FP32, with the velocity gradients formed from u - U (exact differences), its casts of
// the neighbours' states on the integer pipes (to_f32, to_f64)
template <bool MX>
// if_changed: only when an upload changed some pv (the eddy viscosity is a function of the
// cell's and its neighbours' pv)
__global__ void k_eddy(DevPtr d, Par c, long long t0, long long t1, int if_changed = 0) {
  if (if_changed && !*(volatile int*)&d.sc->pv_changed) return;
  long long t = t0 + blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= t1) return;
  int b = find_block_interior(d.blk, d.nblk, t), i, j, k;
  const BlockGeom& B = d.blk[b];
  long long g = interior_cell(B, t - B.int_off, i, j, k);
  const long long n = d.ncell, sj = B.ni, sk = (long long)B.ni * B.nj;
  if (c.iturb == -1) {
    d.tv[2 * n + g] = ke_eddy(d.dv[g], d.pv[7 * n + g], d.pv[8 * n + g], d.tv[g], d.gm[(GM_GRD + 4) * n + g]);
    return;
  }
  const long long nbr[6] = {g - 1, g + 1, g - sj, g + sj, g - sk, g + sk};
  double fa[6][3];
  for (int q = 0; q < 3; ++q) {
    fa[0][q] = d.gm[(GM_CX + q) * n + g - 1]; fa[1][q] = d.gm[(GM_CX + q) * n + g];
    fa[2][q] = d.gm[(GM_EX + q) * n + g - sj]; fa[3][q] = d.gm[(GM_EX + q) * n + g];
    fa[4][q] = d.gm[(GM_TX + q) * n + g - sk]; fa[5][q] = d.gm[(GM_TX + q) * n + g];
  }
  if (MX) {
    const float* G = d.gmf;
    float fa[6][3];
    for (int q = 0; q < 3; ++q) {
      fa[0][q] = G[(GM_CX + q) * n + g - 1]; fa[1][q] = G[(GM_CX + q) * n + g];
      fa[2][q] = G[(GM_EX + q) * n + g - sj]; fa[3][q] = G[(GM_EX + q) * n + g];
      fa[4][q] = G[(GM_TX + q) * n + g - sk]; fa[5][q] = G[(GM_TX + q) * n + g];
    }
    const float ivol = 1.0f / G[GM_GRD * n + g];
    float gr[3][3];
    for (int q = 0; q < 3; ++q) {
      const double* P = d.pv + (1 + q) * n;
      const double U = c.uref_vec[q];
      const float c0 = to_f32(P[g] - U);
      float vv[6];
      for (int m = 0; m < 6; ++m) vv[m] = 0.5f * (to_f32(P[nbr[m]] - U) + c0);
      for (int e = 0; e < 3; ++e)
        gr[q][e] = (vv[1] * fa[1][e] + vv[3] * fa[3][e] + vv[5] * fa[5][e] - vv[0] * fa[0][e] - vv[2] * fa[2][e] - vv[4] * fa[4][e]) * ivol;
    }
    const float kk = to_f32(d.pv[7 * n + g]), oo = to_f32(d.pv[8 * n + g]), rho = to_f32(d.dv[g]), mu = to_f32(d.tv[g]);
    const float y5 = G[(GM_GRD + 4) * n + g];
    const float term1 = sqrtf(kk) / (0.09f * oo * y5);
    const float term2 = 500.0f * mu / rho / (oo * y5 * y5);
    const float arg2 = fmaxf(2.0f * term1, term2);
    const float bigf2 = tanhf(arg2 * arg2);
    const float sij = gr[0][0] * gr[0][0] + gr[1][1] * gr[1][1] + gr[2][2] * gr[2][2] +
                      0.5f * (sq(gr[0][1] + gr[1][0]) + sq(gr[0][2] + gr[2][0]) + sq(gr[1][2] + gr[2][1]));
    const float sss = sqrtf(2.0f * sij);
    d.tv[2 * n + g] = to_f64(0.31f * rho * kk / fmaxf(0.31f * oo, sss * bigf2));
    return;
  }
  double vol = d.gm[GM_GRD * n + g], ivol = 1.0 / vol;
  double gr[3][3];
  for (int q = 0; q < 3; ++q) {
    const double* P = d.pv + (1 + q) * n;
    double c0 = P[g];
    double v1 = 0.5 * (P[nbr[0]] + c0), v2 = 0.5 * (P[nbr[1]] + c0), v3 = 0.5 * (P[nbr[2]] + c0);
    double v4 = 0.5 * (P[nbr[3]] + c0), v5 = 0.5 * (P[nbr[4]] + c0), v6 = 0.5 * (P[nbr[5]] + c0);
    for (int e = 0; e < 3; ++e)
      gr[q][e] = (v2 * fa[1][e] + v4 * fa[3][e] + v6 * fa[5][e] - v1 * fa[0][e] - v3 * fa[2][e] - v5 * fa[4][e]) * ivol;
  }
  double kk = d.pv[7 * n + g], oo = d.pv[8 * n + g], rho = d.dv[g], mu = d.tv[g];
  double y5 = d.gm[(GM_GRD + 4) * n + g];
  double term1 = sqrt(kk) / (0.09 * oo * y5);
  double term2 = 500.0 * mu / rho / (oo * y5 * y5);
  double arg2 = fmax(2.0 * term1, term2);
  double bigf2 = tanh(arg2 * arg2);
  double sij = gr[0][0] * gr[0][0] + gr[1][1] * gr[1][1] + gr[2][2] * gr[2][2] +
               0.5 * (sq(gr[0][1] + gr[1][0]) + sq(gr[0][2] + gr[2][0]) + sq(gr[1][2] + gr[2][1]));
  double sss = sqrt(2.0 * sij);
  d.tv[2 * n + g] = 0.31 * rho * kk / fmax(0.31 * oo, sss * bigf2);
}

// final reduction of the per-CTA partials: 256 threads, fixed assignment and a fixed
// tree, so the norms are bitwise reproducible from run to run
constexpr int FIN_T = 256;
__global__ void __launch_bounds__(FIN_T) k_finish(DevPtr d, Par c, int nparts) {
  __shared__ double s[FIN_T][NPVM];
  __shared__ double sm[FIN_T];
  __shared__ long long si[FIN_T];
  const int npv = c.npv, tid = threadIdx.x;
  double acc[NPVM];
  for (int v = 0; v < NPVM; ++v) acc[v] = 0.0;
  double m = -1.0;
  long long mi = -1;
  for (int q = tid; q < nparts; q += FIN_T) {
    const double* pp = d.partial + (long long)q * (NPVM + 2);
    for (int v = 0; v < npv; ++v) acc[v] += pp[v];
    double om = pp[NPVM];
    long long oi = __double_as_longlong(pp[NPVM + 1]);
    if (om > m || (om == m && oi >= 0 && (mi < 0 || oi < mi))) { m = om; mi = oi; }
  }
  for (int v = 0; v < NPVM; ++v) s[tid][v] = acc[v];
  sm[tid] = m;
  si[tid] = mi;
  __syncthreads();
  for (int h = FIN_T / 2; h > 0; h >>= 1) {
    if (tid < h) {
      for (int v = 0; v < npv; ++v) s[tid][v] += s[tid + h][v];
      double om = sm[tid + h];
      long long oi = si[tid + h];
      if (om > sm[tid] || (om == sm[tid] && oi >= 0 && (si[tid] < 0 || oi < si[tid]))) { sm[tid] = om; si[tid] = oi; }
    }
    __syncthreads();
  }
  if (tid == 0) {
    Scalars* sc = d.sc;
    for (int v = 0; v < npv; ++v) sc->res[v] = sqrt(s[0][v]);
    sc->resmax = sm[0];
    sc->resmax_cell = (sm[0] > 1.0e-12) ? si[0] : -1;
    sc->time_acc += __longlong_as_double((long long)sc->dtmin_bits);
    sc->dtmin_bits = (unsigned long long)__double_as_longlong(1.0e10);
  }
}

// ------------------------------------------------------------------ layout conversion
// Fortran AoS a(nv, -1:imax+3, ...) of one block <-> SoA planes
__global__ void k_aos_to_soa(const double* __restrict__ a, int nv, long long ncb, double* __restrict__ soa,
                             long long ncell, long long off) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= ncb) return;
  for (int v = 0; v < nv; ++v) soa[v * ncell + off + q] = a[q * nv + v];
}
__global__ void k_soa_to_aos(const double* __restrict__ soa, int nv, long long ncb, double* __restrict__ a,
                             long long ncell, long long off) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= ncb) return;
  for (int v = 0; v < nv; ++v) a[q * nv + v] = soa[v * ncell + off + q];
}
// interior AoS a(nv, 2:imax, 2:jmax, 2:kmax) of one block <-> SoA planes
__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, long long m) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < m) b[q] = (float)a[q];
}
__global__ void k_lo_f32(const double* __restrict__ a, const float* __restrict__ hi, float* __restrict__ lo,
                         long long m) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < m) lo[q] = (float)(a[q] - (double)hi[q]);
}

__global__ void k_interior_io(double* __restrict__ a, int nv, BlockGeom B, double* __restrict__ soa, long long ncell,
                              int to_soa) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
  if (q >= nint) return;
  int i, j, k;
  long long g = interior_cell(B, q, i, j, k);
  for (int v = 0; v < nv; ++v) {
    if (to_soa) soa[v * ncell + g] = a[q * nv + v];
    else a[q * nv + v] = soa[v * ncell + g];
  }
}

}  // namespace cfd

// =====================================================================================
//                                     C ABI
// =====================================================================================
using namespace cfd;

struct cfd3d_handle {
  Engine E;
  double* staging = nullptr;
  size_t staging_bytes = 0;
  std::vector<cudaEvent_t> bev;   // one per block: the whole-case transfers' per-block stages
  // the copy stream of upload_state / download_state and one event per staged array:
  // the layout kernel of one array overlaps the host copy of the next
  cudaStream_t cp = nullptr;
  cudaEvent_t ev[6] = {};
};

namespace {

inline unsigned nblk_of(long long n, int T) { return (unsigned)((n + T - 1) / T); }

int ensure_staging(cfd3d_handle* h, size_t bytes) {
  Engine& E = h->E;
  if (h->staging_bytes >= bytes) return CFD3D_OK;
  cudaFree(h->staging);
  h->staging = nullptr;
  h->staging_bytes = 0;
  CFD_CUDA(cudaMalloc(&h->staging, bytes));
  h->staging_bytes = bytes;
  return CFD3D_OK;
}

int ensure_copy_stream(cfd3d_handle* h) {
  Engine& E = h->E;
  if (h->cp) return CFD3D_OK;
  for (auto& e : h->ev) CFD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CFD_CUDA(cudaStreamCreateWithFlags(&h->cp, cudaStreamNonBlocking));
  return CFD3D_OK;
}

// polls of a neighbour's done flag before a dataflow sweep gives up (about 0.1-0.5 s)
constexpr long long SWEEP_SPIN = 1ll << 22;

// k_rhs in the instantiation of the form (mixed / FP64), the time integrator (sweep records
// for LU-SGS) and the extended sources (DES length scale, gravity)
// (over the interior cells of blocks [b0, b1))
template <bool REC>
void launch_rhs_rec(const Engine& E, cudaStream_t s, int T, int b0, int b1, int store_res) {
  const Par& c = E.par;
  const int nb = (int)E.blk.size();
  const long long t0 = E.blk[b0].int_off, t1 = (b1 < nb) ? E.blk[b1].int_off : E.nint;
  const unsigned g = nblk_of(std::max<long long>(t1 - t0, 1), T);
  const bool xs = (c.iturb == 0 && c.ides != 0) || c.gravity != 0 || c.csf != 0 || c.rot != 0;
  if (c.mixed) {
    if (xs) k_rhs<true, REC, true><<<g, T, 0, s>>>(E.d, c, t0, t1, store_res);
    else k_rhs<true, REC, false><<<g, T, 0, s>>>(E.d, c, t0, t1, store_res);
  } else {
    if (xs) k_rhs<false, REC, true><<<g, T, 0, s>>>(E.d, c, t0, t1, store_res);
    else k_rhs<false, REC, false><<<g, T, 0, s>>>(E.d, c, t0, t1, store_res);
  }
}
void launch_rhs(const Engine& E, cudaStream_t s, int T, bool rec, bool store_res, int b0 = 0, int b1 = -1) {
  if (b1 < 0) b1 = (int)E.blk.size();
  if (rec) launch_rhs_rec<true>(E, s, T, b0, b1, store_res ? 1 : 0);
  else launch_rhs_rec<false>(E, s, T, b0, b1, store_res ? 1 : 0);
}

// The face stage and the residual of one pseudo-iteration.  The mixed form with more than
// one group pipelines them over groups of consecutive blocks: the residual of group q runs on
// st2 beside the face stage of group q + 1 on s (the face kernels keep the FP32 pipes busy,
// the residual the FP64 pipe; a block's faces and residual touch only its own padded cells,
// faces and tiles).  st2 forks from s and joins it again, so the stage is one unit of s.
void launch_face_rhs(const Engine& E, cudaStream_t s, bool rec, bool store_res) {
  const Par& c = E.par;
  const int nb = (int)E.blk.size();
  const int ng = std::min(std::max(E.pipe_groups, 1), std::min(nb, Engine::MAX_PIPE));
  if (!c.mixed) {
    launch_face_flux(E, s);
    launch_rhs(E, s, E.tpb_rhs, rec, store_res);
    return;
  }
  if (ng <= 1) {
    launch_face_flux_mixed(E, s, 0, nb);
    launch_rhs(E, s, E.tpb_rhs, rec, store_res);
    return;
  }
  cudaEventRecord(E.pipe_ev[0], s);
  cudaStreamWaitEvent(E.st2, E.pipe_ev[0], 0);
  for (int q = 0; q < ng; ++q) {
    const int b0 = (int)((long long)nb * q / ng), b1 = (int)((long long)nb * (q + 1) / ng);
    launch_face_flux_mixed(E, s, b0, b1);
    cudaEventRecord(E.pipe_ev[1 + q], s);
    cudaStreamWaitEvent(E.st2, E.pipe_ev[1 + q], 0);
    launch_rhs(E, E.st2, E.tpb_rhs, rec, store_res, b0, b1);
  }
  cudaEventRecord(E.pipe_ev[Engine::MAX_PIPE + 1], E.st2);
  cudaStreamWaitEvent(s, E.pipe_ev[Engine::MAX_PIPE + 1], 0);
}

// launches of the face fluxes and the residual: the FP64 form's three face kernels, or the
// mixed form's shadow, its reconstruction and flux kernels of each direction (with the j and
// k faces' column reconstruction under MUSCL), and k_rhs
int face_rhs_launches(const Engine& E) {
  const Par& c = E.par;
  if (!c.mixed) return 4;
  const int nb = (int)E.blk.size();
  const int ng = std::min(std::max(E.pipe_groups, 1), std::min(nb, Engine::MAX_PIPE));
  return ng * (8 + (c.nmuscl > 0 ? 2 : 0) + (c.iturb != -3 ? 3 : 0));
}

// The boundary program -- the total-pressure pools, then faces + halos, edges, corners -- and,
// with the surface-tension source, calvfg and setbc_vfg after it, as timeinteg calls them
// (src/update_module.f90:240-243, 359-362, 479-482).  Returns the number of launches.
int launch_boundary(const Engine& E, cudaStream_t s) {
  const DevPtr& d = E.d;
  const Par& c = E.par;
  int n = 0;
  if (d.ntp) { k_totalp<<<d.ntp, 128, 0, s>>>(d, c); ++n; }
  for (int p = 0; p < 3; ++p)
    if (E.nops[p]) { k_ghost<<<nblk_of(E.nops[p], 128), 128, 0, s>>>(d, c, E.d_ops[p], E.nops[p]); ++n; }
  if (c.csf) {
    k_vf<<<nblk_of(E.ncell, 256), 256, 0, s>>>(d);
    k_vfg<<<nblk_of(E.ncell, 256), 256, 0, s>>>(d);
    n += 2;
    if (d.nvfg_halo) { k_vfg_halo<<<nblk_of(d.nvfg_halo, 256), 256, 0, s>>>(d); ++n; }
  }
  return n;
}

// the launch sequence of one iteration (captured into the graph); `mark` (optional)
// records an event after each stage for the stage profile
void launch_iteration(Engine& E, bool full, cudaEvent_t* mark = nullptr) {
  const DevPtr& d = E.d;
  const Par& c = E.par;
  cudaStream_t s = E.st;
  const int T = 128;
  int n = 0;
  auto stage = [&](int q) { if (mark) cudaEventRecord(mark[q], s); };
  stage(0);
  if (full) {
    if (c.mixed) k_timestep<true><<<nblk_of(E.nint, 256), 256, 0, s>>>(d, c);
    else k_timestep<false><<<nblk_of(E.nint, 256), 256, 0, s>>>(d, c);
    ++n;
  }
  stage(1);
  n += launch_boundary(E, s);
  stage(2);
  // (the residual planes are written when the residual is queried: full = false)
  if (c.mixed && E.pipe_groups > 1) {
    // pipelined: the stage's end only (its face and residual parts overlap)
    launch_face_rhs(E, s, c.timemethod == 3, !full);
    stage(3);
  } else {
    if (c.mixed) launch_face_flux_mixed(E, s, 0, (int)E.blk.size());
    else launch_face_flux(E, s);
    stage(3);
    launch_rhs(E, s, E.tpb_rhs, c.timemethod == 3, !full);
  }
  stage(4);
  n += face_rhs_launches(E);
  if (!full) { E.launches_per_iter = n; return; }
  if (c.timemethod != 3) {
    // explicit Euler (one stage) or RK3 (three; the time step is taken at the first only):
    // each stage is boundary program, fluxes, residual, update and eddy viscosity
    const int nstage = (c.timemethod == 2) ? 3 : 1;
    for (int m = 1; m <= nstage; ++m) {
      if (m > 1) {
        n += launch_boundary(E, s);
        launch_face_rhs(E, s, false, true);
        n += face_rhs_launches(E);
      }
      if (m == nstage) { stage(5); stage(6); }
      if (c.mixed) k_update<true, true><<<E.red_grid, T, 0, s>>>(d, c, m);
      else k_update<false, true><<<E.red_grid, T, 0, s>>>(d, c, m);
      ++n;
      if (m == nstage) stage(7);
      if (c.iturb >= -1) {
        if (c.mixed) k_eddy<true><<<nblk_of(E.nint, T), T, 0, s>>>(d, c, 0, E.nint);
        else k_eddy<false><<<nblk_of(E.nint, T), T, 0, s>>>(d, c, 0, E.nint);
        ++n;
      }
    }
    k_finish<<<1, FIN_T, 0, s>>>(d, c, E.red_grid);
    ++n;
    stage(8);
    E.launches_per_iter = n;
    return;
  }
  if (c.mixed) {
    // tile sweeps: flags and tickets cleared, one persistent launch per sweep
    cudaMemsetAsync(d.tickets, 0, 2 * sizeof(unsigned), s);
    cudaMemsetAsync(d.done, 0, (size_t)d.ntile * sizeof(int), s);
    k_sweep_tile<true><<<E.sweep_grid, 32, TILE_SMEM, s>>>(d, c, SWEEP_SPIN, -1);
    stage(5);
    cudaMemsetAsync(d.done, 0, (size_t)d.ntile * sizeof(int), s);
    k_sweep_tile<false><<<E.sweep_grid, 32, TILE_SMEM, s>>>(d, c, SWEEP_SPIN, -1);
    n += 2;
  } else if (!E.sweep_planes) {
    // dataflow sweeps: flags and tickets cleared, one persistent launch per sweep
    cudaMemsetAsync(d.tickets, 0, 2 * sizeof(unsigned), s);
    cudaMemsetAsync(d.done, 0, (size_t)d.nchunk * sizeof(int), s);
    k_sweep_df<true><<<E.sweep_grid, SW_CH, 0, s>>>(d, c, SWEEP_SPIN, -1);
    stage(5);
    cudaMemsetAsync(d.done, 0, (size_t)d.nchunk * sizeof(int), s);
    k_sweep_df<false><<<E.sweep_grid, SW_CH, 0, s>>>(d, c, SWEEP_SPIN, -1);
    n += 2;
  } else {
    const int np = (int)E.plane_off.size() - 1;
    const int TS = 64;
    for (int q = 0; q < np; ++q) {
      long long a = E.plane_off[q], b = E.plane_off[q + 1];
      if (b > a) { k_sweep<true><<<nblk_of(b - a, TS), TS, 0, s>>>(d, c, a, b); ++n; }
    }
    stage(5);
    for (int q = np - 1; q >= 0; --q) {
      long long a = E.plane_off[q], b = E.plane_off[q + 1];
      if (b > a) { k_sweep<false><<<nblk_of(b - a, TS), TS, 0, s>>>(d, c, a, b); ++n; }
    }
  }
  stage(6);
  if (c.mixed) k_update<true><<<E.red_grid, T, 0, s>>>(d, c, 0);
  else k_update<false><<<E.red_grid, T, 0, s>>>(d, c, 0);
  ++n;
  stage(7);
  if (c.iturb >= -1) {
    if (c.mixed) k_eddy<true><<<nblk_of(E.nint, T), T, 0, s>>>(d, c, 0, E.nint);
    else k_eddy<false><<<nblk_of(E.nint, T), T, 0, s>>>(d, c, 0, E.nint);
    ++n;
  }
  k_finish<<<1, FIN_T, 0, s>>>(d, c, E.red_grid);
  ++n;
  stage(8);
  E.launches_per_iter = n;
}

int build_graph(Engine& E) {
  if (E.graph_ready) return CFD3D_OK;
  cudaGraph_t g;
  CFD_CUDA(cudaStreamBeginCapture(E.st, cudaStreamCaptureModeThreadLocal));
  launch_iteration(E, true);
  CFD_CUDA(cudaStreamEndCapture(E.st, &g));
  CFD_CUDA(cudaGraphInstantiate(&E.graph, g, 0));
  cudaGraphDestroy(g);
  E.graph_ready = 1;
  return CFD3D_OK;
}

int read_scalars(Engine& E, Scalars& s) {
  CFD_CUDA(cudaMemcpyAsync(&s, E.d.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, E.st));
  CFD_CUDA(cudaStreamSynchronize(E.st));
  return CFD3D_OK;
}

bool make_par(const cfd3d_config* in, Par& c, std::string& err) {
  std::memset(&c, 0, sizeof(c));
  if (in->timemethod < 1 || in->timemethod > 3) {
    err = "timemethod must be 1 (explicit Euler), 2 (RK3) or 3 (LU-SGS)"; return false;
  }
  c.timemethod = in->timemethod;
  if (in->iturb == -3) { c.npv = 7; c.ntv = 0; }
  else if (in->iturb == -2) { c.npv = 7; c.ntv = 2; }
  else if (in->iturb == 0 || in->iturb == -1) { c.npv = 9; c.ntv = 3; }
  else { err = "iturb must be -3, -2, -1 or 0"; return false; }
  if (in->iturb == 0 && (in->ides < 0 || in->ides > 4)) { err = "ides must be 0..4"; return false; }
  c.ides = (in->iturb == 0) ? in->ides : 0;
  const int gr = in->gravity;
  if (!(gr == 0 || gr == 4 || (gr >= -3 && gr <= 3))) { err = "gravity must be 0, +-1, +-2, +-3 or 4"; return false; }
  if (gr == 4) {
    if (in->ngravity < 1 || !in->gravity_data) { err = "gravity = 4 without its history"; return false; }
    for (int m = 1; m < in->ngravity; ++m)
      if (!(in->gravity_data[4 * m] > in->gravity_data[4 * (m - 1)])) { err = "gravity history times must increase"; return false; }
  }
  c.gravity = gr;
  if (in->fluid != 1 && in->fluid != 2) { err = "fluid must be 1 (stiffened) or 2 (IAPWS-97)"; return false; }
  if (in->ngas != 1) { err = "ngas must be 1 (ideal gas)"; return false; }
  if (in->nscheme < 1 || in->nscheme > 4 || in->nmuscl < 0 || in->nmuscl > 2 || in->nlim < 0 || in->nlim > 10) {
    err = "nscheme/nmuscl/nlim out of range"; return false;
  }
  if (in->ncav < 0 || in->ncav > 5) { err = "ncav out of range"; return false; }
  if (in->local < -1 || in->local > 1) { err = "local out of range"; return false; }
  if (in->prec < 0 || in->prec > 2) { err = "prec out of range"; return false; }
  if (in->csf != 0 && in->csf != 1) { err = "csf must be 0 or 1"; return false; }
  c.csf = in->csf;
  // rotation, rpm: omega along +-x, +-y, +-z (src/config_module.f90:126-141)
  if (in->rotation < -3 || in->rotation > 3) { err = "rotation must be 0, +-1, +-2 or +-3"; return false; }
  if (in->rotation != 0 && in->precision == CFD3D_MIXED) { err = "the rotating frame runs in the FP64 form"; return false; }
  c.rot = in->rotation != 0;
  if (c.rot)
    c.omega[std::abs(in->rotation) - 1] = (in->rotation > 0 ? 1.0 : -1.0) * in->rpm * 2.0 * (std::atan(1.0) * 4.0) / 60.0;
  if (in->nsteady >= 1 && !(in->dt_phy > 0.0)) { err = "dual time stepping needs dt_phy > 0"; return false; }
  if (in->precision != CFD3D_FP64 && in->precision != CFD3D_MIXED) { err = "precision must be CFD3D_FP64 or CFD3D_MIXED"; return false; }
  c.mixed = (in->precision == CFD3D_MIXED);
  c.nqq = in->nsteady >= 1 ? 2 : 0;
  c.ngrd = (in->iturb >= -1) ? 5 : 4;
  c.nsteady = in->nsteady; c.iturb = in->iturb; c.nscheme = in->nscheme; c.nmuscl = in->nmuscl; c.nlim = in->nlim;
  c.local = in->local; c.prec = in->prec; c.fluid = in->fluid; c.ncav = in->ncav; c.fix_cav_clamp = in->fix_cav_clamp;
  c.with_prop = (in->iturb != -3);
  c.dt_phy = in->dt_phy; c.cfl = in->cfl; c.c_v = in->c_v; c.c_c = in->c_c; c.pref = in->pref; c.uref = in->uref;
  const double pi = std::atan(1.0) * 4.0;
  c.str = in->l_character / pi / in->dt_phy;
  c.l_chord = in->l_chord;
  double aoa = in->aoa * pi / 180.0, aos = in->aos * pi / 180.0;
  c.uref_vec[0] = in->uref * std::cos(aos) * std::cos(aoa);
  c.uref_vec[1] = in->uref * std::cos(aos) * std::sin(aoa);
  c.uref_vec[2] = in->uref * std::sin(aos);
  c.tref = in->tref; c.y1ref = in->y1ref; c.y2ref = in->y2ref;
  return true;
}

}  // namespace

namespace {
// ms per call of `fn` (launches on the engine's stream): one untimed call, then `reps`
// timed between CUDA events
// The integer-pipe conversions (to_f32, to_f64) against the hardware's, bit for bit, on
// seeded bit patterns: random ones over the whole double range, exact halfway cases, the
// ends of the float range (overflow to infinity, subnormal results), signed zeros, and
// values of ordinary magnitude
__global__ void k_convert_check(long long n, unsigned long long seed, unsigned long long* bad) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  unsigned long long z = seed + (unsigned long long)t * 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  unsigned long long bits = z;
  const unsigned long long sm = 0x800fffffffffffffull;   // sign and significand
  switch ((int)(t % 6)) {
    case 1: bits = (z & 0x800fffffe0000000ull) | 0x10000000ull | ((unsigned long long)(993 + (int)(z % 60)) << 52); break;
    case 2: bits = (z & sm) | (1150ull << 52); break;
    case 3: bits = (z & sm) | ((unsigned long long)(897 - (int)(z % 30)) << 52); break;
    case 4: bits = z & 0x8000000000000000ull; break;
    case 5: bits = (z & sm) | ((unsigned long long)(1003 + (int)(z % 40)) << 52); break;
    default: break;
  }
  const double x = __longlong_as_double((long long)bits);
  const float a = __double2float_rn(x), b = to_f32(x);
  if (__float_as_uint(a) != __float_as_uint(b)) atomicAdd(bad, 1ull);
  const double c = (double)a, e = to_f64(a);
  if (__double_as_longlong(c) != __double_as_longlong(e)) atomicAdd(bad + 1, 1ull);
}

template <class F>
float time_calls(Engine& E, int reps, F fn) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fn();
  cudaEventRecord(a, E.st);
  for (int r = 0; r < reps; ++r) fn();
  cudaEventRecord(b, E.st);
  cudaEventSynchronize(b);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / (float)std::max(reps, 1);
}
}  // namespace

extern "C" {

const char* cfd3d_last_error(const cfd3d_handle* h) { return h ? h->E.err.c_str() : "null handle"; }

int cfd3d_eos_eval(int fluid, int ngas, int with_prop, int64_t n, const double* p, const double* t, const double* y1,
                   const double* y2, double* dv, double* tv) {
  if (n <= 0 || !p || !t || !y1 || !y2 || !dv || (fluid != 1 && fluid != 2) || ngas != 1) return CFD3D_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CFD3D_ERR_NODEVICE;
  double *dp = nullptr, *dt = nullptr, *dy1 = nullptr, *dy2 = nullptr, *ddv = nullptr, *dtv = nullptr;
  unsigned long long* fb = nullptr;
  size_t b = (size_t)n * 8;
  int rc = CFD3D_OK;
  if (cudaMalloc(&dp, b) || cudaMalloc(&dt, b) || cudaMalloc(&dy1, b) || cudaMalloc(&dy2, b) ||
      cudaMalloc(&ddv, b * NDV) || cudaMalloc(&dtv, b * 2) || cudaMalloc(&fb, 8)) {
    rc = CFD3D_ERR_NOMEM;
  } else {
    cudaMemcpy(dp, p, b, cudaMemcpyHostToDevice);
    cudaMemcpy(dt, t, b, cudaMemcpyHostToDevice);
    cudaMemcpy(dy1, y1, b, cudaMemcpyHostToDevice);
    cudaMemcpy(dy2, y2, b, cudaMemcpyHostToDevice);
    cudaMemset(fb, 0, 8);
    k_eos_points<<<(unsigned)((n + 127) / 128), 128>>>(fluid, with_prop, n, dp, dt, dy1, dy2, ddv, dtv, fb);
    if (cudaMemcpy(dv, ddv, b * NDV, cudaMemcpyDeviceToHost) != cudaSuccess) rc = CFD3D_ERR_CUDA;
    if (tv && with_prop && cudaMemcpy(tv, dtv, b * 2, cudaMemcpyDeviceToHost) != cudaSuccess) rc = CFD3D_ERR_CUDA;
  }
  cudaFree(dp); cudaFree(dt); cudaFree(dy1); cudaFree(dy2); cudaFree(ddv); cudaFree(dtv); cudaFree(fb);
  return rc;
}

// ---- pointwise EOS through a static device buffer (no allocation)
namespace {
struct EosScratch {
  double p[CFD3D_EOS_NOALLOC_MAX], t[CFD3D_EOS_NOALLOC_MAX], y1[CFD3D_EOS_NOALLOC_MAX], y2[CFD3D_EOS_NOALLOC_MAX];
  double dv[NDV * CFD3D_EOS_NOALLOC_MAX], tv[2 * CFD3D_EOS_NOALLOC_MAX];
  unsigned long long fallbacks;   // must start at zero: the kernel counts into it
};
// The buffer's device address per CUDA context.  A context has its own copy of every
// module's globals, and a context that ends (cudaDeviceReset, a primary context released
// and made again) takes the copy with it, so the cache is keyed on the context's unique id
// (cuCtxGetId; ids are never reused within a process), not on the device index.
struct ScratchSlot { unsigned long long ctx; EosScratch* ptr; };
std::mutex g_eos_scratch_mu;
std::vector<ScratchSlot> g_eos_scratch_slots;

// the current context's id, through the runtime's driver entry points (no link against
// the driver library); 0 when no context is current
using FnCtxGetCurrent = CUresult (*)(CUcontext*);
using FnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);
bool current_ctx_id(unsigned long long& id) {
  static FnCtxGetCurrent get_cur = nullptr;
  static FnCtxGetId get_id = nullptr;
  if (!get_cur || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, nullptr) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, nullptr) != cudaSuccess ||
        !f1 || !f2)
      return false;
    get_cur = reinterpret_cast<FnCtxGetCurrent>(f1);
    get_id = reinterpret_cast<FnCtxGetId>(f2);
  }
  CUcontext ctx = nullptr;
  if (get_cur(&ctx) != CUDA_SUCCESS) return false;
  id = 0;
  return !ctx || get_id(ctx, &id) == CUDA_SUCCESS;
}
}  // namespace
static __device__ __align__(256) EosScratch g_eos_scratch;

int cfd3d_eos_eval_noalloc(int fluid, int ngas, int with_prop, int64_t n, const double* p, const double* t,
                           const double* y1, const double* y2, double* dv, double* tv) {
  if (n <= 0 || n > CFD3D_EOS_NOALLOC_MAX || !p || !t || !y1 || !y2 || !dv || (fluid != 1 && fluid != 2) ||
      ngas != 1)
    return CFD3D_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CFD3D_ERR_NODEVICE;
  EosScratch* S = nullptr;
  {
    // set-up on the first call in a context: the buffer's device address there
    std::lock_guard<std::mutex> lock(g_eos_scratch_mu);
    unsigned long long ctx = 0;
    if (!current_ctx_id(ctx)) return CFD3D_ERR_CUDA;
    for (const ScratchSlot& sl : g_eos_scratch_slots)
      if (ctx && sl.ctx == ctx) S = sl.ptr;
    if (!S) {
      // (with no context current yet, the lookup makes the device's primary context current)
      void* ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_eos_scratch) != cudaSuccess || !ptr) return CFD3D_ERR_CUDA;
      if (!ctx && (!current_ctx_id(ctx) || !ctx)) return CFD3D_ERR_CUDA;
      S = static_cast<EosScratch*>(ptr);
      g_eos_scratch_slots.push_back({ctx, S});
    }
  }
  const size_t b = (size_t)n * 8;
  if (cudaMemcpy(S->p, p, b, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(S->t, t, b, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(S->y1, y1, b, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(S->y2, y2, b, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(&S->fallbacks, 0, sizeof(unsigned long long)) != cudaSuccess)
    return CFD3D_ERR_CUDA;
  k_eos_points<<<(unsigned)((n + 127) / 128), 128>>>(fluid, with_prop, n, S->p, S->t, S->y1, S->y2, S->dv, S->tv,
                                                      &S->fallbacks);
  if (cudaGetLastError() != cudaSuccess) return CFD3D_ERR_CUDA;
  if (cudaMemcpy(dv, S->dv, b * NDV, cudaMemcpyDeviceToHost) != cudaSuccess) return CFD3D_ERR_CUDA;
  if (tv && with_prop && cudaMemcpy(tv, S->tv, b * 2, cudaMemcpyDeviceToHost) != cudaSuccess) return CFD3D_ERR_CUDA;
  return CFD3D_OK;
}

int cfd3d_create(const cfd3d_config* cfg, int nblocks, const cfd3d_block_desc* blocks, cfd3d_handle** out) {
  if (!out) return CFD3D_ERR_ARG;
  *out = nullptr;
  cfd3d_handle* h = new (std::nothrow) cfd3d_handle();
  if (!h) return CFD3D_ERR_NOMEM;
  *out = h;
  Engine& E = h->E;
  if (!cfg || nblocks < 1 || nblocks > MAXBLK || !blocks) { E.err = "bad arguments"; return CFD3D_ERR_ARG; }
  E.cfg = *cfg;
  if (!make_par(cfg, E.par, E.err)) return CFD3D_ERR_ARG;
  // descriptor checks that need no device: they fail the same way on a CPU-only host
  for (int b = 0; b < nblocks; ++b) {
    const cfd3d_block_desc& d = blocks[b];
    if (d.imax < 4 || d.jmax < 4 || d.kmax < 4 || !d.xyz) { E.err = "block too small or no coordinates"; return CFD3D_ERR_DESCRIPTOR; }
    if (d.nbc < 0 || (d.nbc > 0 && !d.bc) || d.ncon < 0 || (d.ncon > 0 && !d.con)) {
      E.err = "bad bc or connection list"; return CFD3D_ERR_DESCRIPTOR;
    }
    for (int q = 0; q < d.nbc; ++q) {
      const int* p = d.bc[q].pnts;
      int nmax[3] = {d.imax, d.jmax, d.kmax}, faces = 0;
      for (int a = 0; a < 3; ++a)
        if (p[a] == p[3 + a] && (p[a] == 1 || p[a] == nmax[a])) ++faces;
      if (faces != 1) { E.err = "bc patch is not a block face"; return CFD3D_ERR_DESCRIPTOR; }
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { E.err = "no CUDA device"; return CFD3D_ERR_NODEVICE; }
  // block layout
  long long off = 0, ioff = 0, foff[3] = {0, 0, 0}, coff[3] = {0, 0, 0};
  for (int b = 0; b < nblocks; ++b) {
    const cfd3d_block_desc& d = blocks[b];
    if (d.imax < 4 || d.jmax < 4 || d.kmax < 4 || !d.xyz) { E.err = "block too small or no coordinates"; return CFD3D_ERR_DESCRIPTOR; }
    BlockGeom G{};
    G.imax = d.imax; G.jmax = d.jmax; G.kmax = d.kmax;
    G.ni = d.imax + 5; G.nj = d.jmax + 5; G.nk = d.kmax + 5;
    G.off = off; G.int_off = ioff;
    for (int q = 0; q < 3; ++q) { G.face_off[q] = foff[q]; G.col_off[q] = coff[q]; }
    coff[1] += (long long)(d.imax - 1) * (d.kmax - 1);
    coff[2] += (long long)(d.imax - 1) * (d.jmax - 1);
    off += (long long)G.ni * G.nj * G.nk;
    ioff += (long long)(d.imax - 1) * (d.jmax - 1) * (d.kmax - 1);
    foff[0] += (long long)d.imax * (d.jmax - 1) * (d.kmax - 1);
    foff[1] += (long long)(d.imax - 1) * d.jmax * (d.kmax - 1);
    foff[2] += (long long)(d.imax - 1) * (d.jmax - 1) * d.kmax;
    E.blk.push_back(G);
  }
  if (off >= (1ll << 31)) { E.err = "case too large for 32-bit cell indices"; return CFD3D_ERR_ARG; }
  E.ncell = off; E.nint = ioff;
  for (int q = 0; q < 3; ++q) { E.nface[q] = foff[q]; E.ncol[q] = coff[q]; }
  CFD_CUDA(cudaStreamCreateWithFlags(&E.st, cudaStreamNonBlocking));
  CFD_CUDA(cudaStreamCreateWithFlags(&E.st2, cudaStreamNonBlocking));
  for (auto& e : E.pipe_ev) CFD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  // device buffers
  const Par& c = E.par;
  const long long n = E.ncell;
  auto alloc = [&](double*& p, long long planes) -> bool {
    if (planes <= 0) { p = nullptr; return true; }
    if (cudaMalloc(&p, (size_t)planes * n * 8) != cudaSuccess) return false;
    cudaMemset(p, 0, (size_t)planes * n * 8);
    return true;
  };
  bool ok = alloc(E.d.pv, c.npv) && alloc(E.d.dv, NDV) && alloc(E.d.tv, std::max(c.ntv, 1)) &&
            alloc(E.d.gm, GM_GRD + c.ngrd) && alloc(E.d.res, c.npv) && alloc(E.d.icav, 4) && alloc(E.d.itt, 4) &&
            alloc(E.d.ocut, 1) && alloc(E.d.dt, 1) && alloc(E.d.rcav, 2) && alloc(E.d.qq, std::max(2 * c.npv * (c.nqq ? 1 : 0), 1)) &&
            alloc(E.d.dqs, c.npv) && alloc(E.d.dcv, c.npv);
  auto allocf = [&](float*& p, long long planes) -> bool {
    if (cudaMalloc(&p, (size_t)planes * n * 4) != cudaSuccess) return false;
    cudaMemset(p, 0, (size_t)planes * n * 4);
    return true;
  };
  if (c.mixed)
    ok = ok && allocf(E.d.pvf, c.npv) && allocf(E.d.fi32, 3 * c.npv) && allocf(E.d.fv32, (c.iturb == -3) ? 1 : 3 * c.npv) &&
         allocf(E.d.frec, 2 * 12) && allocf(E.d.lqf, NLQ);
  else
    ok = ok && alloc(E.d.fi, 3 * c.npv) && alloc(E.d.fv, (c.iturb == -3) ? 1 : 3 * c.npv);
  if (c.csf) ok = ok && alloc(E.d.vf, 1) && alloc(E.d.vfg, 3) && alloc(E.d.csf, 3);
  if (!ok) { E.err = "device allocation failed"; return CFD3D_ERR_NOMEM; }
  E.d.ncell = n;
  E.d.nint = E.nint;
  E.d.nblk = nblocks;
  BlockGeom* dblk = nullptr;
  CFD_CUDA(cudaMalloc(&dblk, sizeof(BlockGeom) * nblocks));
  CFD_CUDA(cudaMemcpy(dblk, E.blk.data(), sizeof(BlockGeom) * nblocks, cudaMemcpyHostToDevice));
  E.d.blk = dblk;
  CFD_CUDA(cudaMalloc(&E.d.sc, sizeof(Scalars)));
  Scalars s0{};
  s0.time_acc = 0.0;
  double big = 1.0e10;
  std::memcpy(&s0.dtmin_bits, &big, 8);
  CFD_CUDA(cudaMemcpy(E.d.sc, &s0, sizeof(Scalars), cudaMemcpyHostToDevice));
  if (E.par.gravity) {
    // the history as n, t[n], a[3 n]; a constant acceleration (src/gravity_module.f90:45-61)
    // is one row at t = 0
    std::vector<double> tab;
    if (E.par.gravity == 4) {
      const int nd = cfg->ngravity;
      tab.push_back((double)nd);
      for (int m = 0; m < nd; ++m) tab.push_back(cfg->gravity_data[4 * m]);
      for (int m = 0; m < nd; ++m) for (int e = 0; e < 3; ++e) tab.push_back(cfg->gravity_data[4 * m + 1 + e]);
    } else {
      double a[3] = {0.0, 0.0, 0.0};
      a[std::abs(E.par.gravity) - 1] = (E.par.gravity > 0 ? 1.0 : -1.0) * 9.80665;
      tab = {1.0, 0.0, a[0], a[1], a[2]};
    }
    CFD_CUDA(cudaMalloc(&E.d_grav, tab.size() * sizeof(double)));
    CFD_CUDA(cudaMemcpy(E.d_grav, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
    E.d.grav = E.d_grav;
  }
  {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // the update's CTAs all resident at once (its grid-stride loop leaves no partial last
    // wave), at most 8 per SM
    int per = 0;
    if (c.mixed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_update<true>, 128, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_update<false>, 128, 0);
    per = std::min(std::max(per, 1), 8);
    E.red_grid = (int)std::min<long long>(nblk_of(E.nint, 128), (long long)std::max(nsm, 1) * per);
  }
  CFD_CUDA(cudaMalloc(&E.d.partial, (size_t)E.red_grid * (NPVM + 2) * 8));
  // reference state: deteos at (pref, tref, y1ref, y2ref), then config%setref
  {
    double hp[4] = {cfg->pref, cfg->tref, cfg->y1ref, cfg->y2ref};
    double dvr[NDV], tvr[2] = {0.0, 0.0};
    int rc = cfd3d_eos_eval(cfg->fluid, cfg->ngas, c.with_prop, 1, &hp[0], &hp[1], &hp[2], &hp[3], dvr, tvr);
    if (rc != CFD3D_OK) { E.err = "reference-state EOS failed"; return rc; }
    E.par.rhoref = dvr[0];
    if (c.iturb == 0) {
      E.par.oref = 10.0 * cfg->uref / cfg->l_domain;
      E.par.emutref = std::pow(10.0, -5) * tvr[0];
      E.par.kref = E.par.emutref / E.par.rhoref * E.par.oref;
      if (cfg->kinf > 0) E.par.kref = cfg->kinf;
      if (cfg->oinf > 0) E.par.oref = cfg->oinf;
    } else if (c.iturb == -1) {
      // config%setref for k-epsilon (src/config_module.f90:191-194): oref is epsilon's
      E.par.kref = 1.5 * (0.0001 * cfg->uref) * (0.0001 * cfg->uref);
      E.par.emutref = std::pow(10.0, -5) * tvr[0];
      E.par.oref = 0.09 * E.par.rhoref * E.par.kref * E.par.kref / E.par.emutref;
      if (cfg->kinf > 0) E.par.kref = cfg->kinf;
      if (cfg->oinf > 0) E.par.oref = cfg->oinf;
    }
    {
      // the total-pressure inlet's construct values (src/bc_module.f90:318-321): its totals
      // and the enthalpy eos%deteos gives there
      E.par.tp_pt = 51551.30907;
      E.par.tp_tt = 300.0003719;
      double hp2[4] = {E.par.tp_pt, E.par.tp_tt, cfg->y1ref, cfg->y2ref};
      double dvt[NDV], tvt[2] = {0.0, 0.0};
      rc = cfd3d_eos_eval(cfg->fluid, cfg->ngas, c.with_prop, 1, &hp2[0], &hp2[1], &hp2[2], &hp2[3], dvt, tvt);
      if (rc != CFD3D_OK) { E.err = "total-pressure EOS failed"; return rc; }
      E.par.tp_ht = dvt[1];
    }
    // mixed form: free-stream flux tensor (gauge pressure) for the stored flux deviations
    E.par.href = dvr[1];
    const double* U = E.par.uref_vec;
    const double H = dvr[1] + 0.5 * (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
    const double sc[NPVM] = {1.0, 0.0, 0.0, 0.0, H, cfg->y1ref, cfg->y2ref, E.par.kref, E.par.oref};
    for (int e = 0; e < 3; ++e) {
      const double m = dvr[0] * U[e];
      for (int v = 0; v < NPVM; ++v) E.par.phi[v][e] = m * sc[v];
      for (int q = 0; q < 3; ++q) E.par.phi[1 + q][e] = m * U[q];
    }
    auto split = [](double x, float* o) { o[0] = (float)x; o[1] = (float)(x - (double)o[0]); };
    split(dvr[0], E.par.rhoref2);
    split(dvr[1], E.par.href2);
    for (int e = 0; e < 3; ++e) { split(U[e], E.par.U2[e]); split(dvr[0] * U[e], E.par.m2[e]); }
    for (int v = 0; v < NPVM; ++v) split((v >= 1 && v <= 3) ? U[v - 1] : sc[v], E.par.sc2[v]);
  }
  if (!setup_geometry(E, blocks, nblocks)) return CFD3D_ERR_DESCRIPTOR;
  if (c.csf && !setup_vfg_halo(E, blocks, nblocks)) return CFD3D_ERR_DESCRIPTOR;
  if (c.mixed) {
    const long long m = (long long)(GM_GRD + c.ngrd) * E.ncell;
    if (cudaMalloc(&E.d.gmf, (size_t)m * 4) != cudaSuccess) { E.err = "device allocation failed (gmf)"; return CFD3D_ERR_NOMEM; }
    k_to_f32<<<nblk_of(m, 256), 256, 0, E.st>>>(E.d.gm, E.d.gmf, m);
    // the face vectors' low parts: gm = gmf + gmlo to ~1e-14 (the df64 flux terms)
    const long long m9 = (long long)GM_GRD * E.ncell;
    if (cudaMalloc(&E.d.gmlo, (size_t)m9 * 4) != cudaSuccess) { E.err = "device allocation failed (gmlo)"; return CFD3D_ERR_NOMEM; }
    k_lo_f32<<<nblk_of(m9, 256), 256, 0, E.st>>>(E.d.gm, E.d.gmf, E.d.gmlo, m9);
    if (cudaMalloc(&E.d.clo, (size_t)c.npv * E.ncell * 8) != cudaSuccess) { E.err = "device allocation failed (closure)"; return CFD3D_ERR_NOMEM; }
    k_closure<<<nblk_of(E.nint, 256), 256, 0, E.st>>>(E.d, E.par);
    CFD_CUDA(cudaStreamSynchronize(E.st));
  }
  if (!setup_ghost_program(E, blocks, nblocks)) return CFD3D_ERR_DESCRIPTOR;
  if (c.mixed) {
    // the mixed form sweeps by tiles (its records are tile records)
    if (!setup_tiles(E)) return CFD3D_ERR_NOMEM;
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    CFD_CUDA(cudaFuncSetAttribute(k_sweep_tile<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, TILE_SMEM));
    CFD_CUDA(cudaFuncSetAttribute(k_sweep_tile<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, TILE_SMEM));
    // the largest shared-memory carveout: three tiles' records per SM
    CFD_CUDA(cudaFuncSetAttribute(k_sweep_tile<true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    CFD_CUDA(cudaFuncSetAttribute(k_sweep_tile<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_tile<true>, 32, TILE_SMEM);
    E.sweep_grid = std::max(1, std::min(std::max(per, 1) * nsm, E.d.ntile));
    CFD_CUDA(cudaDeviceSynchronize());
    return CFD3D_OK;
  }
  setup_planes(E);
  E.d.cells = E.d_planes; E.d.pos = E.d_pos; E.d.nbf = E.d_nbf; E.d.nbb = E.d_nbb;
  if (!E.d_planes || !E.d_pos || !E.d_nbf || !E.d_nbb) { E.err = "device allocation failed (sweep maps)"; return CFD3D_ERR_NOMEM; }
  if (cudaMalloc(&E.d.rec, (size_t)NREC * E.nint * 8) != cudaSuccess) { E.err = "device allocation failed (sweep records)"; return CFD3D_ERR_NOMEM; }
  if (cudaMalloc(&E.d.done, (size_t)E.d.nchunk * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&E.d.tickets, 2 * sizeof(unsigned)) != cudaSuccess) {
    E.err = "device allocation failed (sweep flags)";
    return CFD3D_ERR_NOMEM;
  }
  {
    const char* mode = std::getenv("CFD3D_SWEEP");
    E.sweep_planes = (mode && std::strcmp(mode, "planes") == 0) ? 1 : 0;
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_df<true>, SW_CH, 0);
    E.sweep_grid = std::max(1, std::min(std::min(per, 8) * nsm, E.d.nchunk));
  }
  CFD_CUDA(cudaDeviceSynchronize());
  return CFD3D_OK;
}

void cfd3d_destroy(cfd3d_handle* h) {
  if (!h) return;
  Engine& E = h->E;
  if (E.graph) cudaGraphExecDestroy(E.graph);
  double* bufs[] = {E.d.pv, E.d.dv, E.d.tv, E.d.gm, E.d.res, E.d.icav, E.d.itt, E.d.ocut, E.d.dt, E.d.rcav,
                    E.d.qq, E.d.dqs, E.d.dcv, E.d.fi, E.d.fv, E.d.partial, h->staging, E.d.clo,
                    E.d.vf, E.d.vfg, E.d.csf};
  for (double* p : bufs) cudaFree(p);
  float* fbufs[] = {E.d.pvf, E.d.fi32, E.d.fv32, E.d.frec, E.d.gmf, E.d.gmlo, E.d.lqf};
  for (float* p : fbufs) cudaFree(p);
  cudaFree((void*)E.d.blk);
  cudaFree(E.d.sc);
  for (int p = 0; p < 3; ++p) cudaFree(E.d_ops[p]);
  cudaFree(E.d_planes);
  cudaFree(E.d_pos);
  cudaFree(E.d_nbf);
  cudaFree(E.d_nbb);
  cudaFree(E.d_hft);
  cudaFree(E.d_grav);
  cudaFree((void*)E.d.vfg_halo);
  cudaFree(E.d_tp_off);
  cudaFree(E.d_tp_ent);
  cudaFree(E.d_tp_x);
  cudaFree(E.d.rec);
  cudaFree(E.d.done);
  cudaFree(E.d.tickets);
  cudaFree(E.d_chunk_t0);
  cudaFree(E.d_chunk_of);
  cudaFree(E.d.recf);
  cudaFree(E.d.dqsf);
  cudaFree(E.d_tiles);
  cudaFree(E.d.trf);
  cudaFree(E.d.tq);
  cudaFree(E.d.tyf);
  cudaFree(E.d.tyb);
  cudaFree(E.d.tin);
  adjoint_free(E);
  for (auto e : h->bev) cudaEventDestroy(e);
  if (h->cp) cudaStreamDestroy(h->cp);
  for (auto e : h->ev) if (e) cudaEventDestroy(e);
  for (auto e : E.pipe_ev) if (e) cudaEventDestroy(e);
  if (E.st2) cudaStreamDestroy(E.st2);
  if (E.st) cudaStreamDestroy(E.st);
  delete h;
}

int cfd3d_sizes(const cfd3d_handle* h, int* npv, int* ndv, int* ntv, int* nqq, int* ngrd) {
  if (!h) return CFD3D_ERR_ARG;
  const Par& c = h->E.par;
  if (npv) *npv = c.npv;
  if (ndv) *ndv = NDV;
  if (ntv) *ntv = c.ntv;
  if (nqq) *nqq = c.nqq;
  if (ngrd) *ngrd = c.ngrd;
  return CFD3D_OK;
}

int cfd3d_initialize(cfd3d_handle* h, int block, const double* pv_interior) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  if (block < 0 || block >= (int)E.blk.size()) { E.err = "bad block"; return CFD3D_ERR_ARG; }
  const BlockGeom& B = E.blk[block];
  const Par& c = E.par;
  long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
  std::vector<double> host;
  const double* src = pv_interior;
  if (!src) {
    host.resize((size_t)nint * c.npv);
    for (long long q = 0; q < nint; ++q) {
      double* p = &host[(size_t)q * c.npv];
      p[0] = 0.0; p[1] = c.uref_vec[0]; p[2] = c.uref_vec[1]; p[3] = c.uref_vec[2];
      p[4] = c.tref; p[5] = c.y1ref; p[6] = c.y2ref;
      if (c.npv > 7) { p[7] = c.kref; p[8] = c.oref; }
    }
    src = host.data();
  }
  int rc = ensure_staging(h, (size_t)nint * c.npv * 8);
  if (rc) return rc;
  CFD_CUDA(cudaMemcpyAsync(h->staging, src, (size_t)nint * c.npv * 8, cudaMemcpyHostToDevice, E.st));
  k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(h->staging, c.npv, B, E.d.pv, E.ncell, 1);
  if (c.mixed) k_init<true><<<nblk_of(nint, 128), 128, 0, E.st>>>(E.d, c, block, 1);
  else k_init<false><<<nblk_of(nint, 128), 128, 0, E.st>>>(E.d, c, block, 1);
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  // reset the solution-time accumulator of the local time step
  Scalars s;
  if ((rc = read_scalars(E, s))) return rc;
  s.time_acc = 0.0;
  CFD_CUDA(cudaMemcpy(E.d.sc, &s, sizeof(Scalars), cudaMemcpyHostToDevice));
  return CFD3D_OK;
}

}  // extern "C"

namespace {
// An upload or download that fails part-way has copies queued that read or write the
// caller's host arrays: wait for them before returning, so that no copy touches those
// arrays after the call has returned.
int drain_on_error(cfd3d_handle* h, int rc) {
  if (rc != CFD3D_OK) {
    if (h->cp) cudaStreamSynchronize(h->cp);
    cudaStreamSynchronize(h->E.st);
  }
  return rc;
}

int upload_state(cfd3d_handle* h, int block, const double* pv, const double* dv, const double* tv, const double* qq) {
  Engine& E = h->E;
  if (block < 0 || block >= (int)E.blk.size()) { E.err = "bad block"; return CFD3D_ERR_ARG; }
  const BlockGeom& B = E.blk[block];
  const Par& c = E.par;
  long long ncb = (long long)B.ni * B.nj * B.nk;
  long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
  // each array has its own staging region; the copies run back to back on the copy
  // stream and the layout kernel of each waits only for its own copy
  int rc = ensure_staging(h, (size_t)(ncb * (c.npv + NDV + c.ntv) + nint * 2 * c.npv) * 8);
  if (!rc) rc = ensure_copy_stream(h);
  if (rc) return rc;
  CFD_CUDA(cudaEventRecord(h->ev[5], E.st));          // staging no longer read by earlier work
  CFD_CUDA(cudaStreamWaitEvent(h->cp, h->ev[5], 0));
  struct { const double* a; int nv; double* dst; } items[3] = {{pv, c.npv, E.d.pv}, {dv, NDV, E.d.dv}, {tv, c.ntv, E.d.tv}};
  double* stg = h->staging;
  int q = 0;
  for (auto& it : items) {
    if (!it.a || it.nv == 0) continue;
    CFD_CUDA(cudaMemcpyAsync(stg, it.a, (size_t)ncb * it.nv * 8, cudaMemcpyHostToDevice, h->cp));
    CFD_CUDA(cudaEventRecord(h->ev[q], h->cp));
    CFD_CUDA(cudaStreamWaitEvent(E.st, h->ev[q], 0));
    k_aos_to_soa<<<nblk_of(ncb, 256), 256, 0, E.st>>>(stg, it.nv, ncb, it.dst, E.ncell, B.off);
    stg += ncb * it.nv;
    ++q;
  }
  if (qq && c.nqq) {
    CFD_CUDA(cudaMemcpyAsync(stg, qq, (size_t)nint * 2 * c.npv * 8, cudaMemcpyHostToDevice, h->cp));
    CFD_CUDA(cudaEventRecord(h->ev[q], h->cp));
    CFD_CUDA(cudaStreamWaitEvent(E.st, h->ev[q], 0));
    k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(stg, 2 * c.npv, B, E.d.qq, E.ncell, 1);
  }
  CFD_CUDA(cudaStreamSynchronize(E.st));               // waited for every copy too
  CFD_CUDA(cudaGetLastError());
  return CFD3D_OK;
}

int download_state(cfd3d_handle* h, int block, double* pv, double* dv, double* tv, double* qq, double* rcav) {
  Engine& E = h->E;
  if (block < 0 || block >= (int)E.blk.size()) { E.err = "bad block"; return CFD3D_ERR_ARG; }
  const BlockGeom& B = E.blk[block];
  const Par& c = E.par;
  long long ncb = (long long)B.ni * B.nj * B.nk;
  long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
  // the layout kernels run back to back on the engine's stream; the copy of each array
  // leaves on the copy stream as soon as its own kernel is done
  int rc = ensure_staging(h, (size_t)(ncb * (c.npv + NDV + c.ntv) + nint * (2 * c.npv + 2)) * 8);
  if (!rc) rc = ensure_copy_stream(h);
  if (rc) return rc;
  struct { double* a; int nv; double* src; } items[3] = {{pv, c.npv, E.d.pv}, {dv, NDV, E.d.dv}, {tv, c.ntv, E.d.tv}};
  double* stg = h->staging;
  int q = 0;
  auto send = [&](double* host, size_t bytes) -> int {
    CFD_CUDA(cudaEventRecord(h->ev[q], E.st));
    CFD_CUDA(cudaStreamWaitEvent(h->cp, h->ev[q], 0));
    CFD_CUDA(cudaMemcpyAsync(host, stg, bytes, cudaMemcpyDeviceToHost, h->cp));
    ++q;
    return CFD3D_OK;
  };
  for (auto& it : items) {
    if (!it.a || it.nv == 0) continue;
    k_soa_to_aos<<<nblk_of(ncb, 256), 256, 0, E.st>>>(it.src, it.nv, ncb, stg, E.ncell, B.off);
    if ((rc = send(it.a, (size_t)ncb * it.nv * 8))) return rc;
    stg += ncb * it.nv;
  }
  if (qq && c.nqq) {
    k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(stg, 2 * c.npv, B, E.d.qq, E.ncell, 0);
    if ((rc = send(qq, (size_t)nint * 2 * c.npv * 8))) return rc;
    stg += nint * 2 * c.npv;
  }
  if (rcav) {
    k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(stg, 2, B, E.d.rcav, E.ncell, 0);
    if ((rc = send(rcav, (size_t)nint * 2 * 8))) return rc;
  }
  CFD_CUDA(cudaStreamSynchronize(h->cp));             // every copy waited for its kernel
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  return CFD3D_OK;
}
}  // namespace

extern "C" {

int cfd3d_upload_state(cfd3d_handle* h, int block, const double* pv, const double* dv, const double* tv, const double* qq) {
  if (!h) return CFD3D_ERR_ARG;
  return drain_on_error(h, upload_state(h, block, pv, dv, tv, qq));
}

int cfd3d_download_csf(cfd3d_handle* h, int block, double* csf) {
  if (!h || !csf) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  if (!E.par.csf) { E.err = "the case has no surface-tension source"; return CFD3D_ERR_ARG; }
  if (block < 0 || block >= (int)E.blk.size()) { E.err = "bad block"; return CFD3D_ERR_ARG; }
  const BlockGeom& B = E.blk[block];
  const long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
  int rc = ensure_staging(h, (size_t)nint * 3 * 8);
  if (rc) return rc;
  k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(h->staging, 3, B, E.d.csf, E.ncell, 0);
  CFD_CUDA(cudaMemcpyAsync(csf, h->staging, (size_t)nint * 3 * 8, cudaMemcpyDeviceToHost, E.st));
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  return CFD3D_OK;
}

int cfd3d_download_state(cfd3d_handle* h, int block, double* pv, double* dv, double* tv, double* qq, double* rcav) {
  if (!h) return CFD3D_ERR_ARG;
  return drain_on_error(h, download_state(h, block, pv, dv, tv, qq, rcav));
}

// ---- the whole case in one call: every block's copy leaves as soon as it can, and each
// block's layout kernel overlaps the copies of the blocks after it
namespace {
int block_events(cfd3d_handle* h) {
  Engine& E = h->E;
  while (h->bev.size() < E.blk.size()) {
    cudaEvent_t e;
    CFD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->bev.push_back(e);
  }
  return CFD3D_OK;
}

int upload_primitives_all(cfd3d_handle* h, const double* const* pv, const double* const* qq) {
  Engine& E = h->E;
  const Par& c = E.par;
  const int nb = (int)E.blk.size();
  const bool hist = qq && c.nqq;
  size_t total = 0;
  for (int b = 0; b < nb; ++b) {
    if (!pv[b]) { E.err = "pv is required for every block"; return CFD3D_ERR_ARG; }
    const BlockGeom& B = E.blk[b];
    total += (size_t)B.ni * B.nj * B.nk * c.npv;
    if (hist && qq[b]) total += (size_t)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1) * 2 * c.npv;
  }
  int rc = ensure_staging(h, total * 8);
  if (!rc) rc = ensure_copy_stream(h);
  if (!rc) rc = block_events(h);
  if (rc) return rc;
  CFD_CUDA(cudaMemsetAsync(&E.d.sc->pv_changed, 0, sizeof(int), E.st));
  CFD_CUDA(cudaEventRecord(h->ev[5], E.st));          // staging no longer read by earlier work
  CFD_CUDA(cudaStreamWaitEvent(h->cp, h->ev[5], 0));
  std::vector<double*> spv(nb), sqq(nb, nullptr);
  double* stg = h->staging;
  for (int b = 0; b < nb; ++b) {
    const BlockGeom& B = E.blk[b];
    const size_t ncb = (size_t)B.ni * B.nj * B.nk, nint = (size_t)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
    spv[b] = stg;
    CFD_CUDA(cudaMemcpyAsync(stg, pv[b], ncb * c.npv * 8, cudaMemcpyHostToDevice, h->cp));
    stg += ncb * c.npv;
    if (hist && qq[b]) {
      sqq[b] = stg;
      CFD_CUDA(cudaMemcpyAsync(stg, qq[b], nint * 2 * c.npv * 8, cudaMemcpyHostToDevice, h->cp));
      stg += nint * 2 * c.npv;
    }
    CFD_CUDA(cudaEventRecord(h->bev[b], h->cp));
  }
  for (int b = 0; b < nb; ++b) {
    const BlockGeom& B = E.blk[b];
    const long long ncb = (long long)B.ni * B.nj * B.nk, nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
    CFD_CUDA(cudaStreamWaitEvent(E.st, h->bev[b], 0));
    if (c.mixed) k_take_pv<true><<<nblk_of(ncb, 128), 128, 0, E.st>>>(spv[b], B, E.d, c);
    else k_take_pv<false><<<nblk_of(ncb, 128), 128, 0, E.st>>>(spv[b], B, E.d, c);
    if (sqq[b]) k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(sqq[b], 2 * c.npv, B, E.d.qq, E.ncell, 1);
  }
  if (c.iturb >= -1 && c.ntv >= 3) {
    if (c.mixed) k_eddy<true><<<nblk_of(E.nint, 128), 128, 0, E.st>>>(E.d, c, 0, E.nint, 1);
    else k_eddy<false><<<nblk_of(E.nint, 128), 128, 0, E.st>>>(E.d, c, 0, E.nint, 1);
  }
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  return CFD3D_OK;
}

int download_state_all(cfd3d_handle* h, double* const* pv, double* const* dv, double* const* tv) {
  Engine& E = h->E;
  const Par& c = E.par;
  const int nb = (int)E.blk.size();
  size_t total = 0;
  for (int b = 0; b < nb; ++b) {
    const BlockGeom& B = E.blk[b];
    const size_t ncb = (size_t)B.ni * B.nj * B.nk;
    total += ncb * ((pv && pv[b] ? c.npv : 0) + (dv && dv[b] ? NDV : 0) + (tv && tv[b] ? c.ntv : 0));
  }
  int rc = ensure_staging(h, std::max<size_t>(total, 1) * 8);
  if (!rc) rc = ensure_copy_stream(h);
  if (!rc) rc = block_events(h);
  if (rc) return rc;
  double* stg = h->staging;
  for (int b = 0; b < nb; ++b) {
    const BlockGeom& B = E.blk[b];
    const long long ncb = (long long)B.ni * B.nj * B.nk;
    struct { double* a; int nv; const double* src; } items[3] = {
        {pv ? pv[b] : nullptr, c.npv, E.d.pv}, {dv ? dv[b] : nullptr, NDV, E.d.dv}, {tv ? tv[b] : nullptr, c.ntv, E.d.tv}};
    double* first = stg;
    for (auto& it : items) {
      if (!it.a || it.nv == 0) continue;
      k_soa_to_aos<<<nblk_of(ncb, 256), 256, 0, E.st>>>(it.src, it.nv, ncb, stg, E.ncell, B.off);
      stg += ncb * it.nv;
    }
    CFD_CUDA(cudaEventRecord(h->bev[b], E.st));
    CFD_CUDA(cudaStreamWaitEvent(h->cp, h->bev[b], 0));
    double* s2 = first;
    for (auto& it : items) {
      if (!it.a || it.nv == 0) continue;
      CFD_CUDA(cudaMemcpyAsync(it.a, s2, (size_t)ncb * it.nv * 8, cudaMemcpyDeviceToHost, h->cp));
      s2 += ncb * it.nv;
    }
  }
  CFD_CUDA(cudaStreamSynchronize(h->cp));
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  return CFD3D_OK;
}
}  // namespace

int cfd3d_upload_primitives_all(cfd3d_handle* h, const double* const* pv, const double* const* qq) {
  if (!h || !pv) return CFD3D_ERR_ARG;
  return drain_on_error(h, upload_primitives_all(h, pv, qq));
}

int cfd3d_download_state_all(cfd3d_handle* h, double* const* pv, double* const* dv, double* const* tv) {
  if (!h) return CFD3D_ERR_ARG;
  return drain_on_error(h, download_state_all(h, pv, dv, tv));
}

int cfd3d_upload_primitives(cfd3d_handle* h, int block, const double* pv, const double* qq) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  if (!pv) { E.err = "pv is required"; return CFD3D_ERR_ARG; }
  int rc = drain_on_error(h, upload_state(h, block, pv, nullptr, nullptr, qq));
  if (rc) return rc;
  // dv, tv(1:2) by the EOS of the update, then tv(3) by its eddy viscosity (which reads
  // the block's ghost pv as uploaded: those of the boundary program before the update)
  const BlockGeom& B = E.blk[block];
  const Par& c = E.par;
  const long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
  if (c.mixed) k_init<true><<<nblk_of(nint, 128), 128, 0, E.st>>>(E.d, c, block, 0);
  else k_init<false><<<nblk_of(nint, 128), 128, 0, E.st>>>(E.d, c, block, 0);
  if (c.iturb >= -1 && c.ntv >= 3) {
    if (c.mixed) k_eddy<true><<<nblk_of(nint, 128), 128, 0, E.st>>>(E.d, c, B.int_off, B.int_off + nint);
    else k_eddy<false><<<nblk_of(nint, 128), 128, 0, E.st>>>(E.d, c, B.int_off, B.int_off + nint);
  }
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  return CFD3D_OK;
}

// ---- checkpoints ----------------------------------------------------------------------
// The MPI-IO file of variable%export_variable (src/variable_module.f90:116-182), read back
// by t_ini_restart%restart (src/initial_module.f90:245-389).  Rank r of the reference owns
// block r, so the file is the blocks' records in block order; the displacement of a record
// is the sum of the sizes before it (src/variable_module.f90:80-91).
namespace {

struct CkptRecord {
  long long npad, nint;                     // padded and interior cells of the block
  bool turb, cav, csf;                      // l_turb (iturb >= -1), l_cav (ncav != 0), l_csf
  long long pv_off, emut_off, qq_off, rcav_off, csf_off, bytes;   // byte offsets within the record
};

CkptRecord ckpt_record(const Par& c, const BlockGeom& B, bool with_qq) {
  CkptRecord r;
  r.npad = (long long)B.ni * B.nj * B.nk;
  r.nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
  r.turb = c.iturb >= -1;
  r.cav = c.ncav != 0;
  r.csf = c.csf != 0;
  r.pv_off = 4 + 4 + 8;                      // nt_phy, nt (default integers), time
  r.emut_off = r.pv_off + 8ll * c.npv * r.npad;
  r.qq_off = r.emut_off + (r.turb ? 8ll * r.npad : 0);
  r.rcav_off = r.qq_off + (with_qq ? 8ll * c.nqq * c.npv * r.nint : 0);
  r.csf_off = r.rcav_off + (r.cav ? 16ll * r.nint : 0);
  r.bytes = r.csf_off + (r.csf ? 24ll * r.nint : 0);
  return r;
}

// whole-buffer positional I/O (a single pread/pwrite may move fewer bytes than asked)
bool pio(int fd, void* buf, long long n, long long off, bool wr) {
  char* p = (char*)buf;
  while (n > 0) {
    const ssize_t k = wr ? pwrite(fd, p, (size_t)std::min(n, 1ll << 30), (off_t)off)
                         : pread(fd, p, (size_t)std::min(n, 1ll << 30), (off_t)off);
    if (k <= 0) return false;
    p += k; off += k; n -= k;
  }
  return true;
}

// interior cells (2:imax, 2:jmax, 2:kmax) of one component of a padded Fortran array
// a(nv, -1:imax+3, ..) into out(2:imax, ..)
void padded_to_interior(const BlockGeom& B, const double* a, int nv, int v, double* out) {
  long long q = 0;
  for (int k = 2; k <= B.kmax; ++k)
    for (int j = 2; j <= B.jmax; ++j)
      for (int i = 2; i <= B.imax; ++i)
        out[q++] = a[((((long long)(k + 1) * B.nj) + (j + 1)) * B.ni + (i + 1)) * nv + v];
}

}  // namespace

int cfd3d_checkpoint_write(cfd3d_handle* h, const char* path, int nt_phy, int nt, double time) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  const Par& c = E.par;
  if (!path) { E.err = "checkpoint path is NULL"; return CFD3D_ERR_ARG; }
  // mpi_mode_wronly + mpi_mode_create: created when missing, never truncated
  const int fd = open(path, O_WRONLY | O_CREAT, 0644);
  if (fd < 0) { E.err = std::string("cannot open checkpoint for writing: ") + path; return CFD3D_ERR_IO; }
  long long disp = 0;
  int rc = CFD3D_OK;
  std::vector<double> pv, tv, qq, rcav, emut, csf;
  for (int b = 0; b < (int)E.blk.size() && rc == CFD3D_OK; ++b) {
    const BlockGeom& B = E.blk[b];
    const CkptRecord r = ckpt_record(c, B, true);
    pv.assign((size_t)(c.npv * r.npad), 0.0);
    tv.assign((size_t)(std::max(c.ntv, 1) * r.npad), 0.0);
    qq.assign((size_t)std::max(2ll * c.npv * r.nint, 1ll), 0.0);
    rcav.assign((size_t)(2 * r.nint), 0.0);
    rc = cfd3d_download_state(h, b, pv.data(), nullptr, c.ntv ? tv.data() : nullptr, c.nqq ? qq.data() : nullptr,
                              rcav.data());
    if (rc) break;
    if (r.csf) {
      csf.assign((size_t)(3 * r.nint), 0.0);
      if ((rc = cfd3d_download_csf(h, b, csf.data()))) break;
    }
    char head[16];
    const int32_t i2[2] = {(int32_t)nt_phy, (int32_t)nt};
    memcpy(head, i2, 8);
    memcpy(head + 8, &time, 8);
    bool ok = pio(fd, head, 16, disp, true) && pio(fd, pv.data(), 8ll * c.npv * r.npad, disp + r.pv_off, true);
    if (ok && r.turb) {
      // emut = tv(3, :, :, :) over the padded range (:141-150)
      emut.assign((size_t)r.npad, 0.0);
      if (c.ntv >= 3)
        for (long long q = 0; q < r.npad; ++q) emut[(size_t)q] = tv[(size_t)(q * c.ntv + 2)];
      ok = pio(fd, emut.data(), 8ll * r.npad, disp + r.emut_off, true);
    }
    if (ok && c.nqq) ok = pio(fd, qq.data(), 8ll * c.nqq * c.npv * r.nint, disp + r.qq_off, true);
    if (ok && r.cav) ok = pio(fd, rcav.data(), 16ll * r.nint, disp + r.rcav_off, true);
    if (ok && r.csf) ok = pio(fd, csf.data(), 24ll * r.nint, disp + r.csf_off, true);
    if (!ok) { E.err = std::string("checkpoint write failed: ") + path; rc = CFD3D_ERR_IO; }
    disp += r.bytes;
  }
  if (close(fd) != 0 && rc == CFD3D_OK) { E.err = std::string("checkpoint close failed: ") + path; rc = CFD3D_ERR_IO; }
  return rc;
}

int cfd3d_checkpoint_read(cfd3d_handle* h, const char* path, int steady_start, int* nps, int* nts,
                          double* timeprev) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  const Par& c = E.par;
  if (!path) { E.err = "checkpoint path is NULL"; return CFD3D_ERR_ARG; }
  const int fd = open(path, O_RDONLY);
  if (fd < 0) { E.err = std::string("cannot open checkpoint: ") + path; return CFD3D_ERR_IO; }
  // the steadyini variant (src/initial_module.f90:103-242) reads records without qq
  const bool with_qq = !steady_start;
  long long disp = 0;
  int rc = CFD3D_OK;
  int32_t head_i[2] = {0, 0};
  double head_t = 0.0;
  std::vector<double> pv, buf, interior;
  for (int b = 0; b < (int)E.blk.size() && rc == CFD3D_OK; ++b) {
    const BlockGeom& B = E.blk[b];
    const CkptRecord r = ckpt_record(c, B, with_qq);
    char head[16];
    if (!pio(fd, head, 16, disp, false)) { E.err = "checkpoint shorter than the case's blocks"; rc = CFD3D_ERR_IO; break; }
    int32_t bi[2];
    double bt;
    memcpy(bi, head, 8);
    memcpy(&bt, head + 8, 8);
    if (b == 0) { head_i[0] = bi[0]; head_i[1] = bi[1]; head_t = bt; }
    pv.assign((size_t)(c.npv * r.npad), 0.0);
    if (!pio(fd, pv.data(), 8ll * c.npv * r.npad, disp + r.pv_off, false)) {
      E.err = "checkpoint shorter than the case's blocks"; rc = CFD3D_ERR_IO; break;
    }
    // pv of the interior cells, then dv / tv by the EOS and qq from the state (set_others)
    interior.assign((size_t)(c.npv * r.nint), 0.0);
    buf.assign((size_t)r.nint, 0.0);
    for (int v = 0; v < c.npv; ++v) {
      padded_to_interior(B, pv.data(), c.npv, v, buf.data());
      for (long long q = 0; q < r.nint; ++q) interior[(size_t)(q * c.npv + v)] = buf[(size_t)q];
    }
    if ((rc = cfd3d_initialize(h, b, interior.data()))) break;
    // tv(3) = emut, qq, rcav and the surface-tension source from the file, interior cells only
    struct Part { bool on; long long off; int nv; bool padded; double* dst; };
    const Part parts[4] = {
        {r.turb && c.ntv >= 3, r.emut_off, 1, true, E.d.tv + 2 * E.ncell},
        {with_qq && c.nqq > 0, r.qq_off, c.nqq * c.npv, false, E.d.qq},
        {r.cav, r.rcav_off, 2, false, E.d.rcav},
        {r.csf, r.csf_off, 3, false, E.d.csf}};
    for (const Part& p : parts) {
      if (!p.on) continue;
      const long long cnt = p.nv * (p.padded ? r.npad : r.nint);
      buf.assign((size_t)cnt, 0.0);
      if (!pio(fd, buf.data(), 8ll * cnt, disp + p.off, false)) {
        E.err = "checkpoint shorter than the case's blocks"; rc = CFD3D_ERR_IO; break;
      }
      if (p.padded) {
        interior.assign((size_t)r.nint, 0.0);
        padded_to_interior(B, buf.data(), 1, 0, interior.data());
        buf.swap(interior);
      }
      if ((rc = ensure_staging(h, 8 * (size_t)(p.nv * r.nint)))) break;
      cudaError_t e = cudaMemcpyAsync(h->staging, buf.data(), 8 * (size_t)(p.nv * r.nint), cudaMemcpyHostToDevice, E.st);
      if (e != cudaSuccess) { E.err = cudaGetErrorString(e); rc = CFD3D_ERR_CUDA; break; }
      k_interior_io<<<nblk_of(r.nint, 256), 256, 0, E.st>>>(h->staging, p.nv, B, p.dst, E.ncell, 1);
      e = cudaStreamSynchronize(E.st);
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e != cudaSuccess) { E.err = cudaGetErrorString(e); rc = CFD3D_ERR_CUDA; break; }
    }
    disp += r.bytes;
  }
  close(fd);
  if (rc) return rc;
  // the counters the solve loop restarts from (src/initial_module.f90:238-240,373-381)
  int p = head_i[0], t = head_i[1];
  double tp = head_t;
  if (steady_start) { p = 1; t = 1; tp = 0.0; }
  else {
    ++t; ++p;
    if (c.nsteady >= 1) t = 1;
    else p = 1;
  }
  if (nps) *nps = p;
  if (nts) *nts = t;
  if (timeprev) *timeprev = tp;
  return CFD3D_OK;
}

static int finish_iteration(cfd3d_handle* h, int nt_phy, double timeprev, double* time_out, double* res_l2, int* loc) {
  Engine& E = h->E;
  Scalars s;
  int rc = read_scalars(E, s);
  if (rc) return rc;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { E.err = cudaGetErrorString(e); return CFD3D_ERR_CUDA; }
  double t = (E.par.nsteady == 0) ? s.time_acc + timeprev : E.par.dt_phy * (double)nt_phy;
  if (time_out) *time_out = t;
  if (res_l2) for (int v = 0; v < E.par.npv; ++v) res_l2[v] = s.res[v];
  if (loc) {
    loc[0] = -1; loc[1] = loc[2] = loc[3] = 0;
    if (s.resmax_cell >= 0) {
      long long q = s.resmax_cell;
      int b = 0;
      while (b + 1 < (int)E.blk.size() && q >= E.blk[b + 1].int_off) ++b;
      const BlockGeom& B = E.blk[b];
      long long l = q - B.int_off;
      int ni = B.imax - 1, nj = B.jmax - 1;
      loc[0] = b; loc[1] = (int)(l % ni) + 2; loc[2] = (int)((l / ni) % nj) + 2; loc[3] = (int)(l / ((long long)ni * nj)) + 2;
    }
  }
  if (s.sweep_stall) {
    E.err = "a dataflow sweep's wait for a neighbour cell ran out";
    int zero = 0;
    cudaMemcpy(&E.d.sc->sweep_stall, &zero, sizeof(int), cudaMemcpyHostToDevice);
    return CFD3D_ERR_TIMEOUT;
  }
  if (s.nonfinite) {
    E.err = "non-finite value in the updated state";
    int zero = 0;
    cudaMemcpy(&E.d.sc->nonfinite, &zero, sizeof(int), cudaMemcpyHostToDevice);
    return CFD3D_ERR_NONFINITE;
  }
  return CFD3D_OK;
}

// the time inputs of the boundary program (heat-flux histories) for the next launches
static int set_bc_time(Engine& E, int nt_phy, double timeprev) {
  if (!E.d_hft && !E.d_grav) return CFD3D_OK;
  struct { double tp; int nt; } v{timeprev, nt_phy};
  static_assert(offsetof(Scalars, nt_phy) == offsetof(Scalars, timeprev) + 8, "timeprev, nt_phy of Scalars");
  CFD_CUDA(cudaMemcpyAsync((char*)E.d.sc + offsetof(Scalars, timeprev), &v, 12, cudaMemcpyHostToDevice, E.st));
  return CFD3D_OK;
}

int cfd3d_iterate(cfd3d_handle* h, int nt_phy, int nt, double timeprev, double* time_out, double* res_l2, int* loc) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  (void)nt;
  int rc = build_graph(E);
  if (rc) return rc;
  if ((rc = set_bc_time(E, nt_phy, timeprev))) return rc;
  CFD_CUDA(cudaGraphLaunch(E.graph, E.st));
  return finish_iteration(h, nt_phy, timeprev, time_out, res_l2, loc);
}

int cfd3d_iterate_n(cfd3d_handle* h, int niter, int nt_phy, int nt0, double timeprev, double* time_out, double* res_l2) {
  if (!h || niter < 1) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  (void)nt0;
  int rc = build_graph(E);
  if (rc) return rc;
  if ((rc = set_bc_time(E, nt_phy, timeprev))) return rc;
  for (int q = 0; q < niter; ++q) CFD_CUDA(cudaGraphLaunch(E.graph, E.st));
  return finish_iteration(h, nt_phy, timeprev, time_out, res_l2, nullptr);
}

int cfd3d_unsteady_shift(cfd3d_handle* h) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  if (!E.par.nqq) return CFD3D_OK;
  k_unsteady_shift<<<nblk_of(E.nint, 128), 128, 0, E.st>>>(E.d, E.par);
  CFD_CUDA(cudaStreamSynchronize(E.st));
  return CFD3D_OK;
}

int cfd3d_residual(cfd3d_handle* h, int block, double* res, double* icav, double* itt, double* omega_cut) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  if (block < 0 || block >= (int)E.blk.size()) { E.err = "bad block"; return CFD3D_ERR_ARG; }
  launch_iteration(E, false);
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  const BlockGeom& B = E.blk[block];
  long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
  int rc = ensure_staging(h, (size_t)nint * 9 * 8);
  if (rc) return rc;
  struct { double* a; int nv; double* src; } items[4] = {{res, E.par.npv, E.d.res}, {icav, 4, E.d.icav}, {itt, 4, E.d.itt}, {omega_cut, 1, E.d.ocut}};
  for (auto& it : items) {
    if (!it.a) continue;
    k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(h->staging, it.nv, B, it.src, E.ncell, 0);
    CFD_CUDA(cudaMemcpyAsync(it.a, h->staging, (size_t)nint * it.nv * 8, cudaMemcpyDeviceToHost, E.st));
    CFD_CUDA(cudaStreamSynchronize(E.st));
  }
  return CFD3D_OK;
}

int cfd3d_residual_vjp(cfd3d_handle* h, const double* cot, double* g_state, double* g_params) {
  if (!h || !cot) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  const Par& c = E.par;
  long long maxint = 0;
  for (const BlockGeom& B : E.blk) maxint = std::max(maxint, (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1));
  int rc = ensure_staging(h, (size_t)maxint * c.npv * 8);
  if (rc) return rc;
  if (E.par.iturb == -1) { E.err = "the adjoint does not cover the k-epsilon model"; return CFD3D_ERR_ARG; }
  if (E.d.ntp) { E.err = "the adjoint does not cover total-pressure inlets"; return CFD3D_ERR_ARG; }
  if (E.par.csf) { E.err = "the adjoint does not cover the surface-tension source"; return CFD3D_ERR_ARG; }
  if (E.par.rot) { E.err = "the adjoint does not cover the rotating frame"; return CFD3D_ERR_ARG; }
  if ((rc = adjoint_buffers(E))) return rc;
  // the cotangent, block after block, into the padded interior
  size_t off = 0;
  for (const BlockGeom& B : E.blk) {
    const long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
    CFD_CUDA(cudaMemcpyAsync(h->staging, cot + off, (size_t)nint * c.npv * 8, cudaMemcpyHostToDevice, E.st));
    k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(h->staging, c.npv, B, E.adj_lam, E.ncell, 1);
    CFD_CUDA(cudaStreamSynchronize(E.st));
    off += (size_t)nint * c.npv;
  }
  // the forward boundary program: the ghost values the residual sees
  for (int p = 0; p < 3; ++p)
    if (E.nops[p]) k_ghost<<<nblk_of(E.nops[p], 128), 128, 0, E.st>>>(E.d, c, E.d_ops[p], E.nops[p]);
  if ((rc = adjoint_launch(E))) return rc;
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  if (g_state) {
    off = 0;
    for (const BlockGeom& B : E.blk) {
      const long long nint = (long long)(B.imax - 1) * (B.jmax - 1) * (B.kmax - 1);
      k_interior_io<<<nblk_of(nint, 256), 256, 0, E.st>>>(h->staging, c.npv, B, E.adj_gpv, E.ncell, 0);
      CFD_CUDA(cudaMemcpyAsync(g_state + off, h->staging, (size_t)nint * c.npv * 8, cudaMemcpyDeviceToHost, E.st));
      CFD_CUDA(cudaStreamSynchronize(E.st));
      off += (size_t)nint * c.npv;
    }
  }
  if (g_params) {
    CFD_CUDA(cudaMemcpyAsync(g_params, E.adj_gpar, 3 * 8, cudaMemcpyDeviceToHost, E.st));
    CFD_CUDA(cudaStreamSynchronize(E.st));
  }
  return CFD3D_OK;
}

int cfd3d_autotune(cfd3d_handle* h, int reps, int* choice) {
  if (!h || reps < 1) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  const DevPtr& d = E.d;
  const Par& c = E.par;
  launch_iteration(E, false);   // boundary program, fluxes, residual and sweep records
  CFD_CUDA(cudaStreamSynchronize(E.st));
  const int cands[3] = {64, 128, 256};
  // threads per CTA of the face kernels
  int best = E.tpb_face;
  float tbest = 1e30f;
  for (int T : cands) {
    E.tpb_face = T;
    const float t = time_calls(E, reps, [&] {
      if (c.mixed) launch_face_flux_mixed(E, E.st, 0, (int)E.blk.size());
      else launch_face_flux(E, E.st);
    });
    if (t < tbest) { tbest = t; best = T; }
  }
  E.tpb_face = best;
  // threads per CTA of the residual kernel
  best = E.tpb_rhs;
  tbest = 1e30f;
  for (int T : cands) {
    const float t = time_calls(E, reps, [&] {
      launch_rhs(E, E.st, T, c.timemethod == 3, false);
    });
    if (t < tbest) { tbest = t; best = T; }
  }
  E.tpb_rhs = best;
  // groups of blocks of the mixed form's face / residual pipeline: 1, 2, 4, ... up to the
  // block count
  if (c.mixed) {
    const int nb = (int)E.blk.size();
    int bestp = 1;
    tbest = 1e30f;
    for (int q = 1; q <= std::min(nb, Engine::MAX_PIPE); q *= 2) {
      E.pipe_groups = q;
      const float t = time_calls(E, reps, [&] { launch_face_rhs(E, E.st, c.timemethod == 3, false); });
      if (t < tbest) { tbest = t; bestp = q; }
    }
    E.pipe_groups = bestp;
  }
  // persistent CTAs per SM of the dataflow sweeps (up to the occupancy limit)
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (c.mixed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_tile<true>, 32, TILE_SMEM);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_df<true>, SW_CH, 0);
  const int nwork = c.mixed ? d.ntile : d.nchunk;
  int bestg = E.sweep_grid;
  tbest = 1e30f;
  for (int m = 1; c.timemethod == 3 && m <= std::max(per, 1); ++m) {   // (no sweeps in the explicit schemes)
    if (m > 4 && m % 2 && m != per) continue;   // 1, 2, 3, 4, 6, 8, ... and the occupancy limit
    const int grid = std::max(1, std::min(m * nsm, nwork));
    // (the timed sweeps run on the records of the iteration launched above; the forward one
    // rewrites the right-hand side it reads, which changes the values but not the work)
    const float t = time_calls(E, reps, [&] {
      cudaMemsetAsync(d.tickets, 0, 2 * sizeof(unsigned), E.st);
      cudaMemsetAsync(d.done, 0, (size_t)nwork * sizeof(int), E.st);
      if (c.mixed) k_sweep_tile<true><<<grid, 32, TILE_SMEM, E.st>>>(d, c, SWEEP_SPIN, -1);
      else k_sweep_df<true><<<grid, SW_CH, 0, E.st>>>(d, c, SWEEP_SPIN, -1);
      cudaMemsetAsync(d.done, 0, (size_t)nwork * sizeof(int), E.st);
      if (c.mixed) k_sweep_tile<false><<<grid, 32, TILE_SMEM, E.st>>>(d, c, SWEEP_SPIN, -1);
      else k_sweep_df<false><<<grid, SW_CH, 0, E.st>>>(d, c, SWEEP_SPIN, -1);
    });
    if (t < tbest) { tbest = t; bestg = grid; }
  }
  E.sweep_grid = bestg;
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  Scalars sc;
  int rc = read_scalars(E, sc);
  if (rc) return rc;
  if (sc.sweep_stall) {
    int zero = 0;
    CFD_CUDA(cudaMemcpy(&E.d.sc->sweep_stall, &zero, sizeof(int), cudaMemcpyHostToDevice));
    E.err = "a dataflow sweep's wait for a neighbour cell ran out";
    return CFD3D_ERR_TIMEOUT;
  }
  // the iteration graph is captured again with the new shapes
  if (E.graph) { cudaGraphExecDestroy(E.graph); E.graph = nullptr; }
  E.graph_ready = 0;
  if (choice) { choice[0] = E.tpb_face; choice[1] = E.tpb_rhs; choice[2] = (E.sweep_grid + nsm - 1) / std::max(nsm, 1); }
  return CFD3D_OK;
}

int cfd3d_sweep_stall_test(cfd3d_handle* h) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  const DevPtr& d = E.d;
  const Par& c = E.par;
  // fresh sweep records of the current state, then a forward sweep whose first chunk never
  // raises its flags, with a short poll limit
  launch_iteration(E, false);
  CFD_CUDA(cudaMemsetAsync(d.tickets, 0, 2 * sizeof(unsigned), E.st));
  CFD_CUDA(cudaMemsetAsync(d.done, 0, (size_t)(c.mixed ? d.ntile : d.nchunk) * sizeof(int), E.st));
  if (c.mixed) k_sweep_tile<true><<<E.sweep_grid, 32, TILE_SMEM, E.st>>>(d, c, 1 << 12, 0);
  else k_sweep_df<true><<<E.sweep_grid, SW_CH, 0, E.st>>>(d, c, 1 << 12, 0);
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaGetLastError());
  Scalars sc;
  int rc = read_scalars(E, sc);
  if (rc) return rc;
  if (!sc.sweep_stall) { E.err = "the withheld flags did not stop the sweep's waits"; return CFD3D_OK; }
  int zero = 0;
  CFD_CUDA(cudaMemcpy(&E.d.sc->sweep_stall, &zero, sizeof(int), cudaMemcpyHostToDevice));
  E.err = "a dataflow sweep's wait for a neighbour cell ran out";
  return CFD3D_ERR_TIMEOUT;
}

int cfd3d_grid_metrics(cfd3d_handle* h, int block, double* cx, double* ex, double* tx, double* grd) {
  if (!h) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  if (block < 0 || block >= (int)E.blk.size()) { E.err = "bad block"; return CFD3D_ERR_ARG; }
  const BlockGeom& B = E.blk[block];
  const int ngrd = E.par.ngrd;
  std::vector<double> gm((size_t)(GM_GRD + ngrd) * B.ni * B.nj * B.nk);
  long long ncb = (long long)B.ni * B.nj * B.nk;
  for (int v = 0; v < GM_GRD + ngrd; ++v)
    CFD_CUDA(cudaMemcpy(&gm[(size_t)v * ncb], E.d.gm + v * E.ncell + B.off, ncb * 8, cudaMemcpyDeviceToHost));
  const int im = B.imax, jm = B.jmax, km = B.kmax;
  auto li = [&](int i, int j, int k) { return (size_t)(i + 1) + (size_t)B.ni * ((j + 1) + (size_t)B.nj * (k + 1)); };
  size_t q = 0;
  if (cx) for (int k = 1; k <= km + 1; ++k) for (int j = 1; j <= jm + 1; ++j) for (int i = 1; i <= im; ++i) for (int v = 0; v < 3; ++v) cx[q++] = gm[(GM_CX + v) * ncb + li(i, j, k)];
  q = 0;
  if (ex) for (int k = 1; k <= km + 1; ++k) for (int j = 1; j <= jm; ++j) for (int i = 1; i <= im + 1; ++i) for (int v = 0; v < 3; ++v) ex[q++] = gm[(GM_EX + v) * ncb + li(i, j, k)];
  q = 0;
  if (tx) for (int k = 1; k <= km; ++k) for (int j = 1; j <= jm + 1; ++j) for (int i = 1; i <= im + 1; ++i) for (int v = 0; v < 3; ++v) tx[q++] = gm[(GM_TX + v) * ncb + li(i, j, k)];
  q = 0;
  if (grd) for (int k = 1; k <= km + 1; ++k) for (int j = 1; j <= jm + 1; ++j) for (int i = 1; i <= im + 1; ++i) for (int v = 0; v < ngrd; ++v) grd[q++] = gm[(GM_GRD + v) * ncb + li(i, j, k)];
  return CFD3D_OK;
}

int cfd3d_set_device(int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CFD3D_ERR_NODEVICE;
  if (device < 0 || device >= ndev) return CFD3D_ERR_ARG;
  return cudaSetDevice(device) == cudaSuccess ? CFD3D_OK : CFD3D_ERR_CUDA;
}

int cfd3d_time_iterate(cfd3d_handle* h, int niter, double* ms) {
  if (!h || niter < 1 || !ms) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  int rc = build_graph(E);
  if (rc) return rc;
  cudaEvent_t a, b;
  CFD_CUDA(cudaEventCreate(&a));
  CFD_CUDA(cudaEventCreate(&b));
  CFD_CUDA(cudaStreamSynchronize(E.st));
  CFD_CUDA(cudaEventRecord(a, E.st));
  for (int q = 0; q < niter; ++q) CFD_CUDA(cudaGraphLaunch(E.graph, E.st));
  CFD_CUDA(cudaEventRecord(b, E.st));
  CFD_CUDA(cudaEventSynchronize(b));
  float f = 0.0f;
  CFD_CUDA(cudaEventElapsedTime(&f, a, b));
  *ms = f;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  Scalars s;
  return read_scalars(E, s);
}

int cfd3d_profile_iterate(cfd3d_handle* h, double* stage_ms) {
  if (!h || !stage_ms) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  cudaEvent_t ev[9];
  for (int q = 0; q < 9; ++q) CFD_CUDA(cudaEventCreate(&ev[q]));
  CFD_CUDA(cudaStreamSynchronize(E.st));
  // the stages in sequence: the face / residual pipeline off, so that the face stage and
  // the residual are timed apart
  const int groups = E.pipe_groups;
  E.pipe_groups = 1;
  launch_iteration(E, true, ev);
  E.pipe_groups = groups;
  CFD_CUDA(cudaEventSynchronize(ev[8]));
  for (int q = 0; q < CFD3D_NSTAGES; ++q) {
    float f = 0.0f;
    CFD_CUDA(cudaEventElapsedTime(&f, ev[q], ev[q + 1]));
    stage_ms[q] = f;
  }
  for (int q = 0; q < 9; ++q) cudaEventDestroy(ev[q]);
  CFD_CUDA(cudaGetLastError());
  return CFD3D_OK;
}

int cfd3d_convert_selftest(long long n, unsigned long long seed, long long* mismatches) {
  if (n < 1 || !mismatches) return CFD3D_ERR_ARG;
  unsigned long long* d_bad = nullptr;
  if (cudaMalloc(&d_bad, 2 * sizeof(unsigned long long)) != cudaSuccess) return CFD3D_ERR_NOMEM;
  cudaMemset(d_bad, 0, 2 * sizeof(unsigned long long));
  k_convert_check<<<nblk_of(n, 256), 256>>>(n, seed, d_bad);
  unsigned long long bad[2] = {0, 0};
  const cudaError_t e = cudaMemcpy(bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost);
  cudaFree(d_bad);
  if (e != cudaSuccess) return CFD3D_ERR_CUDA;
  mismatches[0] = (long long)bad[0];
  mismatches[1] = (long long)bad[1];
  return CFD3D_OK;
}

int cfd3d_launch_shapes(const cfd3d_handle* h, int* shapes) {
  if (!h || !shapes) return CFD3D_ERR_ARG;
  const Engine& E = h->E;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nb = (int)E.blk.size();
  shapes[0] = E.tpb_face;
  shapes[1] = E.tpb_rhs;
  shapes[2] = (E.sweep_grid + nsm - 1) / std::max(nsm, 1);
  shapes[3] = E.par.mixed ? std::min(std::max(E.pipe_groups, 1), std::min(nb, Engine::MAX_PIPE)) : 1;
  return CFD3D_OK;
}

int cfd3d_set_launch_shapes(cfd3d_handle* h, const int* shapes) {
  if (!h || !shapes) return CFD3D_ERR_ARG;
  Engine& E = h->E;
  const Par& c = E.par;
  auto threads_ok = [](int T) { return T == 64 || T == 128 || T == 256; };
  if (!threads_ok(shapes[0]) || !threads_ok(shapes[1])) { E.err = "threads per CTA must be 64, 128 or 256"; return CFD3D_ERR_ARG; }
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (c.mixed) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_tile<true>, 32, TILE_SMEM);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_df<true>, SW_CH, 0);
  if (shapes[2] < 1 || shapes[2] > std::max(per, 1)) { E.err = "sweep CTAs per SM outside 1 .. the occupancy limit"; return CFD3D_ERR_ARG; }
  const int nb = (int)E.blk.size();
  if (shapes[3] < 1 || shapes[3] > std::min(nb, Engine::MAX_PIPE) || (!c.mixed && shapes[3] != 1)) {
    E.err = "pipeline groups outside 1 .. min(blocks, 16) (1 in the FP64 form)";
    return CFD3D_ERR_ARG;
  }
  E.tpb_face = shapes[0];
  E.tpb_rhs = shapes[1];
  const int nwork = c.mixed ? E.d.ntile : E.d.nchunk;
  if (!E.sweep_planes) E.sweep_grid = std::max(1, std::min(shapes[2] * nsm, nwork));
  E.pipe_groups = shapes[3];
  E.graph_ready = 0;
  return CFD3D_OK;
}

int cfd3d_stats(const cfd3d_handle* h, int64_t* snd2_fallbacks, int* launches_per_iter) {
  if (!h) return CFD3D_ERR_ARG;
  const Engine& E = h->E;
  Scalars s;
  if (cudaMemcpy(&s, E.d.sc, sizeof(Scalars), cudaMemcpyDeviceToHost) != cudaSuccess) return CFD3D_ERR_CUDA;
  if (snd2_fallbacks) *snd2_fallbacks = (int64_t)s.snd2_fallbacks;
  if (launches_per_iter) *launches_per_iter = E.launches_per_iter;
  return CFD3D_OK;
}

}  // extern "C"
