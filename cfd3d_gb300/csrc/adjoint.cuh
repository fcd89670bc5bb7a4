// adjoint.cuh -- shared part of the discrete adjoint's translation units (adjoint.cu,
// adjoint_face.cu): gradient planes, the EOS Jacobian and chain, dual seeds, the
// reconstruction's clip decisions and the face-gradient stencil coefficients.  Device
// helpers have internal linkage: each unit carries its own copy.
#pragma once
#include "engine.cuh"
#include "dual.cuh"

namespace cfd {

// gdt planes: dv(1), dv(2), dv(6), dv(12), dv(3), dv(4), dv(5), tv(1), tv(2), tv(3) in the
// reference's 1-based numbering
enum { GD_RHO = 0, GD_H, GD_C2, GD_CP, GD_RL, GD_RV, GD_RG, GD_VIS, GD_CON, GD_MUT, NGD };
constexpr int NGD_DV = 7;   // the planes that are dv entries
static __constant__ int kGdDv[NGD_DV] = {0, 1, 5, 11, 2, 3, 4};   // their dv slots

struct AdjPtr {
  const double* lam;   // padded cotangent (npv x ncell), zero outside the interior
  double* gpv;         // padded gradient (npv x ncell)
  double* gdt;         // padded gradient of dv / tv entries (NGD x ncell)
  double* gpar;        // 3 parameter gradients
};

__device__ __forceinline__ void aadd(double* a, double v) {
  if (v != 0.0) atomicAdd(a, v);
}

// mixture rho, h, c2 at (p_abs, T, y1, y2) and their derivatives, by Dual<4>
struct EosJac { double rho, h, c2, drho[4], dh[4], dc2[4]; };
static __device__ __noinline__ EosJac eos_jac(int fluid, double p, double t, double y1, double y2) {
  using D4 = Dual<4>;
  D4 dv[NDV];
  deteos_t<D4>(fluid, 0, D4::seed(p, 0), D4::seed(t, 1), D4::seed(y1, 2), D4::seed(y2, 3), dv, nullptr);
  EosJac j;
  j.rho = dv[0].v; j.h = dv[1].v; j.c2 = dv[5].v;
  for (int m = 0; m < 4; ++m) { j.drho[m] = dv[0].d[m]; j.dh[m] = dv[1].d[m]; j.dc2[m] = dv[5].d[m]; }
  return j;
}

// a cell's dv / tv gradient gd (NGD planes) through eos%deteos to (p, T, y1, y2): ge[4]
static __device__ __noinline__ void eos_chain(const Par& c, double p, double t, double y1, double y2, const double* gd,
                                       double* ge) {
  using D4 = Dual<4>;
  D4 dv[NDV], tv[3];
  deteos_t<D4>(c.fluid, c.with_prop, D4::seed(p, 0), D4::seed(t, 1), D4::seed(y1, 2), D4::seed(y2, 3), dv, tv);
  for (int m = 0; m < 4; ++m) {
    double s = 0.0;
    for (int q = 0; q < NGD_DV; ++q) s += gd[q] * dv[kGdDv[q]].d[m];
    if (c.with_prop) s += gd[GD_VIS] * tv[0].d[m] + gd[GD_CON] * tv[1].d[m];
    ge[m] = s;
  }
}

// ------------------------------------------------------------------ seeds
// Local Jacobians are taken DC seed directions at a time (a few passes of the same code
// on Dual<DC>), which keeps the per-thread dual arrays small.
constexpr int DC = 8;
using DD = Dual<DC>;
__device__ __forceinline__ DD seed(double v, int i, int k0) {
  DD r(v);
  if (i >= k0 && i < k0 + DC) r.d[i - k0] = 1.0;
  return r;
}

// the reconstruction clips of muscl_clip (src/muscl_module.f90:136-158) on values, recording
// per variable whether the state was kept (0), reset to its cell value (1) or clamped to a
// constant (2) -- the derivative of a clipped state follows from the flag
__device__ __forceinline__ void clip_flags(const Par& c, const double* c9, const double* c10, double* xl, double* xr,
                                           int* fl, int* fr) {
  for (int k = 0; k < NPVM; ++k) fl[k] = fr[k] = 0;
  const double pmin = -c.pref + 10.0;
  if (xl[0] < pmin) { xl[0] = pmin; fl[0] = 2; }
  if (xr[0] < pmin) { xr[0] = pmin; fr[0] = 2; }
  for (int k = 5; k <= 6; ++k) {
    if (xl[k] < 0.0 || xl[k] > 1.0) { xl[k] = c9[k]; fl[k] = 1; }
    if (xr[k] < 0.0 || xr[k] > 1.0) { xr[k] = c10[k]; fr[k] = 1; }
  }
  if (xl[5] + xl[6] > 1.0) { xl[5] = c9[5]; xl[6] = c9[6]; fl[5] = fl[6] = 1; }
  if (xr[5] + xr[6] > 1.0) { xr[5] = c10[5]; xr[6] = c10[6]; fr[5] = fr[6] = 1; }
  if (c.npv > 7) {
    for (int k = 7; k <= 8; ++k) {
      if (xl[k] < 0.0 && c9[k] > 0.0) { xl[k] = c9[k]; fl[k] = 1; }
      if (xr[k] < 0.0 && c10[k] > 0.0) { xr[k] = c10[k]; fr[k] = 1; }
    }
  }
}

// coefficients of the face-gradient stencil (face_gradient): d/dx_l of the normal
// difference, the two transverse sums, and the face average
__device__ __forceinline__ void grad_coeffs(int l, double& cn, double& ce, double& ct, double& cc) {
  const double ce_t[18] = {-1, -1, 0, 0, 1, 1, -2, -2, 0, 0, 2, 2, -1, -1, 0, 0, 1, 1};
  const double ct_t[18] = {-1, -1, -2, -2, -1, -1, 0, 0, 0, 0, 0, 0, 1, 1, 2, 2, 1, 1};
  cn = (l == 9) ? 1.0 : ((l == 8) ? -1.0 : 0.0);
  ce = 0.0625 * ce_t[l];
  ct = 0.0625 * ct_t[l];
  cc = (l == 8 || l == 9) ? 0.5 : 0.0;
}

// the stencil cells that MUSCL reads (MLP reads all 38)
static __constant__ int kMusclCells[6] = {8, 9, 22, 31, 36, 37};


// the face VJP, one launch per direction (adjoint_face.cu)
void launch_adj_face(const Engine& E, const AdjPtr& a, cudaStream_t s);

}  // namespace cfd
