// adjoint.cu -- discrete adjoint (vector-Jacobian product) of the FP64 residual.
//
// R(pv) is the residual of cfd3d_residual (bc%setbc + rhs%calrhs, src/rhs_module.f90:260-643)
// as a function of the interior primitive state pv, with every interior cell's dv and
// tv(1:2) given by the EOS of its pv (as the update and the initialisation set them) and
// the eddy viscosity tv(3) and the dual-time history qq held as stored.  For a cotangent
// lambda on the interior residual, cfd3d_residual_vjp returns
//   g_pv  = (dR/dpv)^T lambda          for every interior cell and variable;
//   g_par = (dR/dtheta)^T lambda,      theta = (uref at fixed aoa / aos / k_inf / omega_inf,
//                                      c_v, c_c).
//
// Structure (the forward data flow reversed; nothing is stored by the forward pass: the
// limiter, clip, upwind and branch switches are recomputed from the state):
//   k_ghost x3        the forward boundary program, so the ghost cells hold the values the
//                     residual saw;
//   k_adj_face x3     per face (adjoint_face.cu): the local Jacobian of the inviscid and viscous flux with
//                     respect to its stencil, by forward-mode dual numbers over the same
//                     templated routines as the forward kernels (reconstruction per variable,
//                     face EOS by its derivatives, flux core, viscous core);
//   k_adj_cell        per cell: cavitation, SST and dual-time sources;
//   k_adj_ghost x3    the boundary program in reverse phase order (corners, edges, faces and
//                     halos): each ghost's gradient pushed to the cells it was made from;
//   k_adj_eos         per interior cell: the gradient with respect to its dv / tv pushed
//                     through the EOS to (p, T, y1, y2).
// Gradients accumulate with atomics in padded SoA arrays: gpv (npv planes) and gdt (the dv
// / tv entries that reach the residual, NGD planes).
#include "adjoint.cuh"

namespace cfd {

// ------------------------------------------------------------------ cell sources
// Per interior cell: the cavitation source (res(6)), the SST sources (res(8:9)) and the
// dual-time source, as k_rhs adds them (src/rhs_module.f90:540-642).
__global__ void __launch_bounds__(64) k_adj_cell(DevPtr d, Par c, AdjPtr a) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double wp[3] = {0.0, 0.0, 0.0};
  if (t < d.nint) {
    const int b = find_block_interior(d.blk, d.nblk, t);
    int i, j, k;
    const BlockGeom& B = d.blk[b];
    const long long g = interior_cell(B, t - B.int_off, i, j, k);
    const long long n = d.ncell, sj = B.ni, sk = (long long)B.ni * B.nj;
    const int npv = c.npv;
    double lam[NPVM], pv2[NPVM], dv[NDV];
    for (int v = 0; v < NPVM; ++v) {
      lam[v] = (v < npv) ? a.lam[v * n + g] : 0.0;
      pv2[v] = (v < npv) ? d.pv[v * n + g] : 0.0;
    }
    for (int v = 0; v < NDV; ++v) dv[v] = d.dv[v * n + g];
    const double vol = d.gm[GM_GRD * n + g];
    double gp[NPVM], gd[NGD];
    for (int v = 0; v < NPVM; ++v) gp[v] = 0.0;
    for (int m = 0; m < NGD; ++m) gd[m] = 0.0;
    // ---- cavitation: res(6) += r_v - r_c; seeds p, T, y1, y2, rho, rho_l, rho_v, rho_g (Kunz's
    // gas volume fraction), uref, c_v, c_c
    if (c.ncav && lam[5] != 0.0) {
      const int pvs[4] = {0, 4, 5, 6};
      const int dvs[4] = {0, 2, 3, 4};
      double w[11];
      for (int k0 = 0; k0 < 11; k0 += DC) {
        DD p2[NPVM], dd[NDV];
        for (int v = 0; v < NPVM; ++v) p2[v] = DD(pv2[v]);
        for (int q = 0; q < NDV; ++q) dd[q] = DD(dv[q]);
        for (int m = 0; m < 4; ++m) p2[pvs[m]] = seed(pv2[pvs[m]], m, k0);
        for (int m = 0; m < 4; ++m) dd[dvs[m]] = seed(dv[dvs[m]], 4 + m, k0);
        const CavOutT<DD> o = cavsource_t<DD>(c, p2, dd, vol, seed(c.uref, 8, k0), seed(c.c_v, 9, k0),
                                              seed(c.c_c, 10, k0));
        for (int q = 0; q < DC && k0 + q < 11; ++q) w[k0 + q] = lam[5] * (o.r_v.d[q] - o.r_c.d[q]);
      }
      for (int m = 0; m < 4; ++m) gp[pvs[m]] += w[m];
      gd[GD_RHO] += w[4]; gd[GD_RL] += w[5]; gd[GD_RV] += w[6]; gd[GD_RG] += w[7];
      wp[0] += w[8]; wp[1] += w[9]; wp[2] += w[10];
    }
    // ---- SST: res(8) += r7, res(9) += r8; seeds the 15 cell gradients, k, omega, rho, mu, mu_t
    if (c.iturb == 0 && (lam[7] != 0.0 || lam[8] != 0.0)) {
      const long long nbr[6] = {g - 1, g + 1, g - sj, g + sj, g - sk, g + sk};
      double fa[6][3];
      for (int q = 0; q < 3; ++q) {
        fa[0][q] = d.gm[(GM_CX + q) * n + g - 1]; fa[1][q] = d.gm[(GM_CX + q) * n + g];
        fa[2][q] = d.gm[(GM_EX + q) * n + g - sj]; fa[3][q] = d.gm[(GM_EX + q) * n + g];
        fa[4][q] = d.gm[(GM_TX + q) * n + g - sk]; fa[5][q] = d.gm[(GM_TX + q) * n + g];
      }
      const int gv[5] = {1, 2, 3, 7, 8};
      double grv[5][3];
      const double ivol = 1.0 / vol;
      for (int q = 0; q < 5; ++q) {
        const double* P = d.pv + gv[q] * n;
        const double c0 = P[g];
        const double v1 = 0.5 * (P[nbr[0]] + c0), v2 = 0.5 * (P[nbr[1]] + c0), v3 = 0.5 * (P[nbr[2]] + c0);
        const double v4 = 0.5 * (P[nbr[3]] + c0), v5 = 0.5 * (P[nbr[4]] + c0), v6 = 0.5 * (P[nbr[5]] + c0);
        for (int e = 0; e < 3; ++e)
          grv[q][e] = (v2 * fa[1][e] + v4 * fa[3][e] + v6 * fa[5][e] - v1 * fa[0][e] - v3 * fa[2][e] - v5 * fa[4][e]) * ivol;
      }
      const double mu = d.tv[g], mut = d.tv[2 * n + g];
      const double y5 = d.gm[(GM_GRD + 4) * n + g];
      double w[20];
      const double hmax = c.ides ? grid_hmax<double>(fa, vol) : 0.0;
      for (int k0 = 0; k0 < 20; k0 += DC) {
        DD gr[5][3];
        for (int q = 0; q < 5; ++q)
          for (int e = 0; e < 3; ++e) gr[q][e] = seed(grv[q][e], 3 * q + e, k0);
        const SstOut<DD> so = sst_source<DD>(gr, seed(pv2[7], 15, k0), seed(pv2[8], 16, k0), seed(dv[0], 17, k0),
                                             seed(mu, 18, k0), seed(mut, 19, k0), y5, vol, c.ides, hmax);
        for (int q = 0; q < DC && k0 + q < 20; ++q) w[k0 + q] = lam[7] * so.r7.d[q] + lam[8] * so.r8.d[q];
      }
      // the cell gradients are linear in the face averages 0.5 (P[nbr] + P[g])
      const double sgn[6] = {-1.0, 1.0, -1.0, 1.0, -1.0, 1.0};
      for (int q = 0; q < 5; ++q) {
        double gc = 0.0;
        for (int m = 0; m < 6; ++m) {
          double s = 0.0;
          for (int e = 0; e < 3; ++e) s += w[3 * q + e] * fa[m][e];
          s *= 0.5 * sgn[m] * ivol;
          gc += s;
          aadd(&a.gpv[gv[q] * n + nbr[m]], s);
        }
        gp[gv[q]] += gc;
      }
      gp[7] += w[15]; gp[8] += w[16];
      gd[GD_RHO] += w[17]; gd[GD_VIS] += w[18]; gd[GD_MUT] += w[19];
    }
    // ---- dual-time source: res -= (nsteady bb Q(pv, dv) - history) vol / dt_phy
    if (c.nsteady >= 1) {
      const double bb = (c.nsteady == 1) ? 1.0 : 0.75;
      const double cst = (double)c.nsteady * bb * vol / c.dt_phy;
      double mu_[NPVM];
      for (int v = 0; v < NPVM; ++v) mu_[v] = -cst * lam[v];
      const double r = dv[0], h = dv[1], u1 = pv2[1], u2 = pv2[2], u3 = pv2[3];
      double grho = mu_[0] + mu_[1] * u1 + mu_[2] * u2 + mu_[3] * u3 + mu_[4] * (h + 0.5 * (u1 * u1 + u2 * u2 + u3 * u3));
      for (int v = 5; v < npv; ++v) { grho += mu_[v] * pv2[v]; gp[v] += mu_[v] * r; }
      gp[1] += mu_[1] * r + mu_[4] * r * u1;
      gp[2] += mu_[2] * r + mu_[4] * r * u2;
      gp[3] += mu_[3] * r + mu_[4] * r * u3;
      gp[0] -= mu_[4];
      gd[GD_RHO] += grho;
      gd[GD_H] += mu_[4] * r;
    }
    // ---- gravity: res(2:4) += rho vol a, res(5) += rho vol (a . u)
    if (c.gravity) {
      double ga[3];
      gravity_at(d.grav, bc_time(d, c), ga);
      const double au = ga[0] * pv2[1] + ga[1] * pv2[2] + ga[2] * pv2[3];
      gd[GD_RHO] += vol * (lam[1] * ga[0] + lam[2] * ga[1] + lam[3] * ga[2] + lam[4] * au);
      for (int e = 0; e < 3; ++e) gp[1 + e] += lam[4] * dv[0] * vol * ga[e];
    }
    for (int v = 0; v < npv; ++v) aadd(&a.gpv[v * n + g], gp[v]);
    for (int m = 0; m < NGD; ++m) aadd(&a.gdt[m * n + g], gd[m]);
  }
  for (int q = 0; q < 3; ++q) {
    double s = wp[q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) aadd(&a.gpar[q], s);
  }
}

// ------------------------------------------------------------------ boundary program
// One ghost operation of k_ghost reversed.  Its destination's gradient is taken and
// cleared (the ghost value it overwrote reached nothing), then pushed to the cells the
// operation read.  Within a phase no operation reads another one's destination, so the
// phases run in reverse order (2, 1, 0) with the operations of a phase in parallel.
__device__ __forceinline__ void push_cell(const AdjPtr& a, const Par& c, long long n, long long q, const double* gp,
                                          const double* gd) {
  for (int v = 0; v < c.npv; ++v) aadd(&a.gpv[v * n + q], gp[v]);
  for (int m = 0; m < NGD; ++m) aadd(&a.gdt[m * n + q], gd[m]);
}

__global__ void k_adj_ghost(DevPtr d, Par c, AdjPtr a, const GhostOp* __restrict__ ops, int nops) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  double wu = 0.0;
  if (q < nops) {
    const GhostOp op = ops[q];
    const long long n = d.ncell;
    const int npv = c.npv;
    double gp[NPVM], gd[NGD];
    bool any = false;
    for (int v = 0; v < NPVM; ++v) {
      gp[v] = 0.0;
      if (v < npv) { gp[v] = a.gpv[v * n + op.dst]; a.gpv[v * n + op.dst] = 0.0; }
      any = any || gp[v] != 0.0;
    }
    for (int m = 0; m < NGD; ++m) {
      gd[m] = a.gdt[m * n + op.dst];
      a.gdt[m * n + op.dst] = 0.0;
      any = any || gd[m] != 0.0;
    }
    if (any) {
      const long long src = op.src;
      switch (op.kind) {
        case G_COPY:
        case G_EXTRAP:
          push_cell(a, c, n, src, gp, gd);
          break;
        case G_WALL_VISCOUS:
        case G_CRWALL:   // (the grid velocity is no function of the state)
          gp[1] = -gp[1]; gp[2] = -gp[2]; gp[3] = -gp[3];
          push_cell(a, c, n, src, gp, gd);
          break;
        case G_WALL_KW: {
          // omega_ghost = 1600 mu_b / rho_b / y5^2 - omega_src
          const double vis_b = d.tv[op.bnd], rho_b = d.dv[op.bnd], y5 = d.gm[(GM_GRD + 4) * n + op.bnd];
          const double kw = 1600.0 / (y5 * y5);
          aadd(&a.gdt[GD_VIS * n + op.bnd], gp[8] * kw / rho_b);
          aadd(&a.gdt[GD_RHO * n + op.bnd], -gp[8] * kw * vis_b / (rho_b * rho_b));
          gp[1] = -gp[1]; gp[2] = -gp[2]; gp[3] = -gp[3]; gp[7] = -gp[7]; gp[8] = -gp[8];
          gd[GD_MUT] = -gd[GD_MUT];
          push_cell(a, c, n, src, gp, gd);
          break;
        }
        case G_HFWALL_KW: {
          // T_g = 2 ((q y_b + mu_b |u_b|^2 / 2) / k_b + T_b) - T_src,
          // omega_g = 1600 mu_b / (rho_b y_b^2) - omega_src; u, v, w, k, mu_t reflected
          const long long b = op.bnd;
          const double hf = heatflux_at(d.hft + op.pad, bc_time(d, c));
          const double yb = d.gm[(GM_GRD + 4) * n + b], mub = d.tv[b], kb = d.tv[n + b], rb = d.dv[b];
          const double ub[3] = {d.pv[n + b], d.pv[2 * n + b], d.pv[3 * n + b]};
          const double u2 = ub[0] * ub[0] + ub[1] * ub[1] + ub[2] * ub[2];
          const double gt = gp[4], go = gp[8];
          aadd(&a.gpv[4 * n + b], 2.0 * gt);
          for (int e = 0; e < 3; ++e) aadd(&a.gpv[(1 + e) * n + b], gt * 2.0 * mub * ub[e] / kb);
          aadd(&a.gdt[GD_VIS * n + b], gt * u2 / kb + go * 1600.0 / (rb * yb * yb));
          aadd(&a.gdt[GD_CON * n + b], -gt * 2.0 * (hf * yb + 0.5 * mub * u2) / (kb * kb));
          aadd(&a.gdt[GD_RHO * n + b], -go * 1600.0 * mub / (rb * rb * yb * yb));
          gp[1] = -gp[1]; gp[2] = -gp[2]; gp[3] = -gp[3]; gp[4] = -gp[4]; gp[7] = -gp[7]; gp[8] = -gp[8];
          gd[GD_MUT] = -gd[GD_MUT];
          push_cell(a, c, n, src, gp, gd);
          break;
        }
        case G_CRWALL_KW:
          // u, v, w, k and mu_t reflected, omega and the rest the source cell's
          gp[1] = -gp[1]; gp[2] = -gp[2]; gp[3] = -gp[3]; gp[7] = -gp[7];
          gd[GD_MUT] = -gd[GD_MUT];
          push_cell(a, c, n, src, gp, gd);
          break;
        case G_MASSFLOW_IN: {
          // ghost pv: p = p_src, u = -u_src, T.. = 2 ref - src (y1, y2 clipped); dv and
          // tv(1:2) its EOS, tv(3) the source cell's
          double sp[NPVM], xp[NPVM];
          for (int v = 0; v < NPVM; ++v) sp[v] = (v < npv) ? d.pv[v * n + src] : 0.0;
          const double bpv[NPVM] = {c.pref, c.uref_vec[0], c.uref_vec[1], c.uref_vec[2], c.tref, c.y1ref, c.y2ref,
                                    c.kref, c.oref};
          for (int v = 0; v < NPVM; ++v) xp[v] = sp[v];
          for (int v = 1; v < 4; ++v) xp[v] = -sp[v];
          for (int v = 4; v < npv; ++v) xp[v] = 2.0 * bpv[v] - sp[v];
          const bool c5 = xp[5] > 0.0 && xp[5] < 1.0, c6 = xp[6] > 0.0 && xp[6] < 1.0;
          xp[5] = ::fmin(::fmax(xp[5], 0.0), 1.0);
          xp[6] = ::fmin(::fmax(xp[6], 0.0), 1.0);
          double ge[4];
          eos_chain(c, xp[0] + bpv[0], xp[4], xp[5], xp[6], gd, ge);
          gp[0] += ge[0]; gp[4] += ge[1]; gp[5] += ge[2]; gp[6] += ge[3];
          aadd(&a.gdt[GD_MUT * n + src], gd[GD_MUT]);
          if (!c.with_prop) { aadd(&a.gdt[GD_VIS * n + src], gd[GD_VIS]); aadd(&a.gdt[GD_CON * n + src], gd[GD_CON]); }
          // d(ghost pv)/d(source pv): 1 for p, -1 for the rest (0 where a clip is active)
          aadd(&a.gpv[src], gp[0]);
          for (int v = 1; v < npv; ++v) {
            double s = -gp[v];
            if ((v == 5 && !c5) || (v == 6 && !c6)) s = 0.0;
            aadd(&a.gpv[v * n + src], s);
          }
          break;
        }
        case G_SYMMETRY:
        case G_CRWALL_INV: {
          // u_ghost = 2 (u_b - n (u_b . n) / |n|^2 [- gridvel]) - u_src
          double nx[3];
          face_vec(d, op.fplane, op.fidx, nx);
          for (int v = 0; v < 3; ++v) nx[v] *= (double)op.fsign;
          const double nn = nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2];
          for (int jx = 0; jx < 3; ++jx) {
            double s = 0.0;
            for (int ix = 0; ix < 3; ++ix) s += gp[1 + ix] * 2.0 * ((ix == jx ? 1.0 : 0.0) - nx[ix] * nx[jx] / nn);
            aadd(&a.gpv[(1 + jx) * n + op.bnd], s);
          }
          gp[1] = -gp[1]; gp[2] = -gp[2]; gp[3] = -gp[3];
          push_cell(a, c, n, src, gp, gd);
          break;
        }
        case G_FARFIELD:
        case G_INFLOW_SUB:
        case G_OUTFLOW_SUB:
        case G_INFLOW_SUP: {
          const int ffm = ghost_ff_mode(op.kind);
          double nx[3];
          face_vec(d, op.fplane, op.fidx, nx);
          for (int v = 0; v < 3; ++v) nx[v] *= (double)op.fsign;
          const double dl = 1.0 / ::sqrt(nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2]);
          double sp[NPVM], pb[4], xp[NPVM], bpv[NPVM];
          for (int v = 0; v < NPVM; ++v) sp[v] = (v < npv) ? d.pv[v * n + src] : 0.0;
          for (int m = 0; m < 4; ++m) pb[m] = d.pv[m * n + op.bnd];
          const double rb = d.dv[op.bnd], c2b = d.dv[5 * n + op.bnd];
          bpv[0] = c.pref; bpv[1] = c.uref_vec[0]; bpv[2] = c.uref_vec[1]; bpv[3] = c.uref_vec[2];
          bpv[4] = c.tref; bpv[5] = c.y1ref; bpv[6] = c.y2ref; bpv[7] = c.kref; bpv[8] = c.oref;
          for (int v = 0; v < NPVM; ++v) xp[v] = sp[v];
          farfield_pv<double>(c, nx, dl, pb, rb, c2b, bpv, c.uref * c.uref, xp, ffm);
          // the ghost's dv and tv(1:2) are its EOS; tv(3) (and tv(1:2) without transport
          // properties) is the mirror cell's
          double ge[4];
          eos_chain(c, xp[0] + bpv[0], xp[4], xp[5], xp[6], gd, ge);
          gp[0] += ge[0]; gp[4] += ge[1]; gp[5] += ge[2]; gp[6] += ge[3];
          aadd(&a.gdt[GD_MUT * n + src], gd[GD_MUT]);
          if (!c.with_prop) { aadd(&a.gdt[GD_VIS * n + src], gd[GD_VIS]); aadd(&a.gdt[GD_CON * n + src], gd[GD_CON]); }
          // the ghost pv: seeds mirror pv 0..8, boundary p, u, v, w 9..12, rho_b 13, c2_b 14, uref 15
          double w[16];
          for (int k0 = 0; k0 < 16; k0 += DC) {
            DD x[NPVM], pbd[4], bp[NPVM];
            for (int v = 0; v < NPVM; ++v) x[v] = seed(sp[v], v, k0);
            for (int m = 0; m < 4; ++m) pbd[m] = seed(pb[m], 9 + m, k0);
            const DD ur = seed(c.uref, 15, k0);
            for (int v = 0; v < NPVM; ++v) bp[v] = DD(bpv[v]);
            if (c.uref != 0.0 && 15 >= k0 && 15 < k0 + DC)
              for (int e = 0; e < 3; ++e) bp[1 + e].d[15 - k0] = c.uref_vec[e] / c.uref;
            farfield_pv<DD>(c, nx, dl, pbd, seed(rb, 13, k0), seed(c2b, 14, k0), bp, ur * ur, x, ffm);
            for (int qq = 0; qq < DC && k0 + qq < 16; ++qq) {
              double s = 0.0;
              for (int v = 0; v < npv; ++v) s += gp[v] * x[v].d[qq];
              w[k0 + qq] = s;
            }
          }
          for (int v = 0; v < npv; ++v) aadd(&a.gpv[v * n + src], w[v]);
          for (int m = 0; m < 4; ++m) aadd(&a.gpv[m * n + op.bnd], w[9 + m]);
          aadd(&a.gdt[GD_RHO * n + op.bnd], w[13]);
          aadd(&a.gdt[GD_C2 * n + op.bnd], w[14]);
          wu += w[15];
          break;
        }
        case G_WALLWALL:
        case G_WALLWALL_KW4:
        case G_WALLWALL_KW8: {
          // modified entries: -(src + sum of neighbours); the rest are the source cell's
          bool mod[NPVM];
          for (int v = 0; v < NPVM; ++v) mod[v] = (v >= 1 && v <= 3);
          if (op.kind != G_WALLWALL || npv > 7) { mod[7] = true; mod[8] = true; }
          if (op.kind != G_WALLWALL) {
            // omega_ghost = K 800 mu_src / rho_src / y5^2 + ppv(8)
            const double y5 = d.gm[(GM_GRD + 4) * n + src];
            const double kw = ((op.kind == G_WALLWALL_KW8) ? 8.0 : 4.0) * 800.0 / (y5 * y5);
            const double mu_s = d.tv[src], rho_s = d.dv[src];
            gd[GD_VIS] += gp[8] * kw / rho_s;
            gd[GD_RHO] -= gp[8] * kw * mu_s / (rho_s * rho_s);
          }
          double gs[NPVM];
          for (int v = 0; v < NPVM; ++v) gs[v] = mod[v] ? -gp[v] : gp[v];
          push_cell(a, c, n, src, gs, gd);
          for (int m = 0; m < 6; ++m) {
            if (op.nb[m] < 0) break;
            for (int v = 0; v < npv; ++v)
              if (mod[v]) aadd(&a.gpv[v * n + op.nb[m]], -gp[v]);
          }
          break;
        }
        case G_NOWALL3:
        case G_NOWALL7: {
          // the ghost is the mean of the source cell and its neighbours, then its EOS
          const double f = (op.kind == G_NOWALL7) ? 1.0 / 7.0 : 1.0 / 3.0;
          double sum[NPVM];
          for (int v = 0; v < NPVM; ++v) sum[v] = (v < npv) ? d.pv[v * n + src] : 0.0;
          for (int m = 0; m < 6; ++m) {
            if (op.nb[m] < 0) break;
            for (int v = 0; v < npv; ++v) sum[v] += d.pv[v * n + op.nb[m]];
          }
          double xp[NPVM];
          for (int v = 0; v < NPVM; ++v) xp[v] = f * sum[v];
          double ge[4];
          eos_chain(c, xp[0] + c.pref, xp[4], xp[5], xp[6], gd, ge);
          gp[0] += ge[0]; gp[4] += ge[1]; gp[5] += ge[2]; gp[6] += ge[3];
          double gt[NGD];
          for (int m = 0; m < NGD; ++m) gt[m] = 0.0;
          gt[GD_MUT] = f * gd[GD_MUT];
          if (!c.with_prop) { gt[GD_VIS] = f * gd[GD_VIS]; gt[GD_CON] = f * gd[GD_CON]; }
          double gs[NPVM];
          for (int v = 0; v < NPVM; ++v) gs[v] = f * gp[v];
          push_cell(a, c, n, src, gs, gt);
          for (int m = 0; m < 6; ++m) {
            if (op.nb[m] < 0) break;
            push_cell(a, c, n, op.nb[m], gs, gt);
          }
          break;
        }
        default:
          break;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) wu += __shfl_down_sync(0xffffffffu, wu, o);
  if ((threadIdx.x & 31) == 0) aadd(&a.gpar[0], wu);
}

// ------------------------------------------------------------------ interior EOS
// dv and tv(1:2) of an interior cell are its EOS: their gradient goes to (p, T, y1, y2)
__global__ void k_adj_eos(DevPtr d, Par c, AdjPtr a) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= d.nint) return;
  const int b = find_block_interior(d.blk, d.nblk, t);
  int i, j, k;
  const long long g = interior_cell(d.blk[b], t - d.blk[b].int_off, i, j, k);
  const long long n = d.ncell;
  double gd[NGD];
  bool any = false;
  for (int m = 0; m < NGD; ++m) {
    gd[m] = (m == GD_MUT) ? 0.0 : a.gdt[m * n + g];
    any = any || gd[m] != 0.0;
  }
  if (!any) return;
  double ge[4];
  eos_chain(c, d.pv[g] + c.pref, d.pv[4 * n + g], d.pv[5 * n + g], d.pv[6 * n + g], gd, ge);
  a.gpv[g] += ge[0];
  a.gpv[4 * n + g] += ge[1];
  a.gpv[5 * n + g] += ge[2];
  a.gpv[6 * n + g] += ge[3];
}

// ------------------------------------------------------------------ host side
namespace {
inline unsigned adj_blocks(long long n, int T) { return (unsigned)((n + T - 1) / T); }
}

int adjoint_buffers(Engine& E) {
  const size_t n = (size_t)E.ncell;
  const int npv = E.par.npv;
  if (!E.adj_lam) {
    if (cudaMalloc(&E.adj_lam, n * npv * 8) != cudaSuccess || cudaMalloc(&E.adj_gpv, n * npv * 8) != cudaSuccess ||
        cudaMalloc(&E.adj_gdt, n * NGD * 8) != cudaSuccess || cudaMalloc(&E.adj_gpar, 4 * 8) != cudaSuccess) {
      E.err = "device allocation failed (adjoint buffers)";
      return CFD3D_ERR_NOMEM;
    }
  }
  cudaMemsetAsync(E.adj_lam, 0, n * npv * 8, E.st);
  cudaMemsetAsync(E.adj_gpv, 0, n * npv * 8, E.st);
  cudaMemsetAsync(E.adj_gdt, 0, n * NGD * 8, E.st);
  cudaMemsetAsync(E.adj_gpar, 0, 4 * 8, E.st);
  return CFD3D_OK;
}

void adjoint_free(Engine& E) {
  cudaFree(E.adj_lam); cudaFree(E.adj_gpv); cudaFree(E.adj_gdt); cudaFree(E.adj_gpar);
  E.adj_lam = E.adj_gpv = E.adj_gdt = E.adj_gpar = nullptr;
}

// the reverse pass; the cotangent is in adj_lam and the ghost cells hold the values of the
// forward boundary program
int adjoint_launch(Engine& E) {
  const DevPtr& d = E.d;
  const Par& c = E.par;
  cudaStream_t s = E.st;
  const AdjPtr a{E.adj_lam, E.adj_gpv, E.adj_gdt, E.adj_gpar};
  launch_adj_face(E, a, s);
  k_adj_cell<<<adj_blocks(E.nint, 64), 64, 0, s>>>(d, c, a);
  for (int p = 2; p >= 0; --p)
    if (E.nops[p]) k_adj_ghost<<<adj_blocks(E.nops[p], 64), 64, 0, s>>>(d, c, a, E.d_ops[p], E.nops[p]);
  k_adj_eos<<<adj_blocks(E.nint, 64), 64, 0, s>>>(d, c, a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { E.err = std::string("adjoint launch: ") + cudaGetErrorString(e); return CFD3D_ERR_CUDA; }
  return CFD3D_OK;
}

}  // namespace cfd
