// setup.cu -- build-time work of the engine (runs once per cfd3d_create).
//
//  * grid metrics on the device: face area vectors, volumes, centroids (calnormal /
//    calvolume, src/grid_module.f90:609-1241), their ghost rows and the reference's metric
//    halos across 1-to-1 interfaces (:725-940, :1115-1212), from the node coordinates;
//  * wall distance (calydns, :350-607) as a two-pass brute-force GPU kernel: an FP32
//    pass finds each cell's nearest wall-face distance, an FP64 pass re-evaluates only
//    the faces within a relative margin of it, so the result equals the FP64 minimum;
//  * the boundary program: the reference's BC, 12 edge, 8 corner and halo descriptors
//    (src/bc_module.f90:71-1188) compiled into a flat list of ghost-cell operations in
//    three dependency phases (faces + halos, edges, corners);
//  * the LU-SGS hyperplane schedule: interior cells of all blocks grouped by
//    i + j + k, so each sweep stage is one launch over independent cells.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include "engine.cuh"

namespace cfd {

namespace {

struct Con {
  int donor;
  int s[3], e[3], sd[3], ed[3];
  int tm[3][3];
};

// ---- grid metrics on the device --------------------------------------------------------
// One block's node coordinates x(3, 2:imax+1, 2:jmax+1, 2:kmax+1), the reference's node
// range, as the block descriptor holds them.
struct NodeBlock {
  const double* x;
  int im, jm;
  __device__ double operator()(int v, int i, int j, int k) const {
    return x[v + 3 * ((i - 2) + (long long)im * ((j - 2) + (long long)jm * (k - 2)))];
  }
};
__device__ __forceinline__ long long gidx(const BlockGeom& G, int i, int j, int k) {
  return G.off + (i + 1) + (long long)G.ni * ((j + 1) + (long long)G.nj * (k + 1));
}
// (i, j, k) inside the block's padded box -1..imax+3 (a connection's mapped index must be)
__device__ __forceinline__ bool in_box(const BlockGeom& G, int i, int j, int k) {
  return i >= -1 && i < G.ni - 1 && j >= -1 && j < G.nj - 1 && k >= -1 && k < G.nk - 1;
}
// Products are rounded before they are summed (no multiply-add contraction), as the
// reference's evaluation order gives them; the metrics then equal the CPU restatement's.
__device__ __forceinline__ double mulr(double a, double b) { return __dmul_rn(a, b); }

__device__ double pyramid(const double* pa, const double* pb, const double* pc, const double* pd, const double* cen) {
  double cs[3], va[3], vb[3];
  for (int v = 0; v < 3; ++v) {
    cs[v] = 0.25 * (pa[v] + pb[v] + pc[v] + pd[v]);
    va[v] = pc[v] - pa[v];
    vb[v] = pd[v] - pb[v];
  }
  const double px = mulr(cen[0] - cs[0], mulr(va[1], vb[2]) - mulr(va[2], vb[1]));
  const double py = mulr(cen[1] - cs[1], mulr(va[2], vb[0]) - mulr(va[0], vb[2]));
  const double pz = mulr(cen[2] - cs[2], mulr(va[0], vb[1]) - mulr(va[1], vb[0]));
  return fabs(px + py + pz);
}

// Face area vectors of direction DIR (calnormal, src/grid_module.f90:609-724): half the
// cross product of the face's diagonals, for the face array's whole range -- cx over
// (1..im, 1..jm+1, 1..km+1), ex over (1..im+1, 1..jm, 1..km+1), tx over (1..im+1, 1..jm+1,
// 1..km).  The reference computes the faces of the interior rows and then copies them to
// the ghost rows along each transverse direction in turn; clamping the transverse index to
// the computed rows gives the same values.  A degenerate patch zeroes the whole plane of
// its face (:672-708), edges included, before those copies (zlo, zhi: first, last plane).
template <int DIR>
__global__ void k_geo_faces(BlockGeom G, NodeBlock X, double* __restrict__ gm, long long nc, int zlo, int zhi) {
  const int im = G.imax, jm = G.jmax, km = G.kmax;
  const int n0 = DIR == 0 ? im : im + 1, n1 = DIR == 1 ? jm : jm + 1, n2 = DIR == 2 ? km : km + 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)n0 * n1 * n2) return;
  const int i = (int)(t % n0) + 1;
  const long long r = t / n0;
  const int j = (int)(r % n1) + 1, k = (int)(r / n1) + 1;
  const int a = DIR == 0 ? i : min(max(i, 2), im);
  const int b = DIR == 1 ? j : min(max(j, 2), jm);
  const int c = DIR == 2 ? k : min(max(k, 2), km);
  double p[3], q[3];
  for (int v = 0; v < 3; ++v) {
    if (DIR == 0) { p[v] = X(v, a + 1, b + 1, c) - X(v, a + 1, b, c + 1); q[v] = X(v, a + 1, b + 1, c + 1) - X(v, a + 1, b, c); }
    else if (DIR == 1) { p[v] = X(v, a, b + 1, c) - X(v, a + 1, b + 1, c + 1); q[v] = X(v, a, b + 1, c + 1) - X(v, a + 1, b + 1, c); }
    else { p[v] = X(v, a + 1, b, c + 1) - X(v, a, b + 1, c + 1); q[v] = X(v, a + 1, b + 1, c + 1) - X(v, a, b, c + 1); }
  }
  const int fn = DIR == 0 ? i : (DIR == 1 ? j : k), fmax = DIR == 0 ? im : (DIR == 1 ? jm : km);
  const bool zero = (fn == 1 && zlo) || (fn == fmax && zhi);
  const long long g = gidx(G, i, j, k);
  const int plane = DIR == 0 ? GM_CX : (DIR == 1 ? GM_EX : GM_TX);
  gm[(plane + 0) * nc + g] = zero ? 0.0 : 0.5 * (mulr(p[1], q[2]) - mulr(q[1], p[2]));
  gm[(plane + 1) * nc + g] = zero ? 0.0 : 0.5 * (mulr(q[0], p[2]) - mulr(p[0], q[2]));
  gm[(plane + 2) * nc + g] = zero ? 0.0 : 0.5 * (mulr(p[0], q[1]) - mulr(q[0], p[1]));
}

// Centroid and volume of every interior cell (calvolume, src/grid_module.f90:942-1080):
// the mean of the eight nodes, and the six pyramids from the centroid to the faces.
__global__ void k_geo_cells(BlockGeom G, NodeBlock X, double* __restrict__ gm, long long nc) {
  const int ni = G.imax - 1, nj = G.jmax - 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)ni * nj * (G.kmax - 1)) return;
  const int i = (int)(t % ni) + 2;
  const long long r = t / ni;
  const int j = (int)(r % nj) + 2, k = (int)(r / nj) + 2;
  double cen[3];
  for (int v = 0; v < 3; ++v)
    cen[v] = 0.125 * (X(v, i, j, k) + X(v, i + 1, j, k) + X(v, i, j + 1, k) + X(v, i, j, k + 1) + X(v, i + 1, j + 1, k) +
                      X(v, i, j + 1, k + 1) + X(v, i + 1, j, k + 1) + X(v, i + 1, j + 1, k + 1));
  auto P = [&](int a, int b, int c, double* o) { for (int v = 0; v < 3; ++v) o[v] = X(v, a, b, c); };
  double pa[3], pb[3], pc[3], pd[3], s = 0.0;
  P(i, j, k, pa); P(i + 1, j, k, pb); P(i + 1, j + 1, k, pc); P(i, j + 1, k, pd); s += pyramid(pa, pb, pc, pd, cen);
  P(i, j, k + 1, pa); P(i + 1, j, k + 1, pb); P(i + 1, j + 1, k + 1, pc); P(i, j + 1, k + 1, pd); s += pyramid(pa, pb, pc, pd, cen);
  P(i, j, k, pa); P(i + 1, j, k, pb); P(i + 1, j, k + 1, pc); P(i, j, k + 1, pd); s += pyramid(pa, pb, pc, pd, cen);
  P(i, j + 1, k, pa); P(i + 1, j + 1, k, pb); P(i + 1, j + 1, k + 1, pc); P(i, j + 1, k + 1, pd); s += pyramid(pa, pb, pc, pd, cen);
  P(i, j, k, pa); P(i, j + 1, k, pb); P(i, j + 1, k + 1, pc); P(i, j, k + 1, pd); s += pyramid(pa, pb, pc, pd, cen);
  P(i + 1, j, k, pa); P(i + 1, j + 1, k, pb); P(i + 1, j + 1, k + 1, pc); P(i + 1, j, k + 1, pd); s += pyramid(pa, pb, pc, pd, cen);
  const long long g = gidx(G, i, j, k);
  gm[GM_GRD * nc + g] = s / 6.0;
  for (int v = 0; v < 3; ++v) gm[(GM_GRD + 1 + v) * nc + g] = cen[v];
}

// Ghost cells of the cell geometry (src/grid_module.f90:1082-1113 and the wall distance's
// :560-590), in the reference's three passes: step 0 the j ghosts of the interior rows,
// step 1 the i ghosts of every j, step 2 the k ghosts of every i and j.  The volume and the
// wall distance are copied; the centroid is extrapolated linearly, at k = 1 from the fixed
// cell (3, j, 3) as the reference does.  what: 0 volume and centroid, 1 wall distance.
__global__ void k_geo_ghosts(BlockGeom G, double* __restrict__ gm, long long nc, int step, int what) {
  const int im = G.imax, jm = G.jmax, km = G.kmax;
  const int na = step == 0 ? im - 1 : (step == 1 ? jm + 1 : im + 1);
  const int nb = step == 2 ? jm + 1 : km - 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int ta = (int)(t % na), tb = (int)(t / na);
  for (int side = 0; side < 2; ++side) {
    int i, j, k, i1, j1, k1, i2, j2, k2;   // ghost, nearest interior row, next row
    if (step == 0) {
      i = i1 = i2 = ta + 2; k = k1 = k2 = tb + 2;
      j = side ? jm + 1 : 1; j1 = side ? jm : 2; j2 = side ? jm - 1 : 3;
    } else if (step == 1) {
      j = j1 = j2 = ta + 1; k = k1 = k2 = tb + 2;
      i = side ? im + 1 : 1; i1 = side ? im : 2; i2 = side ? im - 1 : 3;
    } else {
      i = i1 = ta + 1; j = j1 = j2 = tb + 1;
      k = side ? km + 1 : 1; k1 = side ? km : 2;
      i2 = side ? i : 3; k2 = side ? km - 1 : 3;
    }
    const long long g = gidx(G, i, j, k), g1 = gidx(G, i1, j1, k1), g2 = gidx(G, i2, j2, k2);
    if (what == 1) {
      gm[(GM_GRD + 4) * nc + g] = gm[(GM_GRD + 4) * nc + g1];
    } else {
      gm[GM_GRD * nc + g] = gm[GM_GRD * nc + g1];
      for (int v = 1; v <= 3; ++v) gm[(GM_GRD + v) * nc + g] = 2.0 * gm[(GM_GRD + v) * nc + g1] - gm[(GM_GRD + v) * nc + g2];
    }
  }
}

// any interior volume that is not positive
__global__ void k_geo_check(BlockGeom G, const double* __restrict__ gm, long long nc, int* bad) {
  const int ni = G.imax - 1, nj = G.jmax - 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)ni * nj * (G.kmax - 1)) return;
  const int i = (int)(t % ni) + 2;
  const long long r = t / ni;
  const int j = (int)(r % nj) + 2, k = (int)(r / nj) + 2;
  if (!(gm[GM_GRD * nc + gidx(G, i, j, k)] > 0.0)) atomicExch(bad, 1);
}

__host__ __device__ inline void cmap(const Con& g, int i, int j, int k, int& ii, int& jj, int& kk) {
  ii = g.tm[0][0] * (i - g.s[0]) + g.tm[0][1] * (j - g.s[1]) + g.tm[0][2] * (k - g.s[2]) + g.sd[0];
  jj = g.tm[1][0] * (i - g.s[0]) + g.tm[1][1] * (j - g.s[1]) + g.tm[1][2] * (k - g.s[2]) + g.sd[1];
  kk = g.tm[2][0] * (i - g.s[0]) + g.tm[2][1] * (j - g.s[1]) + g.tm[2][2] * (k - g.s[2]) + g.sd[2];
}

bool read_cons(const cfd3d_block_desc& d, int nblocks, std::vector<Con>& out, std::string& err) {
  for (int n = 0; n < d.ncon; ++n) {
    const cfd3d_connection& c = d.con[n];
    if (c.donor < 0 || c.donor >= nblocks) { err = "connection donor out of range"; return false; }
    Con g{};
    g.donor = c.donor;
    for (int q = 0; q < 3; ++q) {
      int t = c.transform[q];
      if (t == 0 || std::abs(t) > 3) { err = "bad connection transform"; return false; }
      g.tm[std::abs(t) - 1][q] = t > 0 ? 1 : -1;
    }
    const int* p = c.pnts;
    const int* pd = c.pnts_donor;
    bool any = false, anyd = false;
    for (int m = 0; m < 3; ++m) {
      if (p[m] == p[3 + m]) {
        any = true;
        for (int q = 0; q < 3; ++q) { g.s[q] = p[q]; g.e[q] = p[3 + q]; }
        if (p[m] == 1) { g.s[m] = p[m] + 1; g.e[m] = p[3 + m] + 1; }
      }
      if (pd[m] == pd[3 + m]) {
        anyd = true;
        for (int q = 0; q < 3; ++q) { g.sd[q] = pd[q]; g.ed[q] = pd[3 + q]; }
        if (pd[m] != 1) { g.sd[m] = pd[m] + 1; g.ed[m] = pd[3 + m] + 1; }
      }
    }
    if (!any || !anyd) { err = "connection range is not a face"; return false; }
    out.push_back(g);
  }
  return true;
}

// Face-vector halo of one 1-to-1 connection (src/grid_module.f90:725-918), on the node-based
// ranges: the two face arrays tangential to the interface, from the block's own faces to
// the donor's ghost row, with the orientation signs s1, s2.
__global__ void k_geo_face_halo(Con g, BlockGeom S, BlockGeom D, int s1, int s2, double* __restrict__ gm, long long nc) {
  const int n0 = g.e[0] - g.s[0] + 1, n1 = g.e[1] - g.s[1] + 1, n2 = g.e[2] - g.s[2] + 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)n0 * n1 * n2) return;
  const int i = g.s[0] + (int)(t % n0);
  const long long r = t / n0;
  const int j = g.s[1] + (int)(r % n1), k = g.s[2] + (int)(r / n1);
  int ii, jj, kk;
  cmap(g, i, j, k, ii, jj, kk);
  if (!in_box(S, i, j, k) || !in_box(D, ii, jj, kk)) return;
  const long long gs = gidx(S, i, j, k), gd = gidx(D, ii, jj, kk);
  const int pa = (g.s[0] == g.e[0]) ? GM_EX : (g.s[1] == g.e[1]) ? GM_TX : GM_CX;
  const int pc = (g.s[0] == g.e[0]) ? GM_TX : (g.s[1] == g.e[1]) ? GM_CX : GM_EX;
  const int qa = (g.sd[0] == g.ed[0]) ? GM_EX : (g.sd[1] == g.ed[1]) ? GM_TX : GM_CX;
  const int qc = (g.sd[0] == g.ed[0]) ? GM_TX : (g.sd[1] == g.ed[1]) ? GM_CX : GM_EX;
  for (int m = 0; m < 3; ++m) {
    const double a = gm[(pa + m) * nc + gs], c = gm[(pc + m) * nc + gs];
    gm[(qa + m) * nc + gd] = s1 * a;
    gm[(qc + m) * nc + gd] = s2 * c;
  }
}

// Halo of one cell-geometry variable across one connection (cell ranges): the donor's
// ghost cell takes the block's interior value (src/grid_module.f90:1115-1212, 592-607).
__global__ void k_geo_exchange(Con g, BlockGeom S, BlockGeom D, int var, double* __restrict__ gm, long long nc) {
  const int n0 = g.e[0] - g.s[0] + 1, n1 = g.e[1] - g.s[1] + 1, n2 = g.e[2] - g.s[2] + 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)n0 * n1 * n2) return;
  const int i = g.s[0] + (int)(t % n0);
  const long long r = t / n0;
  const int j = g.s[1] + (int)(r % n1), k = g.s[2] + (int)(r / n1);
  int ii, jj, kk;
  cmap(g, i, j, k, ii, jj, kk);
  if (!in_box(S, i, j, k) || !in_box(D, ii, jj, kk)) return;
  gm[(GM_GRD + var) * nc + gidx(D, ii, jj, kk)] = gm[(GM_GRD + var) * nc + gidx(S, i, j, k)];
}

// ---- wall distance ------------------------------------------------------------------
// calydns (src/grid_module.f90:350-607): each interior cell's distance to the nearest
// wall-face centre, by brute force over all of them.  An FP32 pass finds the nearest
// squared distance; an FP64 pass re-evaluates only the faces within a relative margin of it,
// so the result is the FP64 minimum.  The cell centre is the centroid in gm.
__global__ void k_wall_distance(const BlockGeom* __restrict__ blk, int nblk, long long nint, double* __restrict__ gm,
                                long long nc, const double* __restrict__ wall, int nwall) {
  extern __shared__ float sw[];
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double cx = 0, cy = 0, cz = 0;
  long long g = -1;
  if (t < nint) {
    const int b = find_block_interior(blk, nblk, t);
    int i, j, k;
    g = interior_cell(blk[b], t - blk[b].int_off, i, j, k);
    cx = gm[(GM_GRD + 1) * nc + g]; cy = gm[(GM_GRD + 2) * nc + g]; cz = gm[(GM_GRD + 3) * nc + g];
  }
  float fx = (float)cx, fy = (float)cy, fz = (float)cz;
  float best = 3.0e38f;
  // pass 1: FP32 minimum of the squared distance
  for (int t0 = 0; t0 < nwall; t0 += blockDim.x) {
    __syncthreads();
    int q = t0 + threadIdx.x;
    if (q < nwall) { sw[3 * threadIdx.x] = (float)wall[3 * q]; sw[3 * threadIdx.x + 1] = (float)wall[3 * q + 1]; sw[3 * threadIdx.x + 2] = (float)wall[3 * q + 2]; }
    __syncthreads();
    int nt = min((int)blockDim.x, nwall - t0);
    for (int q2 = 0; q2 < nt; ++q2) {
      float dx = fx - sw[3 * q2], dy = fy - sw[3 * q2 + 1], dz = fz - sw[3 * q2 + 2];
      best = fminf(best, dx * dx + dy * dy + dz * dz);
    }
  }
  // pass 2: FP64 distance of every face within the FP32 rounding margin
  float thr = best * (1.0f + 1.0e-4f) + 1.0e-30f;
  double ymin = 1.0e6;
  for (int t0 = 0; t0 < nwall; t0 += blockDim.x) {
    __syncthreads();
    int q = t0 + threadIdx.x;
    if (q < nwall) { sw[3 * threadIdx.x] = (float)wall[3 * q]; sw[3 * threadIdx.x + 1] = (float)wall[3 * q + 1]; sw[3 * threadIdx.x + 2] = (float)wall[3 * q + 2]; }
    __syncthreads();
    int nt = min((int)blockDim.x, nwall - t0);
    for (int q2 = 0; q2 < nt; ++q2) {
      float dx = fx - sw[3 * q2], dy = fy - sw[3 * q2 + 1], dz = fz - sw[3 * q2 + 2];
      if (dx * dx + dy * dy + dz * dz <= thr) {
        const double* w = wall + 3 * (size_t)(t0 + q2);
        const double ex = cx - w[0], ey = cy - w[1], ez = cz - w[2];
        double yt = sqrt(mulr(ex, ex) + mulr(ey, ey) + mulr(ez, ez));
        if (yt < ymin) ymin = yt;
      }
    }
  }
  if (g >= 0) gm[(GM_GRD + 4) * nc + g] = ymin;
}

__global__ void k_scale(double* __restrict__ x, long long n, double s) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) x[t] = x[t] * s;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// The grid's metrics, computed on the device in the order of grid%construct: face vectors
// and their halo, the reordering of the connection ranges, volumes and centroids with
// their ghosts and halo, then the wall distance with its ghosts and halo.  The host holds
// only the node coordinates (uploaded once) and the wall-face centres.
bool setup_geometry(Engine& E, const cfd3d_block_desc* blocks, int nblocks) {
  const int ngrd = E.par.ngrd;
  const long long nc = E.ncell;
  double* gm = E.d.gm;
  const double scale = E.cfg.scale;
  std::vector<std::vector<Con>> cons(nblocks);
  std::vector<long long> xoff(nblocks + 1, 0);
  for (int b = 0; b < nblocks; ++b) {
    if (!read_cons(blocks[b], nblocks, cons[b], E.err)) return false;
    xoff[b + 1] = xoff[b] + 3ll * blocks[b].imax * blocks[b].jmax * blocks[b].kmax;
  }
  double* dx = nullptr;
  int* dbad = nullptr;
  if (cudaMalloc(&dx, (size_t)xoff[nblocks] * 8) != cudaSuccess || cudaMalloc(&dbad, sizeof(int)) != cudaSuccess) {
    cudaFree(dx);
    E.err = "device allocation failed (grid nodes)";
    return false;
  }
  auto fail = [&](const char* what) {
    cudaFree(dx); cudaFree(dbad);
    E.err = std::string(what) + ": " + cudaGetErrorString(cudaGetLastError());
    return false;
  };
  const int T = 256;
  auto nblk_of = [T](long long n) { return (unsigned)((n + T - 1) / T); };
  for (int b = 0; b < nblocks; ++b)
    if (cudaMemcpy(dx + xoff[b], blocks[b].xyz, (size_t)(xoff[b + 1] - xoff[b]) * 8, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail("grid node upload");
  k_scale<<<nblk_of(xoff[nblocks]), T>>>(dx, xoff[nblocks], scale);
  cudaMemset(dbad, 0, sizeof(int));
  // face vectors (degenerate patches zero their face's plane)
  for (int b = 0; b < nblocks; ++b) {
    const cfd3d_block_desc& d = blocks[b];
    const BlockGeom& G = E.blk[b];
    int zl[3] = {0, 0, 0}, zh[3] = {0, 0, 0};
    const int nmax[3] = {d.imax, d.jmax, d.kmax};
    for (int n = 0; n < d.nbc; ++n) {
      if (d.bc[n].type != CFD3D_BC_DEGENERATE) continue;
      const int* p = d.bc[n].pnts;
      for (int ax = 0; ax < 3; ++ax) {
        if (p[ax] != p[3 + ax]) continue;
        if (p[ax] == 1) zl[ax] = 1;
        else if (p[ax] == nmax[ax]) zh[ax] = 1;
        break;
      }
    }
    NodeBlock X{dx + xoff[b], d.imax, d.jmax};
    const int im = d.imax, jm = d.jmax, km = d.kmax;
    k_geo_faces<0><<<nblk_of((long long)im * (jm + 1) * (km + 1)), T>>>(G, X, gm, nc, zl[0], zh[0]);
    k_geo_faces<1><<<nblk_of((long long)(im + 1) * jm * (km + 1)), T>>>(G, X, gm, nc, zl[1], zh[1]);
    k_geo_faces<2><<<nblk_of((long long)(im + 1) * (jm + 1) * km), T>>>(G, X, gm, nc, zl[2], zh[2]);
  }
  // face-vector halo, one connection after the other (a later one overwrites an earlier)
  for (int b = 0; b < nblocks; ++b)
    for (auto& g : cons[b]) {
      int s1 = 1, s2 = 1;
      if (g.sd[0] == g.ed[0]) { if (g.sd[1] > g.ed[1]) s1 = -1; if (g.sd[2] > g.ed[2]) s2 = -1; }
      else if (g.sd[1] == g.ed[1]) { if (g.sd[2] > g.ed[2]) s1 = -1; if (g.sd[0] > g.ed[0]) s2 = -1; }
      else { if (g.sd[0] > g.ed[0]) s1 = -1; if (g.sd[1] > g.ed[1]) s2 = -1; }
      const long long n = (long long)(g.e[0] - g.s[0] + 1) * (g.e[1] - g.s[1] + 1) * (g.e[2] - g.s[2] + 1);
      k_geo_face_halo<<<nblk_of(n), T>>>(g, E.blk[b], E.blk[g.donor], s1, s2, gm, nc);
    }
  // node ranges become cell ranges ("reodering", src/grid_module.f90:926-940)
  for (auto& cl : cons)
    for (auto& g : cl)
      for (int m = 0; m < 3; ++m) {
        if (g.s[m] != g.e[m]) g.s[m] += 1;
        if (g.sd[m] != g.ed[m]) {
          if (g.sd[m] < g.ed[m]) g.sd[m] += 1;
          else g.ed[m] += 1;
        }
      }
  auto exchange = [&](int var) {
    for (int b = 0; b < nblocks; ++b)
      for (auto& g : cons[b]) {
        const long long n = (long long)(g.e[0] - g.s[0] + 1) * (g.e[1] - g.s[1] + 1) * (g.e[2] - g.s[2] + 1);
        k_geo_exchange<<<nblk_of(n), T>>>(g, E.blk[b], E.blk[g.donor], var, gm, nc);
      }
  };
  // volumes and centroids, their ghosts, the volume check and halo
  for (int b = 0; b < nblocks; ++b) {
    const cfd3d_block_desc& d = blocks[b];
    const BlockGeom& G = E.blk[b];
    NodeBlock X{dx + xoff[b], d.imax, d.jmax};
    const long long nin = (long long)(d.imax - 1) * (d.jmax - 1) * (d.kmax - 1);
    k_geo_cells<<<nblk_of(nin), T>>>(G, X, gm, nc);
    k_geo_ghosts<<<nblk_of((long long)(d.imax - 1) * (d.kmax - 1)), T>>>(G, gm, nc, 0, 0);
    k_geo_ghosts<<<nblk_of((long long)(d.jmax + 1) * (d.kmax - 1)), T>>>(G, gm, nc, 1, 0);
    k_geo_ghosts<<<nblk_of((long long)(d.imax + 1) * (d.jmax + 1)), T>>>(G, gm, nc, 2, 0);
    k_geo_check<<<nblk_of(nin), T>>>(G, gm, nc, dbad);
  }
  int bad = 0;
  if (cudaMemcpy(&bad, dbad, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return fail("grid metrics");
  if (bad) { cudaFree(dx); cudaFree(dbad); E.err = "zero/negative cell volume"; return false; }
  exchange(0);
  if (ngrd == 5) {
    // wall-face centres of every block's wall patches (from the scaled nodes, as the
    // device has them), then the brute force over all interior cells
    std::vector<double> wall;
    for (int b = 0; b < nblocks; ++b) {
      const cfd3d_block_desc& d = blocks[b];
      auto XN = [&](int v, int i, int j, int k) {
        return d.xyz[v + 3 * ((i - 2) + (size_t)d.imax * ((j - 2) + (size_t)d.jmax * (k - 2)))] * scale;
      };
      for (int n = 0; n < d.nbc; ++n) {
        const int ty = d.bc[n].type;
        if (ty != CFD3D_BC_WALL && ty != CFD3D_BC_WALL_COUNTERROTATING && ty != CFD3D_BC_WALL_HEATFLUX) continue;
        const int* p = d.bc[n].pnts;
        int ax = -1;
        for (int a = 0; a < 3; ++a) if (p[a] == p[3 + a]) ax = a;
        int nmax[3] = {d.imax, d.jmax, d.kmax};
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) { lo[a] = p[a] + 1; hi[a] = p[3 + a]; }
        int plane = (p[ax] == 1) ? 2 : nmax[ax] + 1;
        int t1 = (ax + 1) % 3, t2 = (ax + 2) % 3;
        if (ax == 1) { t1 = 0; t2 = 2; }
        for (int b2 = lo[t2]; b2 <= hi[t2]; ++b2)
          for (int a2 = lo[t1]; a2 <= hi[t1]; ++a2) {
            int q0[3], q1[3], q2[3], q3[3];
            q0[ax] = q1[ax] = q2[ax] = q3[ax] = plane;
            q0[t1] = a2; q0[t2] = b2;
            q1[t1] = a2 + 1; q1[t2] = b2;
            q2[t1] = a2; q2[t2] = b2 + 1;
            q3[t1] = a2 + 1; q3[t2] = b2 + 1;
            for (int v = 0; v < 3; ++v)
              wall.push_back(0.25 * (XN(v, q0[0], q0[1], q0[2]) + XN(v, q1[0], q1[1], q1[2]) +
                                     XN(v, q2[0], q2[1], q2[2]) + XN(v, q3[0], q3[1], q3[2])));
          }
      }
    }
    const int nwall = (int)(wall.size() / 3);
    double* dwall = nullptr;
    if (nwall > 0) {
      if (cudaMalloc(&dwall, wall.size() * 8) != cudaSuccess) return fail("device allocation failed (wall faces)");
      cudaMemcpy(dwall, wall.data(), wall.size() * 8, cudaMemcpyHostToDevice);
    }
    k_wall_distance<<<nblk_of(E.nint), T, 3 * T * sizeof(float)>>>(E.d.blk, nblocks, E.nint, gm, nc, dwall, nwall);
    for (int b = 0; b < nblocks; ++b) {
      const cfd3d_block_desc& d = blocks[b];
      const BlockGeom& G = E.blk[b];
      k_geo_ghosts<<<nblk_of((long long)(d.imax - 1) * (d.kmax - 1)), T>>>(G, gm, nc, 0, 1);
      k_geo_ghosts<<<nblk_of((long long)(d.jmax + 1) * (d.kmax - 1)), T>>>(G, gm, nc, 1, 1);
      k_geo_ghosts<<<nblk_of((long long)(d.imax + 1) * (d.jmax + 1)), T>>>(G, gm, nc, 2, 1);
    }
    exchange(4);
    const cudaError_t e = cudaDeviceSynchronize();
    cudaFree(dwall);
    if (e != cudaSuccess) return fail("wall distance");
  }
  const cudaError_t e = cudaDeviceSynchronize();
  cudaFree(dx); cudaFree(dbad);
  if (e != cudaSuccess) { E.err = std::string("grid metrics: ") + cudaGetErrorString(e); return false; }
  return true;
}

// The halo of the volume-fraction gradient (setbc_vfg, src/bc_module.f90:1398-1804): for
// each 1-to-1 interface, the block's first interior layer into the donor's first ghost
// layer, as (source, target) padded-cell pairs.
bool setup_vfg_halo(Engine& E, const cfd3d_block_desc* blocks, int nblocks) {
  std::vector<int> pairs;
  for (int b = 0; b < nblocks; ++b) {
    std::vector<Con> cons;
    if (!read_cons(blocks[b], nblocks, cons, E.err)) return false;
    const BlockGeom& S = E.blk[b];
    for (auto g : cons) {
      for (int m = 0; m < 3; ++m) {
        if (g.s[m] != g.e[m]) g.s[m] += 1;
        if (g.sd[m] != g.ed[m]) { if (g.sd[m] < g.ed[m]) g.sd[m] += 1; else g.ed[m] += 1; }
      }
      const BlockGeom& D = E.blk[g.donor];
      for (int k = g.s[2]; k <= g.e[2]; ++k)
        for (int j = g.s[1]; j <= g.e[1]; ++j)
          for (int i = g.s[0]; i <= g.e[0]; ++i) {
            int ii, jj, kk;
            cmap(g, i, j, k, ii, jj, kk);
            if (ii < 1 || ii > D.imax + 1 || jj < 1 || jj > D.jmax + 1 || kk < 1 || kk > D.kmax + 1) {
              E.err = "volume-fraction halo target outside the donor block"; return false;
            }
            pairs.push_back((int)(S.off + (i + 1) + (long long)S.ni * ((j + 1) + (long long)S.nj * (k + 1))));
            pairs.push_back((int)(D.off + (ii + 1) + (long long)D.ni * ((jj + 1) + (long long)D.nj * (kk + 1))));
          }
    }
  }
  E.d.nvfg_halo = (int)(pairs.size() / 2);
  if (pairs.empty()) return true;
  int* dp = nullptr;
  if (cudaMalloc(&dp, pairs.size() * sizeof(int)) != cudaSuccess ||
      cudaMemcpy(dp, pairs.data(), pairs.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dp);
    E.err = "device allocation failed (volume-fraction halo)";
    return false;
  }
  E.d.vfg_halo = dp;
  return true;
}

// ---------------------------------------------------------------------------------------
// boundary program
namespace {

enum Face { F_IMIN, F_IMAX, F_JMIN, F_JMAX, F_KMIN, F_KMAX, F_NOFACE };

struct Bc {
  int kind;            // GhostKind
  int type;            // cfd3d BC type (face patches)
  Face face = F_NOFACE;
  int s[3], e[3], o[3] = {0, 0, 0}, dir[3] = {0, 0, 0};
  int nb[6][3];
  bool farfield_sign = false;
  bool shifted = false;   // bcshiftedperiodic: copies from 16 cells along i and the face normal
  int hf_off = 0;         // heat-flux wall: offset of its history in the table
  int tp_index = 0;       // total-pressure inlet: its pool (the patch's number among its block's inlets)
};

int wall_kind(const Par& c) {
  if (c.iturb == 0) return G_WALL_KW;
  if (c.iturb == -1) return G_WALL_KE;
  if (c.iturb == -2) return G_WALL_VISCOUS;
  return G_SYMMETRY;  // bcwallinviscid is the symmetry reflection
}

}  // namespace

bool setup_ghost_program(Engine& E, const cfd3d_block_desc* blocks, int nblocks) {
  const Par& c = E.par;
  std::vector<GhostOp> ops[3];
  std::vector<double> hft;   // heat-flux histories
  // total-pressure inlets: per pool 4 ints per face cell.  The reference reduces each inlet's
  // averages over the communicator of every rank carrying one (bc_comm_world, icolor 12,
  // src/bc_module.f90:321,349,3411-3416), and the n-th inlet of each rank meets the others'
  // n-th in the collective: pool n gathers the n-th total-pressure patch of every block, and
  // all of its patches take the pool's Newton solution.
  std::vector<std::vector<int>> tp_ent;
  for (int b = 0; b < nblocks; ++b) {
    const cfd3d_block_desc& d = blocks[b];
    int tp_ord = 0;
    const BlockGeom& G = E.blk[b];
    const int im = d.imax, jm = d.jmax, km = d.kmax;
    auto gi = [&](int i, int j, int k) -> int {
      return (int)(G.off + (i + 1) + (long long)G.ni * ((j + 1) + (long long)G.nj * (k + 1)));
    };
    // ---- face patches (src/bc_module.f90:126-335)
    std::vector<Bc> bcs;
    for (int n = 0; n < d.nbc; ++n) {
      const int* p = d.bc[n].pnts;
      Bc bi;
      bi.type = d.bc[n].type;
      int ax = -1;
      for (int a = 0; a < 3; ++a) if (p[a] == p[3 + a]) ax = a;
      if (ax < 0) { E.err = "bc patch is not a face"; return false; }
      int nmax[3] = {im, jm, km};
      bool mn = (p[ax] == 1);
      if (!mn && p[ax] != nmax[ax]) { E.err = "bc patch is not on a block face"; return false; }
      for (int a = 0; a < 3; ++a) { bi.s[a] = p[a] + 1; bi.e[a] = p[3 + a]; bi.dir[a] = 1; }
      bi.s[ax] = bi.e[ax] = mn ? 1 : p[ax] + 1;
      bi.dir[ax] = -1;
      if (mn) { bi.s[ax] -= 2; bi.o[ax] = 2 * bi.e[ax] + 1; }
      else { bi.e[ax] += 2; bi.o[ax] = 2 * bi.s[ax] - 1; }
      bi.face = (Face)(2 * ax + (mn ? 0 : 1));
      switch (bi.type) {
        case CFD3D_BC_WALL: bi.kind = wall_kind(c); break;
        // the counter-rotating family (src/bc_module.f90:3516-3810): the wall at rest while
        // the grid turns, so the ghost velocity takes twice the face's grid velocity off
        case CFD3D_BC_WALL_COUNTERROTATING:
          if (c.iturb == -1) { E.err = "counter-rotating walls under k-epsilon are not built"; return false; }
          bi.kind = (c.iturb == 0) ? G_CRWALL_KW : (c.iturb == -2 ? G_CRWALL : G_CRWALL_INV);
          break;
        case CFD3D_BC_WALL_HEATFLUX: {
          // the HeatFlux family (src/bc_module.f90:233-249): the SST variant.  The laminar
          // one reads the wall distance grd(5), which a laminar run does not have (its grd
          // holds 4 values), and an Euler run has no routine for the family at all.
          if (c.iturb != 0) { E.err = "heat-flux walls need the SST model (iturb = 0)"; return false; }
          const cfd3d_bc_patch& bp = d.bc[n];
          if (bp.ndata < 1 || !bp.tdata || !bp.heatflux) { E.err = "heat-flux wall without its history"; return false; }
          for (int m = 1; m < bp.ndata; ++m)
            if (!(bp.tdata[m] > bp.tdata[m - 1])) { E.err = "heat-flux history times must increase"; return false; }
          bi.kind = G_HFWALL_KW;
          bi.hf_off = (int)hft.size();
          hft.push_back((double)bp.ndata);
          for (int m = 0; m < bp.ndata; ++m) hft.push_back(bp.tdata[m]);
          for (int m = 0; m < bp.ndata; ++m) hft.push_back(bp.heatflux[m]);
          break;
        }
        case CFD3D_BC_TOTALPRESSURE_IN:
          bi.kind = G_TOTALP; bi.farfield_sign = true;
          bi.tp_index = tp_ord++;
          if ((int)tp_ent.size() <= bi.tp_index) tp_ent.emplace_back();
          break;
        case CFD3D_BC_MASSFLOWRATE_IN: bi.kind = G_MASSFLOW_IN; break;
        case CFD3D_BC_SHIFTED_PERIODIC: bi.kind = G_COPY; bi.shifted = true; break;
        case CFD3D_BC_SYMMETRY: bi.kind = G_SYMMETRY; break;
        case CFD3D_BC_FARFIELD: bi.kind = G_FARFIELD; bi.farfield_sign = true; break;
        case CFD3D_BC_EXTRAPOLATE: case CFD3D_BC_DEGENERATE: bi.kind = G_EXTRAP; break;
        case CFD3D_BC_INFLOW_SUBSONIC: bi.kind = G_INFLOW_SUB; bi.farfield_sign = true; break;
        case CFD3D_BC_OUTFLOW_SUBSONIC: bi.kind = G_OUTFLOW_SUB; bi.farfield_sign = true; break;
        case CFD3D_BC_INFLOW_SUPERSONIC: bi.kind = G_INFLOW_SUP; bi.farfield_sign = true; break;
        case CFD3D_BC_INFLOW: case CFD3D_BC_OUTFLOW: bi.kind = -1; break;   // bcinflow / bcoutflow: no-ops
        default: E.err = "unknown bc type"; return false;
      }
      for (int q = 0; q < 6; ++q) for (int r = 0; r < 3; ++r) bi.nb[q][r] = 0;
      bcs.push_back(bi);
    }
    auto is_surf = [&](const int* pnt, std::initializer_list<int> axes) {
      for (auto& bc : bcs) {
        if (bc.type != CFD3D_BC_WALL && bc.type != CFD3D_BC_WALL_COUNTERROTATING && bc.type != CFD3D_BC_WALL_HEATFLUX &&
            bc.type != CFD3D_BC_SYMMETRY) continue;
        bool in = true;
        for (int a : axes) in = in && bc.s[a] <= pnt[a] && bc.e[a] >= pnt[a];
        if (in) return true;
      }
      return false;
    };
    // emits the ghost ops of one descriptor into a phase
    bool shift_err = false;
    auto emit = [&](const Bc& bi, int phase, int nnb, bool skip_zero_nb) {
      if (bi.kind < 0) return;
      for (int k = bi.s[2]; k <= bi.e[2]; ++k)
        for (int j = bi.s[1]; j <= bi.e[1]; ++j)
          for (int i = bi.s[0]; i <= bi.e[0]; ++i) {
            GhostOp op{};
            op.kind = bi.kind;
            op.dst = gi(i, j, k);
            int mi = bi.o[0] + bi.dir[0] * i, mj = bi.o[1] + bi.dir[1] * j, mk = bi.o[2] + bi.dir[2] * k;
            if (bi.shifted) {
              // bcshiftedperiodic (src/bc_module.f90:3134-3297): on a j or k face the ghost
              // takes the cell 16 further along i and 16 further into the block; the last
              // 16 cells along i take their mirror cell.  i faces are left alone.
              if (bi.face == F_IMIN || bi.face == F_IMAX) continue;
              const bool lo = (bi.face == F_JMIN || bi.face == F_KMIN);
              const bool shift = lo ? (i <= bi.e[0] - 16) : (i >= bi.s[0] + 16);
              if (shift) {
                const int di = lo ? 16 : -16;
                mi = i + di; mj = j; mk = k;
                if (bi.face == F_JMIN || bi.face == F_JMAX) mj = j + di;
                else mk = k + di;
                if (mi < -1 || mi > im + 3 || mj < -1 || mj > jm + 3 || mk < -1 || mk > km + 3) {
                  shift_err = true;
                  continue;
                }
              }
            }
            op.src = gi(mi, mj, mk);
            op.bnd = op.src;
            for (int q = 0; q < 6; ++q) op.nb[q] = -1;
            op.fidx = op.src; op.fplane = GM_CX; op.fsign = 1.0f;
            op.pad = (bi.kind == G_TOTALP) ? bi.tp_index : bi.hf_off;
            op.gcell = op.src;
            if (bi.kind == G_SYMMETRY || bi.kind == G_FARFIELD || bi.kind == G_WALL_KW || bi.kind == G_HFWALL_KW ||
                bi.kind == G_TOTALP || bi.kind == G_CRWALL || bi.kind == G_CRWALL_INV || bi.kind == G_CRWALL_KW ||
                bi.kind == G_MASSFLOW_IN || ghost_ff_mode(bi.kind)) {
              int ii = mi, jj = mj, kk = mk;
              float s = bi.farfield_sign ? -1.0f : 1.0f;
              switch (bi.face) {
                case F_IMIN: ii = bi.o[0] + bi.dir[0] * bi.e[0]; op.fidx = gi(ii - 1, jj, kk); op.fplane = GM_CX; op.fsign = s; break;
                case F_IMAX: ii = bi.o[0] + bi.dir[0] * bi.s[0]; op.fidx = gi(ii, jj, kk); op.fplane = GM_CX; op.fsign = -s; break;
                case F_JMIN: jj = bi.o[1] + bi.dir[1] * bi.e[1]; op.fidx = gi(ii, jj - 1, kk); op.fplane = GM_EX; op.fsign = s; break;
                case F_JMAX: jj = bi.o[1] + bi.dir[1] * bi.s[1]; op.fidx = gi(ii, jj, kk); op.fplane = GM_EX; op.fsign = -s; break;
                case F_KMIN: kk = bi.o[2] + bi.dir[2] * bi.e[2]; op.fidx = gi(ii, jj, kk - 1); op.fplane = GM_TX; op.fsign = s; break;
                case F_KMAX: kk = bi.o[2] + bi.dir[2] * bi.s[2]; op.fidx = gi(ii, jj, kk); op.fplane = GM_TX; op.fsign = -s; break;
                default: break;  // corner 'Kmin'/'Kmax': the boundary cell stays the mirror cell
              }
              op.bnd = gi(ii, jj, kk);
              switch (bi.face) {
                case F_IMIN: op.gcell = gi(ii - 1, jj, kk); break;
                case F_IMAX: op.gcell = gi(ii + 1, jj, kk); break;
                case F_JMIN: op.gcell = gi(ii, jj - 1, kk); break;
                case F_JMAX: op.gcell = gi(ii, jj + 1, kk); break;
                case F_KMIN: op.gcell = gi(ii, jj, kk - 1); break;
                case F_KMAX: op.gcell = gi(ii, jj, kk + 1); break;
                default: op.gcell = op.bnd; break;
              }
              if (bi.kind == G_TOTALP) {
                // the patch's reduction visits each boundary face once: the outermost layer
                const int ax = (int)bi.face / 2;
                const int idx[3] = {i, j, k};
                if (idx[ax] == (((int)bi.face % 2 == 0) ? bi.s[ax] : bi.e[ax])) {
                  std::vector<int>& te = tp_ent[bi.tp_index];
                  te.push_back(op.bnd); te.push_back(op.fidx); te.push_back(op.fplane); te.push_back(op.gcell);
                }
              }
            }
            int q2 = 0;
            for (int q = 0; q < nnb; ++q) {
              const int* nb = bi.nb[q];
              if (skip_zero_nb && nb[0] == 0 && nb[1] == 0 && nb[2] == 0) continue;
              op.nb[q2++] = gi(nb[0] + bi.dir[0] * i, nb[1] + bi.dir[1] * j, nb[2] + bi.dir[2] * k);
            }
            ops[phase].push_back(op);
          }
    };
    for (auto& bi : bcs) emit(bi, 0, 0, false);
    if (shift_err) { E.err = "shifted periodic patch: the 16-cell source lies outside the block"; return false; }
    // ---- 12 edges (src/bc_module.f90:505-865)
    struct ED { int s[3], e[3], n1[3], n2[3], n3[3], o[3]; };
    const ED EDG[12] = {
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
    for (int m = 0; m < 12; ++m) {
      Bc e;
      for (int q = 0; q < 3; ++q) {
        e.s[q] = EDG[m].s[q]; e.e[q] = EDG[m].e[q]; e.o[q] = EDG[m].o[q]; e.dir[q] = 0;
        e.nb[0][q] = EDG[m].n1[q]; e.nb[1][q] = EDG[m].n2[q]; e.nb[2][q] = EDG[m].n3[q];
        e.nb[3][q] = e.nb[4][q] = e.nb[5][q] = 0;
      }
      bool s1, s2;
      int along;
      if (m < 4) { s1 = is_surf(e.nb[0], {0, 1}); s2 = is_surf(e.nb[1], {0, 1}); along = 2; }
      else if (m < 8) { s1 = is_surf(e.nb[0], {0, 2}); s2 = is_surf(e.nb[2], {0, 2}); along = 1; }
      else { s1 = is_surf(e.nb[1], {1, 2}); s2 = is_surf(e.nb[2], {1, 2}); along = 0; }
      if (s1 && s2) {
        e.kind = (c.iturb == 0) ? G_WALLWALL_KW4 : G_WALLWALL;
        e.dir[along] = 1;
        emit(e, 1, 3, true);
      } else if (s1 || s2) {
        e.kind = wall_kind(c);
        if (m < 4) {
          if (s1) { e.face = (m == 0 || m == 2) ? F_IMIN : F_IMAX; e.o[0] = e.nb[1][0]; e.o[1] = e.nb[1][1]; }
          else { e.face = (m == 0 || m == 1) ? F_JMIN : F_JMAX; e.o[0] = e.nb[0][0]; e.o[1] = e.nb[0][1]; }
        } else if (m < 8) {
          if (s1) { e.face = (m == 4 || m == 6) ? F_IMIN : F_IMAX; e.o[0] = e.nb[2][0]; e.o[2] = e.nb[2][2]; }
          else { e.face = (m == 4 || m == 5) ? F_KMIN : F_KMAX; e.o[0] = e.nb[0][0]; e.o[2] = e.nb[0][2]; }
        } else {
          if (s1) { e.face = (m == 8 || m == 10) ? F_JMIN : F_JMAX; e.o[1] = e.nb[2][1]; e.o[2] = e.nb[2][2]; }
          else { e.face = (m == 8 || m == 9) ? F_KMIN : F_KMAX; e.o[1] = e.nb[1][1]; e.o[2] = e.nb[1][2]; }
        }
        e.dir[along] = 1;
        emit(e, 1, 0, false);
      } else {
        e.kind = G_NOWALL3;
        e.dir[along] = 1;
        emit(e, 1, 3, true);
      }
    }
    // ---- 8 corners (src/bc_module.f90:870-1186)
    for (int m = 0; m < 8; ++m) {
      int mi = m & 1, mj = (m >> 1) & 1, mk = (m >> 2) & 1;
      Bc e;
      e.s[0] = mi ? im + 1 : -1; e.e[0] = mi ? im + 3 : 1;
      e.s[1] = mj ? jm + 1 : -1; e.e[1] = mj ? jm + 3 : 1;
      e.s[2] = mk ? km + 1 : -1; e.e[2] = mk ? km + 3 : 1;
      int gi_ = mi ? im + 1 : 1, ci = mi ? im : 2;
      int gj = mj ? jm + 1 : 1, cj = mj ? jm : 2;
      int gk = mk ? km + 1 : 1, ck = mk ? km : 2;
      int N[6][3] = {{gi_, cj, ck}, {ci, gj, ck}, {ci, cj, gk}, {ci, gj, gk}, {gi_, cj, gk}, {gi_, gj, ck}};
      for (int q = 0; q < 6; ++q) for (int r = 0; r < 3; ++r) e.nb[q][r] = N[q][r];
      e.o[0] = ci; e.o[1] = cj; e.o[2] = ck;
      bool si = is_surf(e.nb[0], {0, 1, 2}), sj = is_surf(e.nb[1], {0, 1, 2}), sk = is_surf(e.nb[2], {0, 1, 2});
      auto org = [&](int q) { for (int r = 0; r < 3; ++r) e.o[r] = N[q][r]; };
      auto setnb = [&](int dst, int src) { for (int r = 0; r < 3; ++r) e.nb[dst][r] = (src < 0) ? 0 : N[src][r]; };
      int ww = (c.iturb == 0) ? G_WALLWALL_KW4 : G_WALLWALL;
      if (si && sj && sk) {
        e.kind = (c.iturb == 0) ? G_WALLWALL_KW8 : G_WALLWALL;
        emit(e, 2, 6, false);
      } else if (!si && sj && sk) {
        org(0); setnb(0, -1); setnb(1, 4); setnb(2, 5); e.kind = ww; emit(e, 2, 3, true);
      } else if (si && !sj && sk) {
        org(1); setnb(0, 3); setnb(1, -1); setnb(2, 5); e.kind = ww; emit(e, 2, 3, true);
      } else if (si && sj && !sk) {
        org(2); setnb(0, 3); setnb(1, 4); setnb(2, -1); e.kind = ww; emit(e, 2, 3, true);
      } else if (!si && !sj && sk) {
        e.face = F_NOFACE;  // the reference's capital-K face label matches no case
        org(5); e.kind = wall_kind(c);
        if (e.kind == G_SYMMETRY) { E.err = "corner with only a k-side wall under inviscid walls is undefined in the reference"; return false; }
        emit(e, 2, 0, false);
      } else if (si && !sj && !sk) {
        e.face = (m % 2 == 0) ? F_IMIN : F_IMAX; org(3); e.kind = wall_kind(c); emit(e, 2, 0, false);
      } else if (!si && sj && !sk) {
        e.face = (m == 0 || m == 1 || m == 4 || m == 5) ? F_JMIN : F_JMAX; org(4); e.kind = wall_kind(c); emit(e, 2, 0, false);
      } else {
        e.kind = G_NOWALL7;
        emit(e, 2, 6, false);
      }
    }
  }
  // ---- halos: own 3-deep slab into the donor's ghost cells (src/bc_module.f90:355-463)
  std::vector<std::vector<Con>> cons(nblocks);
  for (int b = 0; b < nblocks; ++b) {
    if (!read_cons(blocks[b], nblocks, cons[b], E.err)) return false;
    for (auto& g : cons[b])
      for (int m = 0; m < 3; ++m) {
        if (g.s[m] != g.e[m]) g.s[m] += 1;
        if (g.sd[m] != g.ed[m]) { if (g.sd[m] < g.ed[m]) g.sd[m] += 1; else g.ed[m] += 1; }
      }
  }
  for (int b = 0; b < nblocks; ++b) {
    const BlockGeom& S = E.blk[b];
    for (auto g : cons[b]) {
      int ax;
      if (g.s[1] == g.e[1]) ax = 1;
      else if (g.s[0] == g.e[0]) ax = 0;
      else ax = 2;
      int row = -1, sgn = 0;
      for (int r = 0; r < 3; ++r) if (g.tm[r][ax] != 0) { row = r; sgn = g.tm[r][ax]; }
      if (g.s[ax] == 2) { g.e[ax] += 2; g.ed[row] += 2 * sgn; }
      else { g.s[ax] -= 2; g.sd[row] -= 2 * sgn; }
      const BlockGeom& D = E.blk[g.donor];
      for (int k = g.s[2]; k <= g.e[2]; ++k)
        for (int j = g.s[1]; j <= g.e[1]; ++j)
          for (int i = g.s[0]; i <= g.e[0]; ++i) {
            int ii, jj, kk;
            cmap(g, i, j, k, ii, jj, kk);
            if (ii < -1 || ii > D.imax + 3 || jj < -1 || jj > D.jmax + 3 || kk < -1 || kk > D.kmax + 3) {
              E.err = "halo target outside the donor block"; return false;
            }
            GhostOp op{};
            op.kind = G_COPY;
            op.src = (int)(S.off + (i + 1) + (long long)S.ni * ((j + 1) + (long long)S.nj * (k + 1)));
            op.dst = (int)(D.off + (ii + 1) + (long long)D.ni * ((jj + 1) + (long long)D.nj * (kk + 1)));
            op.bnd = op.src;
            for (int q = 0; q < 6; ++q) op.nb[q] = -1;
            ops[0].push_back(op);
          }
    }
  }
  for (int p = 0; p < 3; ++p) {
    E.nops[p] = (int)ops[p].size();
    if (E.nops[p] == 0) continue;
    if (cudaMalloc(&E.d_ops[p], ops[p].size() * sizeof(GhostOp)) != cudaSuccess) { E.err = "cudaMalloc ghost ops"; return false; }
    cudaMemcpy(E.d_ops[p], ops[p].data(), ops[p].size() * sizeof(GhostOp), cudaMemcpyHostToDevice);
  }
  if (!tp_ent.empty()) {
    std::vector<int> off(1, 0), ent;
    for (const auto& te : tp_ent) { ent.insert(ent.end(), te.begin(), te.end()); off.push_back((int)(ent.size() / 4)); }
    const size_t nt = tp_ent.size();
    if (cudaMalloc(&E.d_tp_off, off.size() * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&E.d_tp_ent, std::max<size_t>(ent.size(), 1) * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&E.d_tp_x, 3 * nt * sizeof(double)) != cudaSuccess) {
      E.err = "cudaMalloc total-pressure inlets"; return false;
    }
    cudaMemcpy(E.d_tp_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (!ent.empty()) cudaMemcpy(E.d_tp_ent, ent.data(), ent.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemset(E.d_tp_x, 0, 3 * nt * sizeof(double));
    E.d.ntp = (int)nt; E.d.tp_off = E.d_tp_off; E.d.tp_ent = E.d_tp_ent; E.d.tp_x = E.d_tp_x;
  }
  if (!hft.empty()) {
    if (cudaMalloc(&E.d_hft, hft.size() * sizeof(double)) != cudaSuccess) { E.err = "cudaMalloc heat-flux tables"; return false; }
    cudaMemcpy(E.d_hft, hft.data(), hft.size() * sizeof(double), cudaMemcpyHostToDevice);
    E.d.hft = E.d_hft;
  }
  return true;
}

// ---------------------------------------------------------------------------------------
void setup_planes(Engine& E) {
  // Hyperplanes (i-2)+(j-2)+(k-2) = s of every block, merged by s; within a plane cells are
  // ordered by block, k, j.  The sweep works in this plane-major numbering t: cells[t] is
  // the padded cell, pos[g] its inverse, and nbf / nbb the positions of the three lower /
  // upper interior neighbours (-1 outside the block).  With the (k, j) order, consecutive t
  // of plane s have consecutive neighbours in plane s -/+ 1, so the sweep's loads coalesce.
  long long maxs = 0;
  for (auto& B : E.blk) maxs = std::max<long long>(maxs, (B.imax - 2) + (B.jmax - 2) + (B.kmax - 2));
  std::vector<long long> count(maxs + 2, 0);
  for (auto& B : E.blk)
    for (int k = 2; k <= B.kmax; ++k)
      for (int j = 2; j <= B.jmax; ++j)
        for (int i = 2; i <= B.imax; ++i) ++count[(i - 2) + (j - 2) + (k - 2) + 1];
  E.plane_off.assign(maxs + 2, 0);
  for (long long s = 1; s <= maxs + 1; ++s) E.plane_off[s] = E.plane_off[s - 1] + count[s];
  const long long nint = E.plane_off[maxs + 1];
  std::vector<long long> fill(E.plane_off.begin(), E.plane_off.end() - 1);
  std::vector<int> cells(nint), pos(E.ncell, -1);
  for (auto& B : E.blk)
    for (int k = 2; k <= B.kmax; ++k)
      for (int j = 2; j <= B.jmax; ++j)
        for (int i = 2; i <= B.imax; ++i) {
          long long t = fill[(i - 2) + (j - 2) + (k - 2)]++;
          long long g = B.off + (i + 1) + (long long)B.ni * ((j + 1) + (long long)B.nj * (k + 1));
          cells[t] = (int)g;
          pos[g] = (int)t;
        }
  std::vector<int> nbf(3 * nint, -1), nbb(3 * nint, -1);
  for (auto& B : E.blk) {
    const long long st[3] = {1, B.ni, (long long)B.ni * B.nj};
    for (int k = 2; k <= B.kmax; ++k)
      for (int j = 2; j <= B.jmax; ++j)
        for (int i = 2; i <= B.imax; ++i) {
          long long g = B.off + (i + 1) + (long long)B.ni * ((j + 1) + (long long)B.nj * (k + 1));
          const int t = pos[g];
          const int p3[3] = {i, j, k};
          const int lim[3] = {B.imax, B.jmax, B.kmax};
          for (int q = 0; q < 3; ++q) {
            if (p3[q] - 1 >= 2) nbf[q * nint + t] = pos[g - st[q]];
            if (p3[q] + 1 <= lim[q]) nbb[q * nint + t] = pos[g + st[q]];
          }
        }
  }
  // chunks of the dataflow sweeps: each plane cut into runs of at most SW_CH cells
  std::vector<int> chunks;
  for (long long s = 0; s + 1 < (long long)E.plane_off.size(); ++s)
    for (long long t = E.plane_off[s]; t < E.plane_off[s + 1]; t += SW_CH) chunks.push_back((int)t);
  E.d.nchunk = (int)chunks.size();
  chunks.push_back((int)nint);
  cudaMalloc(&E.d_chunk_t0, chunks.size() * sizeof(int));
  cudaMemcpy(E.d_chunk_t0, chunks.data(), chunks.size() * sizeof(int), cudaMemcpyHostToDevice);
  E.d.chunk_t0 = E.d_chunk_t0;
  std::vector<int> chunk_of(nint);
  for (size_t q = 0; q + 1 < chunks.size(); ++q)
    for (int t = chunks[q]; t < chunks[q + 1]; ++t) chunk_of[t] = (int)q;
  cudaMalloc(&E.d_chunk_of, nint * sizeof(int));
  cudaMemcpy(E.d_chunk_of, chunk_of.data(), nint * sizeof(int), cudaMemcpyHostToDevice);
  E.d.chunk_of = E.d_chunk_of;
  cudaMalloc(&E.d_planes, nint * sizeof(int));
  cudaMemcpy(E.d_planes, cells.data(), nint * sizeof(int), cudaMemcpyHostToDevice);
  cudaMalloc(&E.d_pos, E.ncell * sizeof(int));
  cudaMemcpy(E.d_pos, pos.data(), E.ncell * sizeof(int), cudaMemcpyHostToDevice);
  cudaMalloc(&E.d_nbf, 3 * nint * sizeof(int));
  cudaMemcpy(E.d_nbf, nbf.data(), 3 * nint * sizeof(int), cudaMemcpyHostToDevice);
  cudaMalloc(&E.d_nbb, 3 * nint * sizeof(int));
  cudaMemcpy(E.d_nbb, nbb.data(), 3 * nint * sizeof(int), cudaMemcpyHostToDevice);
}

}  // namespace cfd

namespace cfd {

// The mixed form's tiles: every block's interior cut into boxes of TILE_I x TILE_J x
// TILE_K cells (smaller at the block's far faces), numbered in forward ticket order: by
// tile hyperplane a + b + c, then block, then c, b, a.  A tile's tiles below (-i, -j, -k)
// lie on the previous tile hyperplane, so they always hold earlier tickets.  pos[g] is the
// cell's slot: tile * TILE_SLOTS + lane * TILE_LS + li, lane = lj + TILE_J lk.
bool setup_tiles(Engine& E) {
  struct Raw { int blk, a, b, c; };
  std::vector<Raw> raw;
  std::vector<std::array<int, 3>> nt(E.blk.size());
  for (size_t bi = 0; bi < E.blk.size(); ++bi) {
    const BlockGeom& B = E.blk[bi];
    const int n3[3] = {(B.imax - 1 + TILE_I - 1) / TILE_I, (B.jmax - 1 + TILE_J - 1) / TILE_J,
                       (B.kmax - 1 + TILE_K - 1) / TILE_K};
    nt[bi] = {n3[0], n3[1], n3[2]};
    for (int c = 0; c < n3[2]; ++c)
      for (int b = 0; b < n3[1]; ++b)
        for (int a = 0; a < n3[0]; ++a) raw.push_back({(int)bi, a, b, c});
  }
  std::stable_sort(raw.begin(), raw.end(), [](const Raw& x, const Raw& y) {
    const int sx = x.a + x.b + x.c, sy = y.a + y.b + y.c;
    if (sx != sy) return sx < sy;
    if (x.blk != y.blk) return x.blk < y.blk;
    if (x.c != y.c) return x.c < y.c;
    if (x.b != y.b) return x.b < y.b;
    return x.a < y.a;
  });
  const long long ntile = (long long)raw.size();
  if (ntile * TILE_SLOTS >= (1ll << 31)) { E.err = "case too large for 32-bit tile slots"; return false; }
  // tile index of (block, a, b, c)
  std::vector<std::vector<int>> idx(E.blk.size());
  for (size_t bi = 0; bi < E.blk.size(); ++bi) idx[bi].assign((size_t)nt[bi][0] * nt[bi][1] * nt[bi][2], -1);
  for (long long t = 0; t < ntile; ++t) {
    const Raw& r = raw[t];
    idx[r.blk][((size_t)r.c * nt[r.blk][1] + r.b) * nt[r.blk][0] + r.a] = (int)t;
  }
  std::vector<TileDesc> tiles(ntile);
  std::vector<int> pos(E.ncell, -1);
  for (long long t = 0; t < ntile; ++t) {
    const Raw& r = raw[t];
    const BlockGeom& B = E.blk[r.blk];
    const auto& n3 = nt[r.blk];
    TileDesc& T = tiles[t];
    T.blk = r.blk;
    T.i0 = 2 + r.a * TILE_I; T.j0 = 2 + r.b * TILE_J; T.k0 = 2 + r.c * TILE_K;
    T.ni = std::min(TILE_I, B.imax + 1 - T.i0);
    T.nj = std::min(TILE_J, B.jmax + 1 - T.j0);
    T.nk = std::min(TILE_K, B.kmax + 1 - T.k0);
    auto at = [&](int a, int b, int c) -> int {
      if (a < 0 || b < 0 || c < 0 || a >= n3[0] || b >= n3[1] || c >= n3[2]) return -1;
      return idx[r.blk][((size_t)c * n3[1] + b) * n3[0] + a];
    };
    T.lo[0] = at(r.a - 1, r.b, r.c); T.lo[1] = at(r.a, r.b - 1, r.c); T.lo[2] = at(r.a, r.b, r.c - 1);
    T.hi[0] = at(r.a + 1, r.b, r.c); T.hi[1] = at(r.a, r.b + 1, r.c); T.hi[2] = at(r.a, r.b, r.c + 1);
    for (int lk = 0; lk < T.nk; ++lk)
      for (int lj = 0; lj < T.nj; ++lj)
        for (int li = 0; li < T.ni; ++li) {
          const int i = T.i0 + li, j = T.j0 + lj, k = T.k0 + lk;
          const long long g = B.off + (i + 1) + (long long)B.ni * ((j + 1) + (long long)B.nj * (k + 1));
          pos[g] = (int)(t * TILE_SLOTS + (lj + TILE_J * lk) * TILE_LS + li);
        }
  }
  E.d.ntile = (int)ntile;
  E.d.nslot = ntile * TILE_SLOTS;
  if (cudaMalloc(&E.d_tiles, ntile * sizeof(TileDesc)) != cudaSuccess ||
      cudaMalloc(&E.d_pos, E.ncell * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&E.d.trf, (size_t)ntile * NTR * TILE_SLOTS * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&E.d.tq, (size_t)ntile * NPVM * TILE_SLOTS * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&E.d.tyf, (size_t)ntile * NPVM * TILE_SLOTS * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&E.d.tyb, (size_t)ntile * NPVM * TILE_SLOTS * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&E.d.tin, (size_t)ntile * NPVM * TILE_IN * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&E.d.done, (size_t)ntile * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&E.d.tickets, 2 * sizeof(unsigned)) != cudaSuccess) {
    E.err = "device allocation failed (tile sweeps)";
    return false;
  }
  cudaMemcpy(E.d_tiles, tiles.data(), ntile * sizeof(TileDesc), cudaMemcpyHostToDevice);
  cudaMemcpy(E.d_pos, pos.data(), E.ncell * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemset(E.d.tq, 0, (size_t)ntile * NPVM * TILE_SLOTS * sizeof(float));
  cudaMemset(E.d.tyf, 0, (size_t)ntile * NPVM * TILE_SLOTS * sizeof(float));
  cudaMemset(E.d.tyb, 0, (size_t)ntile * NPVM * TILE_SLOTS * sizeof(float));
  cudaMemset(E.d.trf, 0, (size_t)ntile * NTR * TILE_SLOTS * sizeof(float));
  cudaMemset(E.d.tin, 0, (size_t)ntile * NPVM * TILE_IN * sizeof(float));
  cudaMemset(E.d.done, 0, (size_t)ntile * sizeof(int));
  cudaMemset(E.d.tickets, 0, 2 * sizeof(unsigned));
  E.d.tiles = E.d_tiles;
  E.d.pos = E.d_pos;
  return true;
}

}  // namespace cfd
