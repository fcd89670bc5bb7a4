// engine.cuh -- data layout and host-side engine state shared by the translation units.
//
// HBM layout: every block's padded cell box (-1..imax+3 per direction, the reference's
// storage range, src/variable_module.f90:69-71) is laid end to end in one global cell
// space of `ncell` entries.  Every field is a structure of arrays: variable v of field f
// lives at f[v * ncell + g], with g the padded global cell index, so a warp walking i
// reads consecutive addresses.  Face vectors use the same index: cx(i,j,k) -- the
// i-face between cells i and i+1 -- is stored at the index of cell (i,j,k).
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/cfd3d.h"
#include "physics.cuh"

namespace cfd {

constexpr int MAXBLK = 256;

struct BlockGeom {
  int imax, jmax, kmax;     // node counts
  int ni, nj, nk;           // padded extents imax+5, ...
  long long off;            // first padded cell of the block
  long long int_off;        // first interior cell in the flat interior numbering
  long long face_off[3];    // first face of each direction in the flat face numbering
  long long col_off[3];     // first column of cells along direction 1 (i, k) / 2 (i, j)
};

// gm planes: face vectors and cell geometry
enum { GM_CX = 0, GM_EX = 3, GM_TX = 6, GM_GRD = 9 };

enum GhostKind : int {
  G_COPY = 0, G_EXTRAP, G_WALL_VISCOUS, G_WALL_KW, G_SYMMETRY, G_FARFIELD,
  G_WALLWALL, G_WALLWALL_KW4, G_WALLWALL_KW8, G_NOWALL3, G_NOWALL7,
  G_INFLOW_SUB, G_OUTFLOW_SUB, G_INFLOW_SUP,  // the farfield treatment with a forced branch
  G_CRWALL_KW, G_MASSFLOW_IN, G_HFWALL_KW, G_WALL_KE, G_TOTALP, G_CRWALL, G_CRWALL_INV
};

// the farfield_pv branch of a characteristic ghost kind
__host__ __device__ inline int ghost_ff_mode(int kind) {
  return kind == G_INFLOW_SUB ? 3 : kind == G_OUTFLOW_SUB ? 1 : kind == G_INFLOW_SUP ? 2 : 0;
}

// one ghost cell write of the compiled boundary program
struct GhostOp {
  int kind;
  int dst;        // written cell
  int src;        // mirror / origin cell
  int bnd;        // boundary cell (pv_s / pv_b / wall data)
  int nb[6];      // neighbour cells (edge / corner fills), -1 = unused
  int fidx;       // cell index of the face vector
  int fplane;     // GM_CX / GM_EX / GM_TX
  float fsign;    // +1 / -1
  int pad;
  int gcell;      // the ghost cell across the boundary face from bnd (the face's grid velocity)
};

// device scalars of one iteration
struct Scalars {
  double time_acc;
  unsigned long long dtmin_bits;
  double res[NPVM];
  double resmax;
  long long resmax_cell;
  unsigned long long snd2_fallbacks;
  int nonfinite;
  int sweep_stall;   // a dataflow sweep's wait for a neighbour ran out (the sweep went on)
  // the time the boundary program sees (heat-flux histories): timeprev and nt_phy of the
  // current cfd3d_iterate call, written by the host before each launch
  double timeprev;
  int nt_phy;
  int pv_changed;   // cfd3d_upload_primitives_all: some uploaded pv differed from the device's
};

// the base state of a face state's expansion (k_shadow): d(1/rho_l)/dp, d(1/rho_l)/dT,
// dh_l/dp, dh_l/dT, the rounding of the FP32 shadow's p and T (exact - shadow), the mixture's
// rho - rhoref and h - href, rho, 1/rho_l, h_l - h_g
enum { LQ_VP = 0, LQ_VT, LQ_HP, LQ_HT, LQ_RP, LQ_RT, LQ_RDEV, LQ_HDEV, LQ_RHO, LQ_VL, LQ_HLG, NLQ };

// ---- the mixed form's tile sweeps ------------------------------------------------------
// A tile is a box of at most TILE_I x TILE_J x TILE_K interior cells of one block.  One warp
// sweeps it: lane (lj, lk) = lj + TILE_J lk walks the column of cells (li, lj, lk), li
// ascending (descending in the backward sweep), so that at step s the lanes hold the
// tile's hyperplane li + lj + lk = s; a cell's lower (upper) neighbours within the tile are
// the lane's own previous cell and the previous cells of lanes -1 and -TILE_J (+1, +TILE_J).
constexpr int TILE_I = 8, TILE_J = 8, TILE_K = 4;
static_assert(TILE_J * TILE_K == 32, "one lane per (j, k) column of a tile");
constexpr int TILE_LS = TILE_I + 1;          // slots per lane: odd, so lanes hit distinct banks
constexpr int TILE_SLOTS = 32 * TILE_LS;     // slots per tile
// contributions entering a tile, by face cell: the i face (one per lane), then the j face
// (TILE_K x TILE_I cells) from TILE_IN_J, then the k face (TILE_J x TILE_I) from TILE_IN_K
constexpr int TILE_IN_J = 32, TILE_IN_K = TILE_IN_J + TILE_K * TILE_I, TILE_IN = TILE_IN_K + TILE_J * TILE_I;
// FP32 tile-record fields of a cell: state, beta, viscous term, diagonal block, the cell's
// own part of dq (both sweeps: D^-1 res from k_rhs, replaced by dq* in the forward sweep),
// then its + face vectors and + face spectral radii (the forward sweep's) and its - ones
// (the backward sweep's)
enum {
  TR_PV = 0,       // pv 1, 2, 3, 5, 6, 7, 8
  TR_DV = 7,       // dv 0, 1, 6 .. 13
  TR_EVV = 17,     // (beta follows from the block: rr - (b1 - 1) drho/dp)
  TR_DIAG = 18,    // 23 values of the closed-form diagonal block
  TR_X = 41,       // the own part of dq (npv)
  TR_COMMON = 50,
  TR_FACEP = 50,   // + face vectors cx, ex, tx
  TR_SPECP = 59,   // + face spectral radii of the three directions
  TR_FACEM = 62,   // - face vectors
  TR_SPECM = 71,   // - face spectral radii
  NTR = 74
};
constexpr int TS_FIELDS = TR_COMMON + 12;    // the FP32 fields one sweep reads
struct TileDesc {
  int blk, i0, j0, k0;     // block and first interior cell (the reference's 2-based indices)
  int ni, nj, nk;          // extents, at most TILE_I, TILE_J, TILE_K
  int lo[3], hi[3];        // the tiles before (-i, -j, -k) and after (+i, +j, +k); -1: none
};
// slot s = tile * TILE_SLOTS + lane * TILE_LS + li; per-tile blocks of NTR (FP32 record),
// NPVM (FP64 own part, FP32 sweep corrections) and NPVM x TILE_IN (entering contributions)
// planes
__host__ __device__ __forceinline__ long long trf_at(long long s, int f) {
  const long long tile = s / TILE_SLOTS;
  return (tile * NTR + f) * TILE_SLOTS + (s - tile * TILE_SLOTS);
}
__host__ __device__ __forceinline__ long long tq_at(long long s, int v) {
  const long long tile = s / TILE_SLOTS;
  return (tile * NPVM + v) * TILE_SLOTS + (s - tile * TILE_SLOTS);
}

struct DevPtr {
  double *pv, *dv, *tv, *gm, *res, *icav, *itt, *ocut, *dt, *rcav, *qq, *dqs, *dcv, *qold, *fi, *fv;
  const BlockGeom* blk;
  int nblk;
  long long ncell;
  long long nint;
  Scalars* sc;
  const double* hft;   // heat-flux histories: per table n, t[n], q[n] (GhostOp.pad is its offset)
  const double* grav;  // gravity history: n, t[n], a[3 n] (a constant acceleration is one row)
  // surface tension (csf = 1): per padded cell the vapour + gas volume fraction vf, its
  // gradient vfg (3 planes, cells 1..imax+1 of each block) and the source of the last
  // residual (3 planes, interior cells); the vfg halo as (source, target) cell pairs
  double *vf, *vfg, *csf;
  const int* vfg_halo;
  int nvfg_halo;
  // total-pressure inlets: per pool p (the p-th inlet of every block) [tp_off[p], tp_off[p+1])
  // face entries (boundary cell, face-vector cell, plane, sign) and the solved (p, T, |u|^2)
  // in tp_x[3 p..]
  int ntp;
  const int* tp_off;
  const int* tp_ent;     // 4 ints per entry
  double* tp_x;
  double* partial;   // per-CTA partial residual sums [gridsize][npv+2]
  // mixed form only: FP32 gauge shadow of pv and FP32 face fluxes (fi / fv unused)
  float *pvf, *fi32, *fv32;
  float* gmf;        // mixed form: FP32 copy of gm (metrics of the FP32 viscous and SST terms)
  float* gmlo;       // mixed form: low parts of the face vectors, gm = gmf + gmlo (df64 terms)
  float* frec;       // mixed form: reconstructed face states of one direction (2 x 12 planes)
  // mixed form: per interior cell the free-stream part of its stored flux deviations,
  // (Phi + pref I).sum(n dl) over its faces, which depends on the metrics alone (npv planes)
  double* clo;
  // mixed form: per padded cell, its EOS state as the base of the face states' first-order
  // expansion (k_shadow), NLQ FP32 planes (LQ_*); rho = 0 marks a cell that carries vapour
  float* lqf;
  // LU-SGS sweep records in plane-major order t (REC_* planes of nint entries); dqs and
  // dcv are plane-major too
  double* rec;
  const int *cells, *pos, *nbf, *nbb;
  // dataflow sweeps: chunk starts in t (chunks of at most SW_CH cells, never across a
  // plane; nchunk + 1 entries), the chunk of every t, per-chunk done flags, the two
  // sweeps' chunk tickets
  const int* chunk_t0;
  const int* chunk_of;
  int nchunk;
  int* done;
  unsigned* tickets;
  // mixed form: FP32 copy of the neighbour part of the records (the first REC_DIAG
  // planes) and FP32 dq
  float *recf, *dqsf;
  // mixed form: the tile sweeps (setup_tiles).  tiles in forward ticket order; trf the FP32
  // tile records; tq the own part D^-1 res per slot (k_rhs, an FP32 solve); tyf / tyb the
  // FP32 corrections of the forward / backward sweep, so that dq = tq + tyf + tyb (k_update);
  // tin the contributions entering each tile (written by the neighbouring tiles during a
  // sweep); done flags per tile
  int ntile;
  long long nslot;
  const TileDesc* tiles;
  float* trf;
  float* tq;
  float *tyf, *tyb;
  float* tin;
};

// sweep record planes: what the sweeps read of a cell, as itself and as a neighbour
enum {
  REC_PV = 0,      // pv 1, 2, 3, 5, 6, 7, 8
  REC_DV = 7,      // dv 0, 1, 6 .. 13
  REC_BETA = 17,
  REC_EVV = 18,
  REC_SPEC = 19,   // 6 face spectral radii
  REC_FACE = 25,   // the cell's + face vectors cx, ex, tx
  REC_DIAG = 34,   // 23 values of the closed-form diagonal block
  REC_RES = 57,    // residual (npv)
  NREC = 66
};

struct Engine {
  cfd3d_config cfg;
  Par par;
  std::vector<BlockGeom> blk;
  long long ncell = 0, nint = 0, nface[3] = {0, 0, 0}, ncol[3] = {0, 0, 0};
  DevPtr d{};
  // ghost program: phase 0 faces + halos, 1 edges, 2 corners
  GhostOp* d_ops[3] = {nullptr, nullptr, nullptr};
  int nops[3] = {0, 0, 0};
  double* d_hft = nullptr;   // heat-flux histories (d.hft), null without heat-flux walls
  double* d_grav = nullptr;  // gravity history (d.grav), null without gravity
  int* d_tp_off = nullptr;
  int* d_tp_ent = nullptr;
  double* d_tp_x = nullptr;
  // LU-SGS plane-major numbering (setup_planes): cells[t], pos[g], lower / upper neighbours
  int* d_planes = nullptr;
  int* d_pos = nullptr;
  int* d_nbf = nullptr;
  int* d_nbb = nullptr;
  std::vector<long long> plane_off;
  int* d_chunk_t0 = nullptr;   // dataflow sweep chunks (setup_planes)
  int* d_chunk_of = nullptr;
  TileDesc* d_tiles = nullptr;  // the mixed form's tiles (setup_tiles)
  int sweep_grid = 0;          // persistent CTAs of the dataflow sweep
  int sweep_planes = 0;        // 1: one launch per hyperplane instead (CFD3D_SWEEP=planes)
  // launch shapes chosen by cfd3d_autotune: threads per CTA of the face kernels and of the
  // residual kernel (64, 128 or 256)
  int tpb_face = 128, tpb_rhs = 128;
  // mixed form: the face stage and the residual pipelined over groups of blocks (the
  // residual of group q on st2 beside the face stage of group q + 1 on st): pipe_groups
  // groups, 1 = no pipelining
  int pipe_groups = 1;
  static constexpr int MAX_PIPE = 16;
  cudaStream_t st = nullptr, st2 = nullptr;
  cudaEvent_t pipe_ev[MAX_PIPE + 2] = {};
  cudaGraphExec_t graph = nullptr;
  int graph_ready = 0;
  int launches_per_iter = 0;
  int red_grid = 0;
  double time_host = 0.0;
  std::string err;
  // host copies of the reference state used by the ghost program
  double pv_ref[NPVM];
  // discrete adjoint (allocated by the first cfd3d_residual_vjp): padded cotangent and
  // gradients, and the three parameter gradients
  double *adj_lam = nullptr, *adj_gpv = nullptr, *adj_gdt = nullptr, *adj_gpar = nullptr;
};

// ------------------------------------------------------------------ index helpers
__device__ __forceinline__ int find_block_interior(const BlockGeom* B, int nb, long long t) {
  int b = 0;
  while (b + 1 < nb && t >= B[b + 1].int_off) ++b;
  return b;
}
__device__ __forceinline__ int find_block_cell(const BlockGeom* B, int nb, long long g) {
  int b = 0;
  while (b + 1 < nb && g >= B[b + 1].off) ++b;
  return b;
}
// The heat flux of a history at time tm (bcheatfluxwall*, src/bc_module.f90:4026-4033):
// linear between the bracketing entries, the last value from the last time on.  Before the
// first time the reference leaves it undefined; the first value is taken there.
__device__ __forceinline__ double heatflux_at(const double* tab, double tm) {
  const int nd = (int)tab[0];
  const double* t = tab + 1;
  const double* q = tab + 1 + nd;
  double hf = q[0];
  for (int i = 0; i < nd - 1; ++i)
    if (tm >= t[i] && tm < t[i + 1]) {
      hf = q[i] + (q[i + 1] - q[i]) * (tm - t[i]) / (t[i + 1] - t[i]);
      break;
    }
  if (tm >= t[nd - 1]) hf = q[nd - 1];
  return hf;
}

// the acceleration of the gravity history at tm (gravity%getgravitysource,
// src/gravity_module.f90:110-125): linear between the bracketing rows, the last row from
// its time on; before the first time (undefined in the reference) the first row
__device__ __forceinline__ void gravity_at(const double* tab, double tm, double* a) {
  const int nd = (int)tab[0];
  const double* t = tab + 1;
  const double* g = tab + 1 + nd;
  for (int e = 0; e < 3; ++e) a[e] = g[e];
  for (int i = 0; i < nd - 1; ++i)
    if (tm >= t[i] && tm < t[i + 1]) {
      for (int e = 0; e < 3; ++e) a[e] = g[3 * i + e] + (g[3 * (i + 1) + e] - g[3 * i + e]) * (tm - t[i]) / (t[i + 1] - t[i]);
      break;
    }
  if (tm >= t[nd - 1])
    for (int e = 0; e < 3; ++e) a[e] = g[3 * (nd - 1) + e];
}

// the time bc%setbc receives (bcinfo%time): dt_phy nt_phy when unsteady, else the
// accumulated pseudo time including this iteration's minimum step (no step taken yet in a
// residual-only evaluation), plus timeprev
__device__ __forceinline__ double bc_time(const DevPtr& d, const Par& c) {
  if (c.nsteady >= 1) return c.dt_phy * (double)d.sc->nt_phy;
  const unsigned long long bits = d.sc->dtmin_bits;
  const double dtm = (bits == (unsigned long long)__double_as_longlong(1.0e10)) ? 0.0 : __longlong_as_double((long long)bits);
  return d.sc->time_acc + dtm + d.sc->timeprev;
}

__device__ __forceinline__ long long interior_cell(const BlockGeom& B, long long loc, int& i, int& j, int& k) {
  int ni = B.imax - 1, nj = B.jmax - 1;
  i = (int)(loc % ni) + 2;
  long long r = loc / ni;
  j = (int)(r % nj) + 2;
  k = (int)(r / nj) + 2;
  return B.off + (i + 1) + (long long)B.ni * ((j + 1) + (long long)B.nj * (k + 1));
}

__device__ __forceinline__ void face_vec(const DevPtr& d, int plane, long long g, double* o) {
  o[0] = d.gm[(plane + 0) * d.ncell + g];
  o[1] = d.gm[(plane + 1) * d.ncell + g];
  o[2] = d.gm[(plane + 2) * d.ncell + g];
}

// stencil cell l (0..37) of a face at left cell g: normal stride sn, transverse s1, s2
__device__ __forceinline__ long long stencil_cell(int l, long long g, long long sn, long long s1, long long s2) {
  if (l < 18) {
    int a = l & 1, t1 = (l >> 1) % 3 - 1, t2 = l / 6 - 1;
    return g + a * sn + t1 * s1 + t2 * s2;
  }
  if (l < 36) {
    int m = (l - 18) % 9;
    int a = (l < 27) ? -1 : 2;
    int t1 = m % 3 - 1, t2 = m / 3 - 1;
    return g + a * sn + t1 * s1 + t2 * s2;
  }
  return g + ((l == 36) ? -2 : 3) * sn;
}


// cells per chunk of the dataflow sweeps (one CTA's work item)
constexpr int SW_CH = 32;

// face-flux launchers (flux.cu: FP64 form; flux_mixed.cu: mixed form)
void launch_face_flux(const Engine& E, cudaStream_t s);
void launch_face_flux_mixed(const Engine& E, cudaStream_t s, int b0, int b1);
// discrete adjoint (adjoint.cu): buffers (allocated once, zeroed per call), the reverse
// pass, and release
int adjoint_buffers(Engine& E);
int adjoint_launch(Engine& E);
void adjoint_free(Engine& E);

// host entry points implemented in setup.cu
bool setup_geometry(Engine& E, const cfd3d_block_desc* blocks, int nblocks);
bool setup_ghost_program(Engine& E, const cfd3d_block_desc* blocks, int nblocks);
void setup_planes(Engine& E);
bool setup_vfg_halo(Engine& E, const cfd3d_block_desc* blocks, int nblocks);
bool setup_tiles(Engine& E);

#define CFD_CUDA(call)                                                                 \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      E.err = std::string(#call) + ": " + cudaGetErrorString(e_);                      \
      return CFD3D_ERR_CUDA;                                                           \
    }                                                                                  \
  } while (0)

}  // namespace cfd
