/*
 * cfd3d.h -- C ABI of the GB300-native pseudo-iteration engine (libcfd3d_gb300.so).
 *
 * The engine replaces one hot path of kwonhwi1/3dcode: the per-pseudo-iteration
 * LU-SGS update `t_update%timeinteg` (src/update_module.f90:37-52, implementation
 * `lusgs` :455-733) together with the convergence residual `t_resi%setqres/residual`
 * (src/residual_module.f90:94-186), as called from `solve_equation`
 * (src/solve_module.f90:133-136).  A Fortran caller binds these entry points through
 * ISO_C_BINDING interfaces; Python binds them through ctypes.
 *
 * Conventions
 *  - Plain pointers and sizes only.  All arrays are FP64 in the reference's Fortran
 *    storage order (first index fastest).
 *  - Block sizes imax/jmax/kmax are NODE counts per direction, exactly as the
 *    reference's grid module reads them (src/grid_module.f90:107-116); interior cells
 *    are i = 2..imax, the padded cell range is -1..imax+3 (src/variable_module.f90:69-71).
 *  - Every entry point returns CFD3D_OK (0) or a CFD3D_ERR_* code; the message of the
 *    last failure is available through cfd3d_last_error().  No exception crosses the ABI.
 *  - One host thread per handle.  The handle owns every device buffer, its CUDA stream
 *    and its CUDA graphs; host arrays stay owned by the caller.
 */
#ifndef CFD3D_H
#define CFD3D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------ */
#define CFD3D_OK               0
#define CFD3D_ERR_ARG          1   /* bad argument or unsupported option            */
#define CFD3D_ERR_CUDA         2   /* a CUDA runtime call failed                     */
#define CFD3D_ERR_NONFINITE    3   /* NaN/Inf detected in the updated state          */
#define CFD3D_ERR_VOLUME       4   /* zero or negative cell volume in the grid       */
#define CFD3D_ERR_TIMEOUT      5   /* a bounded device wait ran out                  */
#define CFD3D_ERR_DESCRIPTOR   6   /* inconsistent block / BC / connection descriptor */
#define CFD3D_ERR_NOMEM        7   /* device allocation failed                       */
#define CFD3D_ERR_NODEVICE     8   /* no CUDA device is visible                      */
#define CFD3D_ERR_IO           9   /* a checkpoint file could not be opened, read or written */

/* ---- arithmetic forms ---------------------------------------------------------- */
#define CFD3D_FP64   0   /* every kernel in FP64 (the reference's arithmetic)        */
#define CFD3D_MIXED  1   /* FP32 reconstruction/limiter/flux, FP64 EOS mixture,
                            accumulation, diagonal inversion and update             */

/* ---- boundary-condition kinds (names of the CGNS BC families the reference
 *      dispatches on, src/bc_module.f90:221-335) -------------------------------- */
#define CFD3D_BC_WALL         1   /* BCWall: inviscid / viscous / SST wall by iturb   */
#define CFD3D_BC_SYMMETRY     2   /* BCSymmetryPlane                                  */
#define CFD3D_BC_FARFIELD     3   /* BCFarfield (characteristic, with EOS)            */
#define CFD3D_BC_EXTRAPOLATE  4   /* BCExtrapolate / BCOutflowSupersonic              */
#define CFD3D_BC_DEGENERATE   5   /* BCDegeneratePoint / BCDegenerateLine             */
#define CFD3D_BC_INFLOW       6   /* BCInflow (the reference's routine is a no-op)    */
#define CFD3D_BC_INFLOW_SUBSONIC    7   /* BCInflowSubsonic: characteristic, free-stream state */
#define CFD3D_BC_OUTFLOW_SUBSONIC   8   /* BCOutflowSubsonic: characteristic, p = pref        */
#define CFD3D_BC_INFLOW_SUPERSONIC  9   /* BCInflowSupersonic: free-stream state imposed      */
#define CFD3D_BC_OUTFLOW           10   /* BCOutflow (the reference's routine is a no-op)     */
#define CFD3D_BC_WALL_COUNTERROTATING 11 /* BCWall of family CounterRotating                 */
#define CFD3D_BC_WALL_HEATFLUX     12   /* BCWall of family HeatFlux*: q(t) from the patch's table */
#define CFD3D_BC_MASSFLOWRATE_IN   13   /* BCMassflowrateIn (mass-flow rate 0, as constructed) */
#define CFD3D_BC_SHIFTED_PERIODIC  14   /* BCShiftedPeriodic (the reference's 16-cell shift)   */
#define CFD3D_BC_TOTALPRESSURE_IN  15   /* BCTotalPressureIn (the reference's fixed totals)    */

/* Solver configuration: the fields of the reference's input.inp
 * (src/config_module.f90:100-119, documented in bin/input_templet.inp:34-66). */
typedef struct cfd3d_config {
  int    nsteady, npmax, ntmax, bond;   /* 0 steady, 1 BDF1, 2 BDF2                */
  double dt_phy;
  int    iturb, ides;                   /* -3 Euler, -2 laminar, 0 k-omega SST      */
  int    nscheme, nmuscl, nlim;         /* flux, reconstruction, limiter            */
  int    timemethod, local, prec;       /* 1 Euler, 2 RK3, 3 LU-SGS; local; prec    */
  double cfl;
  int    fluid, ngas;                   /* 1 stiffened water, 2 IAPWS-97; 1 ideal gas */
  int    ncav;                          /* 0 none, 1 Merkle ... 5 Lee               */
  double c_v, c_c;
  double pref, uref, aoa, aos, tref, y1ref, y2ref;   /* aoa, aos in degrees       */
  double l_chord, l_character, scale, l_domain;
  /* extensions (0 keeps the reference's behaviour) */
  int    fix_cav_clamp;   /* 1: clamp r_c by rho*y1 and r_v by rho*(1-y1-y2)
                             instead of the reference's temperature-indexed clamp */
  int    precision;       /* CFD3D_FP64 or CFD3D_MIXED                            */
  double kinf, oinf;      /* >0: replace the SST free-stream k / omega that
                             config%setref derives (src/config_module.f90:186-189) */
  /* the gravity source rhs%gravity (src/gravity_module.f90:24-133): 0 none; +-1, +-2, +-3 a
     constant +-9.80665 m/s^2 along x, y, z; 4 the history of gravity.dat, given here as
     ngravity rows (t, gx, gy, gz) with t ascending */
  int    gravity, ngravity;
  const double *gravity_data;
  /* the surface-tension source rhs%csf (src/csf_module.f90:97-175): 0 none, 1 on */
  int    csf;
  /* the rotating frame (src/rotation_module.f90, src/config_module.f90:126-141): rotation
     0 none, +-1, +-2, +-3 about +-x, +-y, +-z at rpm revolutions per minute */
  int    rotation;
  double rpm;
} cfd3d_config;

/* A boundary patch: CGNS PointRange in 1-based NODE indices
 * (imin, jmin, kmin, imax, jmax, kmax), one index pair collapsed to a face.
 * CFD3D_BC_WALL_HEATFLUX also carries the heat-flux history that the reference reads from
 * <family>.dat (src/bc_module.f90:233-249): ndata pairs (tdata[m], heatflux[m]), tdata
 * ascending; the other types leave ndata = 0 and the pointers NULL. */
typedef struct cfd3d_bc_patch {
  int type;
  int pnts[6];
  int ndata;
  const double *tdata, *heatflux;
} cfd3d_bc_patch;

/* A point-matched 1-to-1 interface, as cg_1to1_read_f returns it: own range,
 * donor range (1-based node indices) and the transform vector. */
typedef struct cfd3d_connection {
  int donor;            /* 0-based block index of the neighbouring block */
  int pnts[6];
  int pnts_donor[6];
  int transform[3];
} cfd3d_connection;

typedef struct cfd3d_block_desc {
  int imax, jmax, kmax;             /* node counts                                   */
  const double *xyz;                /* node coordinates x(3, imax, jmax, kmax)        */
  int nbc;
  const cfd3d_bc_patch *bc;
  int ncon;
  const cfd3d_connection *con;
} cfd3d_block_desc;

typedef struct cfd3d_handle cfd3d_handle;

/* Build the engine: config%construct + grid%construct + variable%construct +
 * update%construct (src/main.f90:15-35).  Computes the metrics, the wall distance,
 * the BC/edge/corner ghost programs and the halo copy lists, and allocates every
 * device buffer.  Replaces: src/config_module.f90:90-165, src/grid_module.f90:75-332,
 * src/update_module.f90:77-178, src/bc_module.f90:71-1188. */
int  cfd3d_create(const cfd3d_config *cfg, int nblocks, const cfd3d_block_desc *blocks,
                  cfd3d_handle **out);
void cfd3d_destroy(cfd3d_handle *h);
const char *cfd3d_last_error(const cfd3d_handle *h);

/* Derived sizes (config%getnpv/getndv/getntv/getnqq, grid%getngrd). */
int  cfd3d_sizes(const cfd3d_handle *h, int *npv, int *ndv, int *ntv, int *nqq, int *ngrd);

/* Initial state: t_ini_initial + set_others (src/initial_module.f90:678-771).
 * pv_interior == NULL gives the uniform free stream; otherwise it holds
 * pv(npv, 2:imax, 2:jmax, 2:kmax) (k and omega are taken from it when iturb = 0). */
int  cfd3d_initialize(cfd3d_handle *h, int block, const double *pv_interior);

/* Copy a full padded state in/out: pv(npv,-1:imax+3,..), dv(ndv,..), tv(ntv,..),
 * qq(npv,nqq,2:imax,..) and (out only) rcav(2,2:imax,..).  Any pointer may be NULL.
 * Pinned (page-locked) host arrays move at the link's full rate. The handle keeps one
 * device staging region per array, (npv+ndv+ntv) padded + (2 npv+2) interior doubles
 * per cell of the largest block, so that the layout change of one array overlaps the copy
 * of the next. Both calls return after every copy has finished.
 * Replaces the accessors t_variable%getpv/setpv.. (src/variable_module.f90:22-39). */
int  cfd3d_upload_state(cfd3d_handle *h, int block, const double *pv, const double *dv,
                        const double *tv, const double *qq);
int  cfd3d_download_state(cfd3d_handle *h, int block, double *pv, double *dv, double *tv,
                          double *qq, double *rcav);

/* Set a block's state from its primitives alone: pv(npv,-1:imax+3,..) padded as
 * cfd3d_upload_state takes it, and qq(npv,nqq,2:imax,..) (NULL keeps the history on the
 * device).  dv and tv of the interior follow from pv as the update sets them: the mixture
 * EOS with transport properties (eos%deteos, src/update_module.f90:689) and the eddy
 * viscosity (src/update_module.f90:701-732, reading the uploaded ghost pv), so the result
 * equals a cfd3d_upload_state of pv, dv, tv that an iteration produced.  A caller that
 * keeps the state on the host moves pv and qq instead of pv, dv, tv and qq.  Ghost cells
 * are set by the next iteration's boundary program.  No counterpart in the reference (its
 * state never leaves the host); it serves the drop-in mode's per-step upload. */
int  cfd3d_upload_primitives(cfd3d_handle *h, int block, const double *pv, const double *qq);

/* The two transfers of the drop-in mode for every block in one call: pv[b] (and qq[b],
 * either array or any entry may be NULL) for block b = 0..nblocks-1 as cfd3d_upload_primitives
 * takes them, and pv / dv / tv of every block as cfd3d_download_state gives them (NULL arrays
 * or entries are skipped).  The copies of all blocks leave back to back at the link's rate
 * and each block's layout kernel overlaps the copies of the blocks after it; the results
 * equal the per-block calls'.  The upload runs the EOS only for the cells whose uploaded pv
 * differs from the device's (an unchanged cell's dv and tv already are the EOS of its pv),
 * and the eddy viscosity only when some pv changed.  The handle's staging region grows to
 * the case's whole state.  No counterpart in the reference (its state never leaves the
 * host). */
int  cfd3d_upload_primitives_all(cfd3d_handle *h, const double *const *pv, const double *const *qq);
int  cfd3d_download_state_all(cfd3d_handle *h, double *const *pv, double *const *dv, double *const *tv);

/* With the surface-tension source (csf = 1): csf(3, 2:imax, 2:jmax, 2:kmax) of one block, the
 * momentum source of the last residual (its volume included), as calrhs stores it in
 * variable%csf (src/rhs_module.f90:632-634) for export_variable.  CFD3D_ERR_ARG without csf.
 * Replaces t_variable%getcsf-style access to variable%csf (src/variable_module.f90:21). */
int  cfd3d_download_csf(cfd3d_handle *h, int block, double *csf);

/* Checkpoint file out_########.dat in the layout of variable%export_variable
 * (src/variable_module.f90:116-182), native byte order: one record per block, in block
 * order (rank r of the reference owns block r), each record
 *   int32 nt_phy, int32 nt, float64 time,
 *   pv(npv, -1:imax+3, -1:jmax+3, -1:kmax+3),
 *   emut(-1:imax+3, ..) = tv(3, ..)        when iturb >= -1,
 *   qq(npv, nqq, 2:imax, 2:jmax, 2:kmax),
 *   rcav(2, 2:imax, ..)                    when ncav != 0.
 * The file is created when missing and not truncated (mpi_mode_wronly+mpi_mode_create). */
int  cfd3d_checkpoint_write(cfd3d_handle *h, const char *path, int nt_phy, int nt, double time);

/* Restart from such a file: t_ini_restart%restart (src/initial_module.f90:245-389).  The
 * interior pv is read, dv and tv follow from the EOS, tv(3) from emut, qq and rcav from the
 * file.  Returns the loop counters the solve loop restarts from: nps = nt_phy + 1 and
 * nts = 1 for unsteady runs, nts = nt + 1 and nps = 1 for steady ones, and the stored time.
 * steady_start != 0 reads the steadyini variant (:103-242): records without qq, qq rebuilt
 * from the state, nps = nts = 1, timeprev = 0.  A file shorter than the case's records
 * returns CFD3D_ERR_IO. */
int  cfd3d_checkpoint_read(cfd3d_handle *h, const char *path, int steady_start, int *nps, int *nts,
                           double *timeprev);

/* One pseudo-iteration: resi%setqres + update%timeinteg + resi%residual, timeinteg being
 * LU-SGS (timemethod 3), explicit Euler (1) or RK3 (2) (src/update_module.f90:214-733)
 * (src/solve_module.f90:134-136).  Outputs the solution time, the L2 norms
 * res_l2[npv] of the state change, and the location (block,i,j,k) of the largest
 * pressure change.  Any output pointer may be NULL. */
int  cfd3d_iterate(cfd3d_handle *h, int nt_phy, int nt, double timeprev, double *time_out,
                   double *res_l2, int *resmax_loc);

/* niter pseudo-iterations back to back on the device (CUDA-graph replays), with one
 * host synchronisation at the end; res_l2 receives the norms of the last one. */
int  cfd3d_iterate_n(cfd3d_handle *h, int niter, int nt_phy, int nt0, double timeprev,
                     double *time_out, double *res_l2);

/* Physical-time BDF history shift: solve%unsteadyupdate (src/solve_module.f90:155-183). */
int  cfd3d_unsteady_shift(cfd3d_handle *h);

/* Ghost fill + residual only (bc%setbc + rhs%calrhs, src/rhs_module.f90:260-643) on the
 * current state, without updating it: res(npv,2:imax,..), icav(4,..), itt(4,..),
 * omega_cut(2:imax,..).  Pointers may be NULL. */
int  cfd3d_residual(cfd3d_handle *h, int block, double *res, double *icav, double *itt,
                    double *omega_cut);

/* Discrete adjoint of the FP64 residual: the vector-Jacobian product of R(pv), the
 * residual of cfd3d_residual on the current state as a function of the interior pv of all
 * blocks, with each interior cell's dv and tv(1:2) its EOS (as the update sets them) and
 * the eddy viscosity tv(3) and the history qq held.  cot and g_state are res-shaped,
 * (npv,2:imax,2:jmax,2:kmax) per block, blocks concatenated in order: g_state = (dR/dpv)^T cot.
 * g_params[3] = cot . dR/d(uref, c_v, c_c), uref the free-stream speed at fixed angles and
 * fixed k_inf / omega_inf.  Limiter, clip and flux switches are recomputed from the state;
 * nothing is taped.  g_state and g_params may be NULL.  No counterpart in the reference:
 * it serves gradient checks of the residual. */
int  cfd3d_residual_vjp(cfd3d_handle *h, const double *cot, double *g_state, double *g_params);

/* Launch-shape autotuner (no counterpart in the reference).  On the current state it
 * times, with CUDA events over `reps` calls each, the face-flux kernels and the residual
 * kernel at 64, 128 and 256 threads per CTA, the mixed form's face / residual pipeline at
 * 1, 2, 4, ... block groups and the sweeps at 1, 2, 3, 4, 6, ... persistent CTAs per SM (up
 * to the occupancy limit), keeps the fastest of each, and re-captures the
 * iteration graph at the next iteration.  choice (may be NULL) receives the threads per
 * CTA of the face and residual kernels and the sweep CTAs per SM.  Results do not depend on
 * the shapes: each thread's arithmetic is unchanged. */
int  cfd3d_autotune(cfd3d_handle *h, int reps, int *choice);

/* Self-test of the float <-> double conversions the mixed form runs on the integer pipes
 * (no counterpart in the reference; on a GB300 the hardware conversions take FP64-pipe
 * slots): n seeded bit patterns -- random ones over the double range, exact halfway cases,
 * the ends of the float range, signed zeros, ordinary magnitudes -- converted by them and by
 * the hardware.  mismatches[0] / [1] receive the number of double -> float / float -> double
 * results whose bits differ (0 expected). */
int  cfd3d_convert_selftest(long long n, unsigned long long seed, long long *mismatches);

/* The launch shapes in use (no counterpart in the reference): shapes[0..3] receive the
 * threads per CTA of the face and residual kernels, the sweep CTAs per SM, and the number
 * of block groups over which the mixed form pipelines its face stage and residual (the
 * residual of one group beside the face stage of the next, on a second stream; 1 = none).
 * The autotuner chooses all four; results do not depend on them. */
int  cfd3d_launch_shapes(const cfd3d_handle *h, int *shapes);
/* Sets the four launch shapes of cfd3d_launch_shapes (for instance those a tuning run
 * found): threads per CTA 64, 128 or 256; sweep CTAs per SM from 1 to the occupancy limit;
 * pipeline groups from 1 to min(blocks, 16), 1 in the FP64 form.  CFD3D_ERR_ARG otherwise,
 * with nothing changed.  The iteration graph is re-captured at the next iteration. */
int  cfd3d_set_launch_shapes(cfd3d_handle *h, const int *shapes);

/* Test hook of the dataflow sweeps' bounded waits (no counterpart in the reference): one
 * forward sweep on the current state's records in which the first chunk of cells never
 * signals completion, with a short wait limit.  The cells that depend on it give up
 * waiting, the launch completes and the call returns CFD3D_ERR_TIMEOUT with the device
 * context intact; the state is not updated. */
int  cfd3d_sweep_stall_test(cfd3d_handle *h);

/* Grid metrics as the reference stores them: cx(3,1:imax,1:jmax+1,1:kmax+1),
 * ex(3,1:imax+1,1:jmax,1:kmax+1), tx(3,1:imax+1,1:jmax+1,1:kmax),
 * grd(ngrd,1:imax+1,1:jmax+1,1:kmax+1) (src/grid_module.f90:609-1241). */
int  cfd3d_grid_metrics(cfd3d_handle *h, int block, double *cx, double *ex, double *tx,
                        double *grd);

/* Pointwise mixture EOS on the device: eos%deteos_simple (with_prop = 0) or
 * eos%deteos with transport properties (with_prop = 1)
 * (src/eos_module.f90:1064-1234).  Host arrays of n points; dv is dv(18, n),
 * tv is tv(2, n) (may be NULL when with_prop = 0). */
int  cfd3d_eos_eval(int fluid, int ngas, int with_prop, int64_t n, const double *p,
                    const double *t, const double *y1, const double *y2, double *dv,
                    double *tv);

/* cfd3d_eos_eval without any device allocation: the points pass through one static
 * device buffer of CFD3D_EOS_NOALLOC_MAX points (about 0.8 MB of each context that loads
 * the library's device code, held until the context ends) instead of cudaMalloc'd arrays.  No counterpart in the reference.  It serves
 * callers that cannot allocate device memory: a caller evaluating a few points while the
 * engine's iterations run on their own stream (cudaFree synchronises the whole device,
 * so cfd3d_eos_eval would wait for them), and a caller whose device memory is taken by
 * a large case or by another allocator's pool (cudaMalloc would fail).  Same arguments
 * and results as cfd3d_eos_eval.  n > CFD3D_EOS_NOALLOC_MAX returns CFD3D_ERR_ARG before
 * any device work.  The first call in a context (a device's primary context, or a new
 * one after cudaDeviceReset) looks up the buffer's device address, so make it before any
 * stream capture there.  Under lazy module loading (the CUDA default) that first call is
 * also when the buffer is reserved: make it while device memory is still free, or load
 * modules eagerly (CUDA_MODULE_LOADING=EAGER).  All calls on one device share the buffer:
 * calls must not overlap (serialise them across host threads). */
#define CFD3D_EOS_NOALLOC_MAX 4096
int  cfd3d_eos_eval_noalloc(int fluid, int ngas, int with_prop, int64_t n, const double *p,
                            const double *t, const double *y1, const double *y2, double *dv,
                            double *tv);

/* Device-side statistics of the last iterate call: how many EOS evaluations took
 * the reference's "alternative calculation for snd2" branch
 * (src/eos_module.f90:1104-1111), and the kernel launches of one iteration. */
int  cfd3d_stats(const cfd3d_handle *h, int64_t *snd2_fallbacks, int *launches_per_iter);

/* Select the CUDA device used by the handles created afterwards on the calling thread
 * (one GPU per process; the reference's MPI rank -> GPU mapping). */
int  cfd3d_set_device(int device);

/* Timing on the handle's own stream (CUDA events, graph replays): milliseconds for
 * niter back-to-back pseudo-iterations.  No reference counterpart (measurement only). */
int  cfd3d_time_iterate(cfd3d_handle *h, int niter, double *ms);

/* One pseudo-iteration launched stage by stage with CUDA events between the stages (the
 * mixed form's face / residual pipeline off, so that the two are timed apart);
 * stage_ms[CFD3D_NSTAGES] receives: time step, boundary program, face fluxes, residual
 * + sources, forward sweep, backward sweep, update + EOS, eddy + norms.
 * No reference counterpart (measurement only). */
#define CFD3D_NSTAGES 8
int  cfd3d_profile_iterate(cfd3d_handle *h, double *stage_ms);

/* FP64 throughput of the current device in TFLOP/s: every thread of a full grid runs
 * independent fused multiply-add chains on doubles for about `seconds` (at most 60),
 * timed with CUDA events.  The denominator of the FP64 compute roofline of this path's
 * kernels.  No reference counterpart (measurement only). */
int  cfd3d_fp64_peak(double seconds, double *tflops);

/* Throughput of float <-> double conversions on the current device, in G conversions/s:
 * rates[0] / [1] double -> float by the hardware / on the integer pipes (the mixed form's),
 * rates[2] / [3] float -> double likewise; 2^24 threads of 64 conversions each, timed with
 * CUDA events.  No reference counterpart (measurement only). */
int  cfd3d_convert_rate(double *rates);

#ifdef __cplusplus
}
#endif
#endif /* CFD3D_H */
