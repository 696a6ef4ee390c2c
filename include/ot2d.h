/*
 * ot2d.h -- C ABI of the GB300-native OVERTURNS-2D hot path
 * (library libturns2d_gb300.so, sm_103a).
 *
 * Two layers:
 *
 * 1. Drop-in routines (ot2d_rhsup, ot2d_visrhs, ot2d_ilu2d, ...).  Each one
 *    replaces one Fortran subroutine of the reference and takes the same
 *    arguments in the same order: every argument by reference, arrays in the
 *    reference's column-major layout (q(jd,kd,nq) for one time instance of
 *    q(jd,kd,nspec,nq) -- see OT2D_QSTRIDE below).  The module-level inputs
 *    the reference reads from `params_global` are set once per mesh with
 *    ot2d_set_params().  Pointers may be host memory (copied in and out
 *    around the call), host memory registered with ot2d_register() (its
 *    device mirror is used; no copy), or device memory (used in place).
 *    Every routine returns an int status (0 = OK); ot2d_last_error() repeats
 *    the last non-zero status of the calling thread.
 *
 * 2. A batched solver (ot2d_solver_*): many meshes of uneven size resident
 *    in HBM, one launch per kernel family per iteration over all of them,
 *    FP64 plain or FP32-mixed arithmetic, per-instance convergence.
 *
 * Nothing here allocates memory the caller must free, except the solver
 * handle (ot2d_solver_destroy).
 */
#ifndef OT2D_H
#define OT2D_H

#include <stddef.h>
#include <stdint.h>
#include "ot2d_params.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define OT2D_OK            0
#define OT2D_ERR_ARG       1   /* bad argument / unsupported switch combination      */
#define OT2D_ERR_NORM      2   /* L2 norm > 1000: the reference's `stop 'norm'`      */
#define OT2D_ERR_MONITOR   3   /* negative a^2 or NaN: the reference's mstop         */
#define OT2D_ERR_CUDA      4   /* a CUDA call failed                                 */
#define OT2D_ERR_NOPARAMS  5   /* no ot2d_set_params() before a drop-in routine      */
#define OT2D_ERR_NOMEM     6   /* device allocation failed                           */
#define OT2D_ERR_TIMEOUT   7   /* a bounded device wait gave up                      */
#define OT2D_ERR_IO        8   /* a file could not be opened / read / written, or a
                                  record is shorter than the data it should hold      */

/* precision modes of the solver and of the drop-in routines */
#define OT2D_FP64          0   /* plain FP64, operation order of the reference       */
#define OT2D_FP32_MIXED    1   /* FP32 residual/Jacobian/sweeps, FP64 state update   */

/* ---------------------------------------------------------------------- */
/* set-up (host)                                                           */
/* ---------------------------------------------------------------------- */

/* read_inputs derived constants + set_pointers_globals
 * (src/setup.f:876-1268, src/setup.f:55-108, src/init.f:59-66). */
int ot2d_params_from_inputs(const ot2d_inputs* in, ot2d_params* out);
/* single C-mesh &bcinp table: wall(5), wake(51), far field(47) x3. */
int ot2d_cmesh_bc_table(ot2d_inputs* in, int32_t jtail);
/* seeded algebraic NACA 4-digit C-mesh standing in for fort.1
 * (read by grid, src/io.f:343-380). */
int ot2d_mesh_naca4_cmesh(int32_t jmax, int32_t kmax, int32_t n_wake, double m, double p, double t,
                          double ds_wall, double r_far, double* xv, double* yv);

/* ---------------------------------------------------------------------- */
/* drop-in layer (one call = one reference subroutine)                     */
/* ---------------------------------------------------------------------- */

/* module params_global for the calling thread's current mesh
 * (replaces set_pointers_globals + the namelist state, src/setup.f:55-108). */
int ot2d_set_params(const ot2d_params* p);
/* precision of the drop-in routines (default OT2D_FP64). */
int ot2d_set_precision(int32_t mode);
/* last non-zero status returned on this thread. */
int ot2d_last_error(void);
/* device residency: keep `bytes` at host pointer `h` mirrored on the GPU.
 * Drop-in calls that receive `h` use the mirror without copying; call
 * ot2d_sync_to_host / ot2d_sync_to_device around host-side reads/writes. */
int ot2d_register(void* h, size_t bytes);
int ot2d_unregister(void* h);
int ot2d_sync_to_host(void* h);
int ot2d_sync_to_device(void* h);

/* src/eulerrhs.f:2-3 */
int ot2d_rhsup(double* q, double* s, double* xx, double* xy, double* yx, double* yy, double* x, double* y,
               double* xv, double* yv, double* xold, double* yold, double* xole, double* yole, int32_t* iblank,
               double* ugv, double* vgv, int32_t* jd, int32_t* kd, int32_t* nei, int32_t* im, double* bt);
/* src/visrhs.f:2-3 */
int ot2d_visrhs(double* turmu, double* q, double* s, double* xx, double* xy, double* yx, double* yy, double* ug,
                double* vg, double* tscale, int32_t* iblank, int32_t* jd, int32_t* kd);
/* src/bc.f:2 */
int ot2d_bc(double* q, double* x, double* y, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
            int32_t* im, int32_t* jd, int32_t* kd, double* bt);
/* src/bc.f:88 */
int ot2d_rbc(double* q, double* s, double* x, double* y, double* xx, double* xy, double* yx, double* yy, double* ug,
             double* vg, int32_t* im, int32_t* jd, int32_t* kd, double* bt);
/* src/time.f:2 (one time instance per call when nspec = 1) */
int ot2d_time_step(double* q, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
                   double* tscale, double* bt, int32_t* iblank, int32_t* jd, int32_t* kd);
/* src/lhs.f:470-471 */
int ot2d_ilu2d(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
               double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* turmu,
               double* tscale);
/* src/lhs.f:2-3: ilu2d with Turkel's low-Mach preconditioner (bSq =
 * Mp**2/(bt - Mp**2 (bt-1)) per cell, Mp from the params whatever iprecon
 * says); bt as time_step wrote it */
int ot2d_preilu2d(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
                  double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* turmu,
                  double* tscale, double* bt);
/* src/sources.f:97: the residual s(1:4) of the interior cells multiplied by
 * the low-Mach preconditioner */
int ot2d_rhslom(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
                double* bt);
/* src/lhs.f:817-818: pentadiagonal lhsinv (lhs.f:1536-1816), or the
 * upwind-split lhsinv_up (lhs.f:1333-1533) when params ilhs = 3 */
int ot2d_arc2d(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks, int32_t* ke,
               double* xx, double* xy, double* yx, double* yy, double* ug, double* vg, double* turmu, int32_t* iblank,
               double* tscale, double* bt);
/* src/lhs.f:1060-1061: arc2d with Turkel's preconditioned eigenvectors in
 * the T_xi^-1, N^-1 and T_eta transforms (bSq per cell from bt and the
 * params' Mp whatever iprecon says); line inversions as ot2d_arc2d */
int ot2d_arc2d_precon(double* q, double* s, int32_t* jd, int32_t* kd, int32_t* js, int32_t* je, int32_t* ks,
                      int32_t* ke, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
                      double* turmu, int32_t* iblank, double* tscale, double* bt);
/* src/connectivity.f:2-3: overset interpolation of q between the meshes of
 * one grid system (the donor / fringe lists of the reference's connectivity,
 * 1-based, Fortran-ordered; qg holds each mesh's q(jmx,kmx,nspec,nq) one
 * after another).  Every donor is gathered before any fringe cell is
 * written; a fringe cell listed twice takes its last entry.  Donor stencils
 * must lie inside their mesh and rows inside qbc (OT2D_ERR_ARG otherwise). */
int ot2d_do_interpolations(double* qg, int32_t* jmx, int32_t* kmx, int32_t* ibcg, int32_t* imeshg, int32_t* idonorg,
                           double* fracg, int32_t* nfringeg, int32_t* ndonorg, int32_t* iisptrg, int32_t* iieptrg,
                           int32_t* idsize, int32_t* qsize, int32_t* nmesh);
/* src/samodel2d.f:2-3 */
int ot2d_vmu_sa(double* q, double* s, double* turmu, double* x, double* y, double* xv, double* yv, double* xx,
                double* xy, double* yx, double* yy, double* ug, double* vg, int32_t* jd, int32_t* kd,
                double* tscale, int32_t* iblank, int32_t* im, int32_t* nsp);
/* src/komegasst.f:2-3 (no transition model: itrans = 0) */
int ot2d_komegasst(double* q, double* s, double* turmu, double* x, double* y, double* xv, double* yv, double* xx,
                   double* xy, double* yx, double* yy, double* ug, double* vg, int32_t* jd, int32_t* kd,
                   double* tscale, int32_t* iblank, int32_t* im);
/* src/sources.f:2 (q, s: full (jd,kd,nspec,nv) arrays) */
int ot2d_timespectralrhs(double* q, double* s, double* Ds, int32_t* jd, int32_t* kd, int32_t* nsp);
/* src/step.f:2-7 (full arrays over nspec; norms of the last call via
 * ot2d_last_norms).  Time accurate (iunst = 1): xold..yole give the
 * swept-area face speeds and ug, vg the cell grid speeds; itnmax > 1: qnewt
 * gives newton's physical-time term (time.f:178-210), or with the time-spectral
 * form newtonTS's pseudo-time term (time.f:213-241, added after the norms).
 * iprecon:
 * roetrklflx fluxes, rhslom after the norms and preilu2d or arc2d_precon,
 * all reading bt, which must then be given. */
int ot2d_step(double* q, double* qtn, double* qtnm1, double* qnewt, double* s, double* x, double* y, double* xv,
              double* yv, int32_t* iblank, double* xx, double* xy, double* yx, double* yy, double* ug, double* vg,
              double* ugv, double* vgv, double* xold, double* yold, double* xole, double* yole, double* turmu,
              double* tscale, double* bt, double* Ds, int32_t* im, int32_t* jd, int32_t* kd);
/* rsum, resrho, resmax per time instance of the last ot2d_step (step.f:58-93) */
int ot2d_last_norms(double* out, int32_t n);
/* src/step.f:332 */
int ot2d_monitor(int32_t* mstop, double* q, int32_t* jd, int32_t* kd);
/* src/forces.f:130-131; the four outputs are the raw integrals */
int ot2d_force2d(int32_t* jd, int32_t* kd, double* x, double* y, double* xv, double* yv, double* q, double* xx,
                 double* xy, double* yx, double* yy, double* cfx, double* cfy, double* cm0, double* cpower,
                 int32_t* nsp);
/* src/motion.f:546-632 (pitch, motiontype 1): rotates x, y (cell centres)
 * and xv, yv by step istep's increment, shifts xold/xole, sets ug, vg; the
 * step's sines and cosines are taken on the host, the rest runs on the
 * device */
int ot2d_pitch(int32_t* init, double* x, double* y, double* xv, double* yv, double* xold, double* yold, double* xole,
               double* yole, double* ug, double* vg, int32_t* jd, int32_t* kd);
/* src/time.f:110-175 (q(jd,kd,nspec,nq); qtn, qtnm1, qnewt (jd,kd,nspec,nv)) */
int ot2d_stqol(double* q, double* qtn, double* qtnm1, double* qnewt, int32_t* jd, int32_t* kd);
/* src/setup.f:111 and src/setup.f:440 (q: one instance, only q(:,:,nq) is written) */
int ot2d_find_cellcenter(double* x, double* y, double* xv, double* yv, int32_t* jd, int32_t* kd, int32_t* im);
int ot2d_metfv(double* q, double* x, double* y, double* xv, double* yv, double* xx, double* xy, double* yx,
               double* yy, int32_t* jd, int32_t* kd, int32_t* im);

/* Residual norms of step.f:58-93 -- rsum, resrho, resmax -- of one
 * instance's residual s(jd,kd,nmv) already in device memory (double),
 * computed without allocating device memory.  No counterpart in the
 * reference (step.f computes these inline).  For callers that cannot
 * allocate during their iteration loop (a driver whose device memory is all
 * in its own pool, a loop that must not take cudaMalloc's implicit device
 * synchronisation): the per-block partials live in a fixed static device
 * array, which limits jd*kd to OT2D_NOALLOC_MAX_CELLS (larger: OT2D_ERR_ARG,
 * nothing launched).  The first call on a device looks the array's device
 * address up with that device current and keeps it for the life of the
 * process; after cudaDeviceReset that address is stale, so do not call this
 * routine again in a process that has reset the device.  The call ends with a
 * stream synchronisation and a copy to host memory, so it must not be made
 * while its stream is being captured into a graph.  Calls share the array:
 * calls that overlap in time race, so serialise them.  s, iblank:
 * device pointers; js..ke: the interior (jbeg..jend, kbeg..kend); nmv >= 4;
 * out (host, 6 doubles): rsum, resrho, resmax and the j, k, n of resmax
 * (1-based; 0 when there is no interior cell).  stream: a cudaStream_t
 * (null = the default stream); the call returns after the stream has
 * finished the work. */
#define OT2D_NOALLOC_MAX_CELLS 1048576
int ot2d_norms_noalloc(const double* s, const int32_t* iblank, int32_t jd, int32_t kd, int32_t js, int32_t je,
                       int32_t ks, int32_t ke, int32_t nmv, double* out, void* stream);

/* ---------------------------------------------------------------------- */
/* solution / restart files (src/io.f, src/init.f:138-206)                 */
/* ---------------------------------------------------------------------- */
/* Files are Fortran sequential unformatted files (4-byte record markers,
 * 8-byte reals, 4-byte integers) in the record layout the reference writes
 * and reads; Tecplot files use its '(3F22.13)' / '(3I10)' formats.  The
 * library keeps its own table of Fortran unit numbers: the unit-level
 * routines below read and write units opened with ot2d_unit_open, in the
 * place of the reference's `open(unit=..., form=...)`.  Only itrans = 0 and
 * num_grids = 1 grid reads are supported (OT2D_ERR_ARG otherwise). */
/* open(unit, file=path, form='unformatted'|'formatted'), status 'unknown'
 * (created / truncated) for writing, 'old' for reading */
int ot2d_unit_open(int32_t unit, const char* path, int32_t formatted, int32_t for_write);
int ot2d_unit_close(int32_t unit);
/* one record of n integers (the mesh-size header of astore / init, istep0) */
int ot2d_unit_write_ints(int32_t unit, const int32_t* v, int32_t n);
/* the first n integers of the next record (the rest of the record is skipped) */
int ot2d_unit_read_ints(int32_t unit, int32_t* v, int32_t n);
/* src/io.f:2-170: writes fort.9 / fort.8 (fort_TS<n>.9 / .8 when ts) and
 * SA.dat / komega.dat (SA_TS<n>.dat, komega_TS<n>.dat) in the current
 * directory for the nmesh meshes of x, y, iblank (igrd) and q (iqdim) at the
 * 1-based offsets ipointer(nmesh,5); jd, kd are set to the last mesh's
 * sizes as set_pointers_globals does.  q(1:4) of every mesh goes through the
 * (Q/J)*J -> /J round trip of store on the device, as in the reference. */
int ot2d_astore(double* x, double* y, int32_t* iblank, double* q, int32_t* iturb, int32_t* itrans, int32_t* jgmx,
                int32_t* kgmx, int32_t* nmesh, int32_t* ipointer, int32_t* igrd, int32_t* iqdim, int32_t* jd,
                int32_t* kd, int32_t* istep0, int32_t* ts, int32_t* nspec);
/* src/io.f:278-340: q(jd,kd,nspec,nq), x, y, iblank (jd,kd,nspec); lg, lq:
 * nspec unit numbers (unformatted, open for writing) */
int ot2d_store(double* q, double* x, double* y, int32_t* iblank, int32_t* jd, int32_t* kd, int32_t* lg, int32_t* lq);
/* src/io.f:173-215 and :218-275: ltur formatted units, lq unformatted
 * (storekomega writes q(5:nv) to lq once more, io.f:253) */
int ot2d_storevnu(double* x, double* y, int32_t* iblank, double* q, int32_t* jd, int32_t* kd, int32_t* lq,
                  int32_t* ltur);
int ot2d_storekomega(double* x, double* y, int32_t* iblank, double* q, int32_t* jd, int32_t* kd, int32_t* lq,
                     int32_t* ltur);
/* src/io.f:343-380: xv, yv (jmax,kmax) from unit logg; iblank(jd,kd) = 1 */
int ot2d_grid(double* xv, double* yv, int32_t* iblank, int32_t* jd, int32_t* kd, int32_t* logg);
/* src/io.f:383-405 (q: one instance q(jd,kd,nq); sets totime of the
 * current parameters) and src/io.f:408-425 */
int ot2d_restr2(double* q, int32_t* jd, int32_t* kd, int32_t* logq);
int ot2d_restr_turb(double* q, int32_t* jd, int32_t* kd, int32_t* logq);
/* src/init.f:180-206: q(jd,kd,nq) of one instance, q(1:4) /= q(nq) */
int ot2d_qdivj(double* q, int32_t* jd, int32_t* kd);

/* ---------------------------------------------------------------------- */
/* batched solver (host runtime over device-resident meshes)               */
/* ---------------------------------------------------------------------- */

typedef struct ot2d_solver ot2d_solver;

/* per-instance result record */
typedef struct ot2d_result {
  int32_t id, status, iterations, converged;
  double rsum_first, rsum_last;    /* L2 norm (step.f:86-93) at it 1 and last  */
  double cl, cd, cm, cpower;       /* compute_forces, FP64 (forces.f:2-127)     */
  double t_admit, t_done;          /* seconds since solver creation: admitted to
                                      the device, retired (t_admit < 0: queued)  */
  double t_submit;                 /* seconds since solver creation: submitted  */
} ot2d_result;

/* solver options (ot2d_solver_set_option) */
#define OT2D_OPT_CHECK_EVERY   1  /* iterations between host status reads (default 25) */
#define OT2D_OPT_KEEP_Q        2  /* 1: keep q of retired instances for ot2d_solver_get_q */
#define OT2D_OPT_FORCE_EVERY   3  /* force rule: iterations between the CL/CD samples of
                                     its 8-sample window (default 0: every status check) */
#define OT2D_OPT_FORCE_DECADES 4  /* force rule: decades the L2 norm must be below its peak
                                     before the rule may retire an instance (default 1) */
#define OT2D_OPT_BUDGET_MB     6  /* device memory the live instances may hold, MiB
                                     (default 0: 90 % of the memory free when the solver
                                     was created) */
#define OT2D_OPT_LU_LAG        7  /* LU-SGS schedule: steps each 32-row band trails the
                                     band it depends on beyond the minimum (default 0) */
#define OT2D_OPT_LU_GROUP      8  /* LU-SGS records streamed per bulk copy: 1, 2, 4 or 8
                                     (default 0: the largest the shared memory allows) */
#define OT2D_OPT_RT_SHAPE      9  /* residual tile: 0 16x16 (default), 1 32x8, 2 8x32, 3 32x16 cells */
#define OT2D_OPT_PIPELINE     10  /* 1 (default): a batch of 16 or more time instances runs
                                     as two halves on two streams, each half's residual
                                     beside the other half's LU-SGS sweeps; 2: as four
                                     independent parts on four streams (and at least four
                                     requests); 0: one graph */
#define OT2D_OPT_POLL_LIMIT    5  /* polls a LU-SGS sweep wait makes before it gives up
                                     (default 4194304).  An instance whose wait gave up
                                     keeps its state and retires with OT2D_ERR_TIMEOUT;
                                     small values make the waits run out on purpose */

ot2d_solver* ot2d_solver_create(int32_t device, int32_t precision);
void ot2d_solver_destroy(ot2d_solver* s);
int ot2d_solver_set_option(ot2d_solver* s, int32_t key, int32_t value);
/* Also count an instance as converged once its CL and CD stayed within a
 * band of width dcl / dcd over the last 8 force samples (one per status
 * check, or one every OT2D_OPT_FORCE_EVERY iterations) and its L2 norm is
 * OT2D_OPT_FORCE_DECADES (default 1) decades below its peak (0, 0: residual
 * criterion only, the default).  This is the convergence rule of the
 * FP32-mixed path, whose f32 residual has a floor a few decades below its
 * peak and cannot show a 8-10 decade drop. */
int ot2d_solver_set_force_tol(ot2d_solver* s, double dcl, double dcd);
/* Launch choices for batches of one mesh-size class, as an autotuner
 * measured them (turns2d_urans_git_gb300/tune.py).  When a batch is built,
 * the first entry whose kd_max / jd_max bound the batch's largest mesh (the
 * one with most cells) sets the residual tile shape, the LU-SGS copy group,
 * the LU-SGS band lag and whether a batch of 16 or more time instances runs
 * as two pipelined halves; without a matching entry the OT2D_OPT_* values
 * apply.  The choices change the launch geometry and schedule only: every
 * variant gives the same state bit for bit (the L2 norm is summed per
 * residual tile, so it agrees to rounding across tile shapes). */
typedef struct ot2d_tuning {
  int32_t kd_max, jd_max;   /* class bound: kd <= kd_max and jd <= jd_max      */
  int32_t rt_shape;         /* 0 16x16, 1 32x8, 2 8x32                          */
  int32_t lu_group;         /* 0 (largest that fits), 1, 2, 4, 8                */
  int32_t lu_lag;           /* 0..64                                            */
  int32_t pipeline;         /* 0 one graph, 1 two pipelined halves, 2 four parts (OT2D_OPT_PIPELINE) */
} ot2d_tuning;
/* replace the tuning table (n entries, copied; n = 0 clears it) */
int ot2d_solver_set_tuning(ot2d_solver* s, const ot2d_tuning* t, int32_t n);

/* Append one JSON line per retired request to the file at path (id,
 * status, convergence, iterations, precision, mesh and flow, first and last
 * L2 norm, CL / CD / CM, submission / admission / retirement times); NULL
 * stops logging.  The solver also marks admissions and retirements and
 * brackets iterations and status checks with NVTX ranges, which cost
 * nothing unless a profiler is attached. */
int ot2d_solver_set_log(ot2d_solver* s, const char* path);

/* read the device status table now and retire finished instances */
int ot2d_solver_sync(ot2d_solver* s);
/* the CUDA stream (cudaStream_t) the solver launches on */
void* ot2d_solver_stream(ot2d_solver* s);
/* Phase timers: runs `iters` iterations phase by phase with CUDA events
 * between the kernel families and returns the mean milliseconds per phase:
 * 0 time_step, 1 bc, 2 residual (inviscid + viscous fluxes, assembly and
 * norms in one tiled kernel), 3 rbc, 4 LU-SGS, 5 SA, 6 update + monitor. */
#define OT2D_NPHASE 7
int ot2d_solver_profile(ot2d_solver* s, int32_t iters, double* ms, int32_t nphase);
/* Kernel launches of one batched iteration: the kernel nodes of the
 * iteration's CUDA graph (both graphs when the batch runs as two halves),
 * after building it for the live set; negative status on error. */
int ot2d_solver_graph_kernels(ot2d_solver* s);
/* Host-resident state, as a Fortran caller that owns q: every iteration
 * copies q(jd,kd,nspec,nq) of the listed live instances host->device, runs
 * one batched iteration and copies q back (the host arrays are updated). */
int ot2d_solver_iterate_host(ot2d_solver* s, int32_t n, const int32_t* ids, double* const* q_host, int32_t iters);
/* Submit one solve: params + vertex grid of time instance 1 (jmax*kmax).
 * Returns the instance id (>= 0) or -status.  `orders` = target L2 drop in
 * decades; max_iters caps the iterations.  Admission is by device memory:
 * a solve whose arrays (ot2d_instance_bytes) fit the memory budget next to
 * the live instances is admitted at once; otherwise it waits in a FIFO
 * queue and is admitted when retirements free enough memory (at a status
 * check or at the next ot2d_solver_iterate); a solve larger than the whole
 * budget is refused (-OT2D_ERR_NOMEM).  A time-accurate solve (iunst = 1,
 * motiontype = 1: the pitching grid of motion.f:546-632, dual time stepping
 * with itnmax Newton iterations per physical step, Turns_overset.f:360-505)
 * runs exactly max_iters physical steps, has no residual convergence test,
 * and is retired after its last Newton iteration.  A steady solve runs at
 * most max_iters iterations. */
int ot2d_solver_add(ot2d_solver* s, const ot2d_params* p, const double* xv, const double* yv, double orders,
                    int32_t max_iters);
/* Run `iters` iterations over every live instance (one launch per kernel
 * family per iteration).  Instances that converge, fail or reach their cap
 * are retired and their slot freed.  Returns OT2D_OK or a CUDA status. */
int ot2d_solver_iterate(ot2d_solver* s, int32_t iters);
/* number of submitted, not yet retired instances (queued ones included) */
int ot2d_solver_live(const ot2d_solver* s);
/* number of submitted instances still waiting for device memory */
int ot2d_solver_queued(const ot2d_solver* s);
/* copy the result of instance `id` (valid once retired, or a live snapshot) */
int ot2d_solver_result(ot2d_solver* s, int32_t id, ot2d_result* out);
/* download q (jd,kd,nspec,nq) of a live or retired-but-kept instance */
int ot2d_solver_get_q(ot2d_solver* s, int32_t id, double* q_out);
/* total device bytes held by the live instances */
size_t ot2d_solver_device_bytes(const ot2d_solver* s);
/* device bytes one instance with these params would take */
size_t ot2d_instance_bytes(const ot2d_params* p, int32_t precision);
/* Snapshot of a live instance into the files astore writes (src/io.f:2-170)
 * in directory dir: fort.8 / fort.9 (fort_TS<n>.*) and SA.dat / komega.dat.
 * The conversion runs on the device over the resident state, including the
 * (Q/J)*J -> /J round trip store applies to q; istep0 is the instance's
 * step counter. */
int ot2d_solver_store(ot2d_solver* s, int32_t id, const char* dir);
/* store instance `id` into dir when it retires (converged, failed or capped),
 * before its device memory is freed; dir = NULL cancels */
int ot2d_solver_store_on_retire(ot2d_solver* s, int32_t id, const char* dir);
/* Admit one solve that starts from the restart file dir/fort.3 (fort_TS<n>.3)
 * as init.f:138-170 reads it with iread > 0: header, restr2, restr_turb and
 * istep0 records, q(1:4)/J on the device; totime and istep0 come from the
 * file, and the instance runs with iread = 1 as a reference restart does.
 * Returns the instance id or -status. */
int ot2d_solver_add_restart(ot2d_solver* s, const ot2d_params* p, const double* xv, const double* yv,
                            const char* dir, double orders, int32_t max_iters);

/* Admit one solve that starts from the caller's state instead of the
 * freestream: q(jd,kd,nspec,nq) in the reference layout (init.f:180-206:
 * Q/J in 1..4, the turbulence variables in 5..nv); q(...,nq) is ignored, J
 * comes from the grid (setup.f:440-724).  This is how a driver that owns q
 * (Turns_overset.f:199-207) hands a state to the batched solver.  Returns
 * the instance id or -status. */
int ot2d_solver_add_state(ot2d_solver* s, const ot2d_params* p, const double* xv, const double* yv,
                          const double* q, double orders, int32_t max_iters);

#ifdef __cplusplus
}
#endif
#endif /* OT2D_H */
