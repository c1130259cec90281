/*
 * astr_gpu.h — C ABI of the GB300 (sm_103a) right-hand-side hot path for
 * the ASTR compressible Navier-Stokes solver.
 *
 * The Fortran main loop of ASTR calls argument-less module routines that
 * act on module arrays (src/mainloop.F90:396-486).  This library replaces
 * their bodies.  A context holds every field resident in HBM on one GPU,
 * for one single-rank block; host arrays cross the boundary only on upload
 * and download, in the reference's own Fortran layout:
 *   halo arrays      var(-hm:im+hm,-hm:jm+hm,-hm:km+hm[,n]), hm = 5
 *   interior arrays  var(0:im,0:jm,0:km[,n])
 * (src/commarray.F90:14-27, 56-108).  All entry points are extern "C",
 * take plain pointers and sizes, never throw, and return ASTR_OK (0) or a
 * negative status; astr_gpu_last_error() gives the message.
 *
 * Threading: one context per host thread at a time; each context owns its
 * own CUDA stream.
 */
#ifndef ASTR_GPU_H
#define ASTR_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define ASTR_OK 0
#define ASTR_ERR_ARG -1        /* bad dimensions or parameters            */
#define ASTR_ERR_OOM -2        /* device allocation failed                */
#define ASTR_ERR_CUDA -3       /* CUDA runtime error                      */
#define ASTR_ERR_UNSUPPORTED -4 /* configuration outside what is built   */
#define ASTR_ERR_NONFINITE -5  /* crash check: non-finite or rho <= 0     */
#define ASTR_ERR_STATE -6      /* call out of order (e.g. no metrics)     */
#define ASTR_ERR_TIMEOUT -7    /* batched call: deadline passed           */
#define ASTR_ERR_CANCELLED -8  /* batched call: cancelled by the host     */

/* Stage ordering. */
#define ASTR_ORDER_MAIN 0     /* src/mainloop.F90:396-486                 */
#define ASTR_ORDER_MINIAPP 1  /* miniapps/tgv_solver_3d/tgvsolver.F90:994-1082 */

/* Precision forms. */
#define ASTR_FP64 0           /* plain FP64: the drop-in                  */
#define ASTR_FP32_STORAGE 1   /* FP32 streams, FP64 RK accumulation       */

/* Block dimensions and boundary types (src/commvar.F90:17-18;
 * npdc* as set by src/parallel.F90:1042-1228: 3 = periodic/inner block,
 * 4 = physical boundary at both ends). */
typedef struct {
  int im, jm, km;          /* intervals; km == 0 for a 2-D case            */
  int ia, ja, ka;          /* global intervals (statistics normalisation)  */
  int npdci, npdcj, npdck;
} astr_dims;

/* Scheme and flow constants (src/commvar.F90; refcal src/solver.F90:28-173). */
typedef struct {
  int order;               /* ASTR_ORDER_*                                  */
  int precision;           /* ASTR_FP64 or ASTR_FP32_STORAGE                */
  int lfilter;             /* compact filter at each stage                 */
  int diffterm;            /* viscous terms                                 */
  double alfa_filter;      /* filter alpha (0.49)                           */
  double beter_halo;       /* filter end-row alpha at block interfaces (1.11) */
  double beter_bound;      /* filter boundary-row parameter (0.98; mini-app 1.09) */
  double mach, reynolds, prandtl;
  double ref_tem;          /* reference temperature (Sutherland)           */
  double suth_const;       /* Sutherland constant (110.3 main, 110.4 mini-app) */
  double deltat;
  int channel;             /* flowtype 'channel': noslip isothermal j-walls
                              (boucon, src/bc.F90:327-409, 6423-6611), src_chan
                              (src/solver.F90:295-353) and the mass-flux
                              controller (src/statistic.F90:641-657, 1494-1533);
                              needs npdcj = 4 and the grid (astr_gpu_set_grid) */
  double twall;            /* isothermal wall temperature (twall, bctype 41) */
  int conschm;             /* ASTR_CONSCHM_*: convective scheme (conschm,
                              src/commvar.F90; dispatch in rhscal,
                              src/solver.F90:208-236)                        */
  int lchardecomp;         /* compact MP: characteristic decomposition and
                              the Ducros shock sensor (ducrossensor,
                              src/commcal.F90:196-353)                      */
  double bfacmpld;         /* compact MP: b factor of the compact upwind
                              interface scheme (src/flux.F90:72-82; 0.3)    */
  double shkcrt;           /* compact MP: shock-sensor threshold (0.01)     */
  int bctype[6];           /* boundary routine of each face (xmin, xmax, ymin,
                              ymax, zmin, zmax), bctype of boucon
                              (src/bc.F90:327-409): 41 isothermal no-slip
                              (6306-6712), 42 adiabatic no-slip (6728-7036,
                              x and y faces), 411 isothermal slip/no-slip
                              wall (7038-7229, y faces), 421 adiabatic slip wall
                              (7231-7430, y faces), 21 outflow (3404-3617,
                              xmax and ymax), 51 farfield (3008-3392, y and
                              z faces), 50 zero-gradient extrapolation
                              (2356-2652), 60 symmetry (2664-2996); 0 or 1:
                              none.  A face with a routine needs npdc = 4 in
                              its direction.  A channel has 41 on the y
                              faces unless set otherwise.                    */
  double twall_face[6];    /* wall temperature of each 41/411 face (0: twall) */
  double xslip;            /* 411 on ymin: slip where x(i,0,k,1) <= xslip,
                              isothermal no-slip beyond (the slip-nonslip
                              point, src/bc.F90:29, 7132); needs the grid
                              (astr_gpu_set_grid)                           */
} astr_params;

/* Convective schemes.  CENTRAL is '643c' (convrsdcal6,
 * src/solver.F90:2173-2341).  MP is '543c' (convrsdcmp,
 * src/solver.F90:1271-1937): Steger-Warming flux splitting
 * (src/riemann.F90:23-160), fifth-order compact upwind interface fluxes
 * (src/flux.F90:32-256), MP5 limiting (src/flux.F90:363-496) and, with
 * lchardecomp, Roe-averaged characteristic projection
 * (src/solver.F90:1958-2162).  MP needs ASTR_FP64 and the main ordering. */
enum { ASTR_CONSCHM_CENTRAL = 0, ASTR_CONSCHM_MP = 1 };

typedef struct {
  double kenergy;          /* kenergycal, src/statistic.F90:938-992         */
  double enstrophy;        /* enstophycal, src/statistic.F90:871-936        */
  int crash;               /* 1 when a non-finite value or rho <= 0 was seen */
} astr_status;

typedef struct astr_ctx astr_ctx;

/* Create a context and allocate every field in HBM.  Replaces the set-up of
 * solvrinit (src/comsolver.F90:47-146) and allocommarray
 * (src/commarray.F90:56-108).  Returns ASTR_OK and *out on success. */
int astr_gpu_create(const astr_dims* dims, const astr_params* params, astr_ctx** out);
void astr_gpu_destroy(astr_ctx* ctx);

/* Copy the grid metrics: dxi(-hm:..,1:3,1:3) and jacob(-hm:..) in Fortran
 * layout, as produced by gridgeom (src/geom.F90:99-930).  Host pointers.
 * Metrics whose off-diagonals are all exactly zero run the rectilinear
 * kernels; any other set (curvilinear grids, or the rounding residue
 * gridgeom's symmetric conservative form leaves on a stretched rectilinear
 * grid) runs the general-metric kernels, which hold all nine dxi arrays
 * (9 more halo arrays of device memory, allocated on first use). */
int astr_gpu_set_metrics(astr_ctx* ctx, const double* dxi, const double* jacob);

/* Node coordinates x(-hm:..,1:3) in Fortran layout (gridgeom's x after its
 * halo fill).  A channel context keeps the y coordinates for the bulk
 * integrals of src_chan and massfluxchan; a context with 411 on ymin keeps
 * which of that face's nodes lie at x <= xslip; a context with 23 (gcnscbc)
 * on xmax or ymax keeps that face's normal spacing and the grid's extent
 * along it, one with 12 (inflow_nscbc) the grid's x extent; others ignore
 * the call. */
int astr_gpu_set_grid(astr_ctx* ctx, const double* x);

/* Inflow arrays of bctypes 11 (inflow, src/bc.F90:1366-1562) and 12
 * (inflow_nscbc, src/bc.F90:2114-2344) on xmin: vel_in(0:jm,0:km,1:3),
 * tmp_in(0:jm,0:km), tmp_prof(0:jm) and prs_in(0:jm,0:km) in Fortran
 * layout, the values alloinflow's arrays hold after the profile routine
 * (freestreaminflow, profileinflow, ...).  A NULL array takes
 * freestreaminflow's values (u = 1, v = w = 0, T = 1, p = pinf), which a
 * context with an inflow face starts from.  11 reads vel_in, tmp_in and
 * tmp_prof; 12 reads vel_in and prs_in.  The turbulent inflow fluctuations
 * (turbinf) are not applied.  ASTR_ERR_STATE without an inflow face. */
int astr_gpu_set_inflow(astr_ctx* ctx, const double* vel_in, const double* tmp_in,
                        const double* tmp_prof, const double* prs_in);

/* Asynchronous stepping (no counterpart in the reference; used by the
 * request loop that serves many independent cases on one GPU): enqueue
 * nsteps RK3 steps on the context's stream and return at once, without
 * statistics.  The first call captures one step as a CUDA graph on the
 * context's stream (no other work may be issued to that stream meanwhile);
 * every step is then one graph launch.  Contexts on different streams run
 * concurrently.  Not for channel contexts (their controller counts steps on
 * the host). */
int astr_gpu_step_async(astr_ctx* ctx, int nsteps);
/* 1 when all work enqueued on the context has finished, 0 while it is in
 * flight, < 0 on a CUDA error. */
int astr_gpu_poll(astr_ctx* ctx);

/* Batches (continuous batching of independent cases; no counterpart in the
 * reference).  A batch steps all its cases with one launch per phase of an
 * RK3 stage (filter, qswap, RK3 base, convective + gradient, stress,
 * viscous, update): persistent kernels walk a work list of (case, block)
 * items of every case, each case with its own geometry, fields, schemes and
 * time step.  A case advances exactly as astr_gpu_rk3_step would advance it
 * alone (same kernels, same order, same arithmetic).  Cases join with
 * astr_batch_add after their metrics and state are set; a batch takes cases
 * of its own precision that run the tiled sweeps (main ordering, diagonal
 * metrics, central scheme; FP64 only with ASTR_V2=2 set at create), are
 * periodic (no boundary routines), not channels, without crash control.
 * Each case keeps its own context: uploads, downloads and statistics go
 * through it, ordered after the batch's work by stream events.  Destroying
 * a context removes it from its batch. */
typedef struct astr_batch astr_batch;
int astr_batch_create(int precision, astr_batch** out);
void astr_batch_destroy(astr_batch* batch);
/* ASTR_ERR_UNSUPPORTED (with the reason in astr_batch_last_error) for a case
 * outside what batches run, checked first; then ASTR_ERR_STATE when the case
 * is already in a batch or a call of this batch is in flight. */
int astr_batch_add(astr_batch* batch, astr_ctx* ctx);
int astr_batch_remove(astr_batch* batch, astr_ctx* ctx);
int astr_batch_size(astr_batch* batch);
/* Grid of the batch's persistent kernels: share (0, 1] of the blocks the
 * GPU holds resident at once (default 1: the whole GPU).  Batches that run
 * concurrently on their own streams take a share each, so that the phases
 * of one fill the GPU while another's end. */
int astr_batch_set_share(astr_batch* batch, double share);
/* Enqueue nsteps RK3 steps of every case and return at once.  budget_ms > 0
 * sets a deadline that many milliseconds after the call's work starts on the
 * GPU (its global timer).  Each step begins with a gate that reads the
 * cancel word (astr_batch_cancel) and the timer: once either says stop, no
 * later step starts, and a step that has started runs to its end, so every
 * case is always left at a step boundary.  One call in flight at a time. */
int astr_batch_step_async(astr_batch* batch, int nsteps, double budget_ms);
/* 1 when the call in flight has finished (or none is), 0 while it runs,
 * < 0 on a CUDA error. */
int astr_batch_poll(astr_batch* batch);
/* Wait for the call in flight; *steps_done (may be NULL) receives the steps
 * every case advanced.  ASTR_OK when all ran, ASTR_ERR_TIMEOUT when the
 * deadline stopped it, ASTR_ERR_CANCELLED when the cancel word did. */
int astr_batch_wait(astr_batch* batch, int* steps_done);
/* Set the batch's cancel word (page-locked host memory mapped into the
 * GPU); the next step gate of the call in flight sees it.  Thread-safe
 * against a concurrent astr_batch_wait. */
int astr_batch_cancel(astr_batch* batch);
/* astr_batch_step_async followed by astr_batch_wait. */
int astr_batch_step(astr_batch* batch, int nsteps, double budget_ms, int* steps_done);
int astr_batch_last_error(astr_batch* batch, char* buf, int len);
/* Kernel launches issued by this batch since creation. */
long long astr_batch_launch_count(astr_batch* batch);

/* crashcheck (src/mainloop.F90:709-812): count the interior nodes whose
 * density is negative or not a number; ijk (may be NULL) receives the
 * first such node (i fastest), or -1s.  The state is not modified. */
int astr_gpu_crashcheck(astr_ctx* ctx, long long* ncrash, int* ijk);

/* Crash control (lcracon; src/mainloop.F90:709-1198), main ordering.  On:
 * astr_gpu_rk3_step runs crashcheck before every step, rolling a crashed
 * state back to the older of two snapshots kept in HBM (databakup's
 * 'recovery', which restores nstep and the channel controller, recovers the
 * primitives and, from the second rollback to the same snapshot on, expands
 * the critical-node mask by one node: crinod_expansion) and otherwise taking
 * a snapshot when nstep reaches the next backup step (first after 5 steps,
 * the interval doubling up to 500: databakup's 'backup'); after every stage
 * it runs crashfix.  A rollback is reported in status->crash and is not an
 * error.  Enabling allocates two snapshots (80 bytes per stored node) and
 * three byte masks; astr_gpu_step_async refuses while it is on. */
int astr_gpu_set_crash_control(astr_ctx* ctx, int on);
/* databakup (src/mainloop.F90:824-972) on demand: mode 0 backup, 1 recovery
 * (*nstep, may be NULL, receives the step count after the call).  Needs
 * crash control to have been enabled once (the snapshots). */
int astr_gpu_databakup(astr_ctx* ctx, int mode, long long* nstep);
/* crashfix (src/mainloop.F90:1045-1198), one pass: every interior node with
 * rho, p or T below its floor (1e-5, 1e-5, and p of those) takes the mean q
 * of its neighbours with non-negative rho, p and T, node by node in the
 * reference's loop order; *wiped (may be NULL) receives the nodes replaced. */
int astr_gpu_crashfix(astr_ctx* ctx, long long* wiped);
/* Counters of crash control: out6 = {rollbacks, backups, nodes wiped by
 * crashfix, critical nodes (crinod), nstep, next backup step or -1}. */
int astr_gpu_crash_report(astr_ctx* ctx, long long* out6);

/* cflcal (src/commcal.F90:27-87) on the resident state: *cfl = deltat *
 * (Di + Dj + Dk), D the largest of 0 and the contravariant velocity plus
 * sound speed (sqrt(T)/mach) along each computational direction over the
 * interior nodes; delta3 (may be NULL) receives Di, Dj, Dk.  Diagonal
 * metrics, as everywhere in this library. */
int astr_gpu_cflcal(astr_ctx* ctx, double deltat, double* cfl, double* delta3);

/* boucon (src/bc.F90:327-409) for the per-routine drop-in: the boundary
 * routine of every face that has one (bctype, the channel's isothermal
 * j-walls included); no-op when no face has one. */
int astr_gpu_boucon(astr_ctx* ctx);

/* Channel controller state: out[0] force(1), out[1] mass flux and out[2]
 * its target at the last statcal, out[3] wall friction (fbcxchan), out[4]
 * completed time steps.  ASTR_ERR_STATE unless the context is a channel. */
int astr_gpu_channel_state(astr_ctx* ctx, double* out5);

/* Upload the conserved variables q(-hm:..,1:5) (halo layout) alone: the
 * primitives of the interior nodes are recomputed from them on the device
 * (updatefvar, src/fludyna.F90:191-242), the halo primitives are rebuilt by
 * qswap at the start of each stage in periodic directions.  The state of a
 * step is q; this is the per-step input when the host owns the state. */
int astr_gpu_upload_q(astr_ctx* ctx, const double* q);

/* Upload the conserved variables q(-hm:..,1:5) (halo layout) and the
 * primitive arrays rho, vel(..,1:3), prs, tmp (halo layout).  The
 * primitives are part of the solver state: interior primitives are the
 * ones updatefvar left at the end of the previous stage. */
int astr_gpu_upload_state(astr_ctx* ctx, const double* q, const double* rho,
                          const double* vel, const double* prs, const double* tmp);
/* Download the same arrays (any pointer may be NULL to skip it). */
int astr_gpu_download_state(astr_ctx* ctx, double* q, double* rho, double* vel,
                            double* prs, double* tmp);
/* Download qrhs(0:im,..,1:5), dvel(0:im,..,1:3,1:3), dtmp(0:im,..,1:3). */
int astr_gpu_download_rhs(astr_ctx* ctx, double* qrhs, double* dvel, double* dtmp);

/* nsteps full RK3 steps (time_integration_rk, src/mainloop.F90:301-601).
 * If hist != NULL it receives {kenergy, enstrophy} per step, sampled at
 * stage 1 (where rkfirst/statcal sample them).  status may be NULL. */
int astr_gpu_rk3_step(astr_ctx* ctx, int nsteps, double* hist, astr_status* status);

/* Finer drop-in entry points, one per reference routine. */
int astr_gpu_filterq(astr_ctx* ctx);     /* src/comsolver.F90:514-632   */
int astr_gpu_qswap(astr_ctx* ctx);       /* src/parallel.F90:4848-5318  */
int astr_gpu_gradcal(astr_ctx* ctx);     /* src/comsolver.F90:244-497   */
int astr_gpu_rhscal(astr_ctx* ctx);      /* src/solver.F90:185-282      */
int astr_gpu_updatefvar(astr_ctx* ctx);  /* src/fludyna.F90:191-242     */

/* Device-side statistics of the current state (uses the last gradients). */
int astr_gpu_reduce_stats(astr_ctx* ctx, double* kenergy, double* enstrophy);

/* Wait for all work of the context; returns the first asynchronous error. */
int astr_gpu_synchronize(astr_ctx* ctx);

/* Message of the last failed call on this context (or of the last failed
 * astr_gpu_create when ctx is NULL). Returns its length. */
int astr_gpu_last_error(astr_ctx* ctx, char* buf, int len);

/* Bytes of HBM held by a context with these dimensions and parameters. */
size_t astr_gpu_footprint(const astr_dims* dims, const astr_params* params);

/* Number of kernel launches issued by this context since creation. */
long long astr_gpu_launch_count(astr_ctx* ctx);

/* Diagonal-metric upload: dxi(:,:,:,1,1), dxi(:,:,:,2,2), dxi(:,:,:,3,3)
 * and jacob, each one halo-layout array.  Equivalent to
 * astr_gpu_set_metrics with every off-diagonal dxi equal to zero, without
 * the host holding the six zero arrays (no counterpart in the reference,
 * whose gridgeom always stores all nine). */
int astr_gpu_set_metrics_diag(astr_ctx* ctx, const double* dxi11, const double* dxi22,
                              const double* dxi33, const double* jacob);

/* Page-locked host memory for uploads and downloads (cudaMallocHost);
 * a Fortran host can c_f_pointer onto it.  NULL on failure. */
void* astr_gpu_host_alloc(size_t bytes);
void astr_gpu_host_free(void* p);

/* nsteps RK3 steps without statistics, bracketed by CUDA events on the
 * context's stream; *elapsed_ms receives the device time. */
int astr_gpu_timed_steps(astr_ctx* ctx, int nsteps, double* elapsed_ms);

/* Per-kernel-class device times.  With profiling on, every launch is
 * bracketed by CUDA events; astr_gpu_kernel_times synchronises and returns,
 * per class, the summed milliseconds and the launch counts.  Classes:
 * 0 filter, 1 halo (qswap/bchomo), 2 convective+gradient, 3 viscous(+RK),
 * 4 pointwise, 5 statistics.  Returns the number of classes. */
int astr_gpu_set_profiling(astr_ctx* ctx, int on);
int astr_gpu_kernel_times(astr_ctx* ctx, double* ms, long long* launches, int nclass);

/* Measurement helper: FP64 FMA throughput of this device in TFLOP/s (each
 * FMA counts two flops), from a register-resident FMA loop. */
int astr_gpu_measure_fp64_peak(double* tflops);

/* Kinetic energy and enstrophy without allocating anything (no counterpart
 * in the reference: it exists for callers that cannot call cudaMalloc, such
 * as a host whose HBM is all handed to its own pool, or a time loop that must
 * not synchronise the device through an allocation between steps).
 * Computes what astr_gpu_reduce_stats computes, from device arrays the
 * caller owns: rho and vel(:,:,:,1:3) in the halo layout, dvel(:,:,:,1:3,1:3)
 * in the interior layout, for the block `dims` (l0: enstrophy length scale,
 * 0 means 1).  Runs on `stream` (a cudaStream_t, NULL for the default
 * stream) and waits for it before returning.
 * Scratch: a fixed device array of 2*ASTR_NOALLOC_STATS_MAX_BLOCKS doubles
 * (1 MiB, held by every GPU that loads the library until exit), one pair of
 * partial sums per 4096 stored nodes; a block whose stored nodes
 * (im+1)*(jm+1)*(km+1) exceed 4096 * (ASTR_NOALLOC_STATS_MAX_BLOCKS - 1) =
 * 268,431,360 is rejected with ASTR_ERR_UNSUPPORTED, and dims that
 * astr_gpu_create would reject (im, jm (, km) < 8; km != 0 in 2-D) with
 * ASTR_ERR_ARG.  All calls share that array, so calls whose work overlaps on
 * the GPU race; serialise them.  A call outside a stream capture looks up
 * the array's device address in the current context; a call made while its
 * stream is being captured reuses the address found by the last uncaptured
 * call on that device, so make one call on the device before capturing.
 * Errors left pending by other work are neither reported nor cleared. */
#define ASTR_NOALLOC_STATS_MAX_BLOCKS 65536
int astr_gpu_stats_noalloc(const double* rho, const double* vel, const double* dvel,
                           const astr_dims* dims, double l0, void* stream,
                           double* kenergy, double* enstrophy);

#ifdef __cplusplus
}
#endif
#endif
