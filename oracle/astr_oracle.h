/*
 * ORACLE — test infrastructure only.
 *
 * CPU restatement (FP64, OpenMP over lines) of the ASTR right-hand-side hot
 * path: compact first derivative, compact low-pass filter, Thomas solver,
 * periodic halo swaps, convective and viscous residuals, primitive recovery
 * and the RK3 stage loop, in both stage orderings found in the reference
 * (the main solver `src/mainloop.F90` and the TGV mini-app
 * `miniapps/tgv_solver_3d/tgvsolver.F90`).
 *
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark
 * may load this library, and only as the checker.  The GPU product never
 * links it.
 *
 * Parity pin: the mini-app ordering reproduces the reference's own golden
 * history `miniapps/tgv_solver_3d/state.ref_128` (tests/golden/).  The
 * main-solver ordering shares every numerical kernel with it and is pinned
 * by that kernel-level agreement plus the analytic known-answer tests of
 * `src/test.F90`.
 *
 * Array layout is the reference's Fortran layout: `var(-hm:im+hm,
 * -hm:jm+hm,-hm:km+hm[,n])` column-major (i fastest) for halo arrays, and
 * `var(0:im,0:jm,0:km[,n])` for interior-only arrays.
 */
#ifndef ASTR_ORACLE_H
#define ASTR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

/* Stage ordering. */
enum { ORC_MODE_MAIN = 0, ORC_MODE_MINIAPP = 1 };

/* Boundary types per direction (npdc in src/parallel.F90:1042-1228). */
enum { ORC_NPDC_INNER = 3, ORC_NPDC_WALLS = 4 };

typedef struct {
  int im, jm, km;          /* local sizes (intervals); km==0 for 2-D */
  int ia, ja, ka;          /* global sizes used in normalisations */
  int npdci, npdcj, npdck; /* 3 = periodic/inner block, 4 = both ends physical */
  int mode;                /* ORC_MODE_* */
  int lfilter, diffterm;
  int channel;             /* 1: channel flow (noslip j-walls + src_chan) */
  double alfa_filter, beter_halo, beter_bound;
  double mach, reynolds, prandtl, ref_tem, suth_const; /* 110.3 main, 110.4 mini-app */
  double deltat;
  double twall;            /* isothermal wall temperature (channel) */
  /* convective scheme: 0 = central 643c (convrsdcal6), 1 = compact MP
   * 543c (convrsdcmp, src/solver.F90:1271-1937) */
  int conschm_mp;
  int lchardecomp;         /* characteristic projection + Ducros sensor */
  double bfacmpld;         /* b factor of the compact upwind scheme */
  double shkcrt;           /* shock-sensor threshold */
  /* boundary routine of each face (xmin, xmax, ymin, ymax, zmin, zmax),
   * bctype of src/bc.F90:327-409: 41 isothermal no-slip, 42 adiabatic
   * no-slip, 411 isothermal slip/no-slip (y faces), 421 adiabatic slip
   * (y faces), 21 outflow (xmax, ymax), 51 farfield (y, z faces), 50
   * zero-gradient extrapolation, 60 symmetry; 0 or 1 none.
   * A channel (channel = 1) with 0 on the y faces has 41 there. */
  int bctype[6];
  double twall6[6];        /* wall temperature of each 41/411 face (0: twall) */
  /* 411 on ymin: slip where x(i,0,k,1) <= xslip, no-slip beyond */
  double xslip;
} orc_config;

orc_ctx* orc_create(const orc_config* cfg);
void orc_destroy(orc_ctx* c);

/* Direct access to internal arrays (Fortran layout). Names:
 * "q","rho","vel","prs","tmp","x","dxi","jacob" (halo arrays),
 * "qrhs","qsave","dvel","dtmp" (0:im arrays), "sigma","qflux","ssf" (halo). */
double* orc_field(orc_ctx* c, const char* name);
/* Scheme coefficients: dir 0..2, kind 0 = derivative, 1 = filter.
 * Copies a,c,ac1,ac2,ac3 for nodes first..last into out (5*n doubles);
 * returns n and writes first node index. */
int orc_scheme(orc_ctx* c, int dir, int kind, int* first, double* out, int cap);
/* Filter RHS coefficient tables: coef10i(0:5), coef8i(0:4), coef6i(0:3),
 * coefb(0:4,0:8) (column-major), coefh(0:4,0:10) (column-major). */
void orc_filter_tables(orc_ctx* c, double* c10, double* c8, double* c6, double* cb, double* ch);
void orc_constants(orc_ctx* c, double* out8); /* const1..const7, tempconst, tempconst1 -> 9 */

/* Set-up restatements. */
void orc_gridcube(orc_ctx* c, double lx, double ly, double lz);
void orc_gridgeom(orc_ctx* c);      /* metrics dxi, jacob from x (src/geom.F90:99-930) */
void orc_init_tgv(orc_ctx* c);      /* tgvini + updateq (main) / flowfield_init (mini-app) */
void orc_updateq(orc_ctx* c);       /* q from primitives at 0:im (fvar2q with T) */

/* Hot-path restatements (each acts on the context's arrays). */
void orc_filterq(orc_ctx* c);
void orc_qswap(orc_ctx* c);
void orc_boucon(orc_ctx* c);       /* the faces' boundary routines, in face order */
/* Channel controller state: force(1), mass flux, its target, wall friction,
 * completed steps (5 doubles). */
void orc_chan_state(orc_ctx* c, double* out5);
void orc_gradcal(orc_ctx* c);
void orc_convrsdcal6(orc_ctx* c);
void orc_diffrsdcal6(orc_ctx* c);
void orc_rhscal(orc_ctx* c);        /* conv, negate, diff, src_chan */
void orc_updatefvar(orc_ctx* c);
void orc_bchomo(orc_ctx* c);        /* mini-app halo fill */

/* One RK3 step in the configured ordering. stats (may be NULL) receives
 * {kinetic energy, enstrophy} sampled where the reference samples them. */
void orc_rk3_step(orc_ctx* c, double* stats);
void orc_rk3_steps(orc_ctx* c, int nsteps, double* stats /* 2*nsteps or NULL */);

/* Stand-alone line kernels (used by the known-answer tests). */
void orc_line_derivative(orc_ctx* c, int dir, const double* f /* -5..dim+5 */, double* df /* 0..dim */);
void orc_line_filter(orc_ctx* c, int dir, const double* f, double* ff);

/* Compact MP convective path (conschm 543c). */
void orc_ducrossensor(orc_ctx* c);  /* ssf, lshock from dvel and prs */
void orc_convrsdcmp(orc_ctx* c);    /* qrhs += interface-flux differences */
/* lshock(0:im,0:jm,0:km) as bytes (0/1); returns 0 before the first sensor call */
int orc_lshock(orc_ctx* c, unsigned char* out);
/* Line kernels of the MP path: the compact upwind (wind=+1) or downwind
 * (wind=-1) interface flux fh(-1..dim) of f(-5..dim+5) along dir. */
void orc_line_flux(orc_ctx* c, int dir, int wind, const double* f, double* fh);
double orc_mp5(const double* u5, double ul, int discont);
/* Steger-Warming split at one node: prim = {rho,u,v,w,p,T}, q5, dxi row
 * (3), jacob -> fplus(5), fminus(5). */
void orc_steger_warming(orc_ctx* c, const double* prim, const double* q5, const double* dxi3,
                        double jac, double* fp, double* fm);
/* Roe-averaged eigenvectors between two nodes: st = {T,rho,p,E,u,v,w,dxi1,dxi2,dxi3}
 * of the left and right node; REV, LEV (5x5, column-major). */
void orc_chardecomp(const double* stl, const double* str, double* rev, double* lev);

/* Diagnostics. */
double orc_kenergy(orc_ctx* c);
double orc_enstrophy(orc_ctx* c);
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
