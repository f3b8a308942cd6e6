/*
 * fluid2d_gb300.h -- C ABI of libfluid2d_gb300.so, the GB300 (sm_103a)
 * implementation of Fluid2d's time-step hot path.
 *
 * Conventions
 *  - Every array argument is a DEVICE pointer.  A field is a row-major
 *    (m, n) array: m rows along y, n columns along x, halo included, exactly
 *    the numpy layout of the reference (numpy a[j, i] == Fortran a(j+1, i+1)).
 *  - Masks are int8 (0 = solid, 1 = fluid), fields are float64.
 *  - A stencil array "A" is stored plane by plane: A[k*m*n + j*n + i] with
 *    k = 0..4 for the reference's A(j,i,1..5) (SW, S, SE, W, C of the
 *    symmetric 9-point operator); 9 planes for coarsenmatrix.
 *  - "stream" is a cudaStream_t (NULL = the legacy default stream).  Calls
 *    are asynchronous; outputs are ready when the stream reaches them.
 *  - Every function returns 0 on success or an F2D_ERR_* code; nothing ever
 *    exits the process (the reference's Fortran "stop" becomes F2D_ERR_NH).
 *    f2d_last_error() gives the message of the last failure on this thread.
 *  - Functions marked (scratch) use a device scratch buffer owned by the
 *    library (allocated on first use, grown on demand, one per device);
 *    such calls must not overlap on the GPU with another (scratch) call on
 *    the same device.
 *  - The f2d_set_* switches are process-wide settings without locking: set
 *    them from one host thread, before the models or graphs they are to
 *    affect are created or captured, not while another thread launches.
 *
 * Each declaration names the reference routine it replaces (file:line in
 * pvthinker/Fluid2d).
 */
#ifndef FLUID2D_GB300_H
#define FLUID2D_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* the library is built with hidden visibility; only these entry points are exported */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define F2D_OK 0
#define F2D_ERR_NH 1       /* nh != 3 where the reference stops */
#define F2D_ERR_SHAPE 2    /* unusable array dimensions */
#define F2D_ERR_ARG 3      /* bad argument */
#define F2D_ERR_CUDA 4     /* CUDA runtime failure */
#define F2D_ERR_DIVERGED 5 /* multigrid diverged (core/gmg/hierarchy.py:182-188) */
#define F2D_ERR_LIMIT 6    /* size beyond a fixed capacity */

/* library version, 100*major + minor */
int f2d_version(void);
/* message of the last failing call on this host thread ("" if none) */
const char *f2d_last_error(void);
/* 1 if the library was compiled to round every operation separately (no FMA
 * contraction) */
int f2d_exact_arithmetic(void);

/* ------------------------------------------------ fortran_advection ---- */
/* core/fortran_advection.f90:2-165 adv_upwind(msk,x,y,u,v,cst,nh,method,order[,m,n]),
 * called from core/operators.py:227-230.  cst: DEVICE pointer to the 5
 * doubles [dx, dy, logcosh, umax, aparab] (core/operators.py:111-117).
 * Writes y on the interior only. */
int f2d_adv_upwind(const int8_t *msk, const double *x, double *y, const double *u,
                   const double *v, const double *cst, int nh, int method, int order,
                   int m, int n, void *stream);
/* core/fortran_advection.f90:169-284 adv_centered (even orders 2/4/6) */
int f2d_adv_centered(const int8_t *msk, const double *x, double *y, const double *u,
                     const double *v, const double *cst, int nh, int method, int order,
                     int m, int n, void *stream);

/* ------------------------------------------------ fortran_fluxes ------- */
/* core/fortran_fluxes.f90:2-170 adv_upwind(msk,x,y,u,v,xflx,yflx,cst,nh,method,order),
 * called from core/fluxes.py:199-203 */
int f2d_flx_adv_upwind(const int8_t *msk, const double *x, double *y, const double *u,
                       const double *v, double *xflx, double *yflx, const double *cst,
                       int nh, int method, int order, int m, int n, void *stream);
/* core/fortran_fluxes.f90:174-279 adv_centered with edge fluxes (orders 2/4) */
int f2d_flx_adv_centered(const int8_t *msk, const double *x, double *y, const double *u,
                         const double *v, double *xflx, double *yflx, const double *cst,
                         int nh, int method, int order, int m, int n, void *stream);

/* ------------------------------------------------ fortran_operators ---- */
/* core/fortran_operators.f90:2-39 computeorthogradient(msk,psi,dx,dy,nh,u,v),
 * called from core/operators.py:493 */
int f2d_computeorthogradient(const int8_t *msk, const double *psi, double dx, double dy,
                             int nh, int m, int n, double *u, double *v, void *stream);
/* core/fortran_operators.f90:44-64 celltocorner(xr,xp), core/operators.py:440 */
int f2d_celltocorner(const double *xr, double *xp, int m, int n, void *stream);
/* core/fortran_operators.f90:102-122 cornertocell(xp,xr), core/quasigeostrophic.py:199 */
int f2d_cornertocell(const double *xp, double *xr, int m, int n, void *stream);
/* core/fortran_operators.f90:125-156 add_diffusion(msk,trac,dx,nh,Kdiff,dtrac),
 * core/operators.py:298 */
int f2d_add_diffusion(const int8_t *msk, const double *trac, double dx, int nh, double Kdiff,
                      double *dtrac, int m, int n, void *stream);
/* core/fortran_operators.f90:330-381 add_torque(msk,buoy,dx,nh,gravity,domega),
 * core/operators.py:312 */
int f2d_add_torque(const int8_t *msk, const double *buoy, double dx, int nh, double gravity,
                   double *domega, int m, int n, void *stream);
/* core/fortran_operators.f90:221-277 total=computenoslipsourceterm(msk,x,y,dx,dy,nh),
 * called from core/operators.py:256 (rhs_noslip).  y is written wherever the
 * Fortran loop writes it (rows 1..m-nh+1 in 1-based terms, including the
 * scattered terms in row and column nh); other cells keep their values.
 * total: DEVICE pointer to one double, the intent(out) sum of the terms in
 * the Fortran's order (bit-identical), or NULL to skip it.  nh >= 2. */
int f2d_computenoslipsourceterm(const int8_t *msk, const double *x, double *y, double dx,
                                double dy, int nh, int m, int n, double *total, void *stream);

/* ------------------------------------------------ fortran_diag --------- */
/* The f2py intent(out) scalars are written to the DEVICE array "out".
 * (scratch: the per-block partial sums) */
/* core/fortran_diag.f90:3-30 z=computedotprod(msk,x,y,nh) -> out[0]=z */
int f2d_computedotprod(const int8_t *msk, const double *x, const double *y, int nh, int m,
                       int n, double *out, void *stream);
/* core/fortran_diag.f90:33-60 y=computemax(msk,x,nh) -> out[0] */
int f2d_computemax(const int8_t *msk, const double *x, int nh, int m, int n, double *out,
                   void *stream);
/* core/fortran_diag.f90:63-90 y=computesum(msk,x,nh) -> out[0] */
int f2d_computesum(const int8_t *msk, const double *x, int nh, int m, int n, double *out,
                   void *stream);
/* core/fortran_diag.f90:93-120 y,y2=computesumandnorm(msk,x,nh) -> out[0..1] */
int f2d_computesumandnorm(const int8_t *msk, const double *x, int nh, int m, int n,
                          double *out, void *stream);
/* core/fortran_diag.f90:123-152 y,ymax=computenormmaxu(msk,x,nh) -> out[0..1] */
int f2d_computenormmaxu(const int8_t *msk, const double *x, int nh, int m, int n,
                        double *out, void *stream);
/* core/fortran_diag.f90:155-195 ke,maxu=computekemaxu(msk,u,v,nh) -> out[0..1],
 * called from core/euler.py:197 */
int f2d_computekemaxu(const int8_t *msk, const double *u, const double *v, int nh, int m,
                      int n, double *out, void *stream);
/* core/fortran_diag.f90:198-236 ke,maxu,maxv=computekemaxuv(msk,u,v,nh) -> out[0..2] */
int f2d_computekemaxuv(const int8_t *msk, const double *u, const double *v, int nh, int m,
                       int n, double *out, void *stream);
/* core/fortran_diag.f90:239-267 ke=computekewithpsi(msk,omega,psi,nh) -> out[0] */
int f2d_computekewithpsi(const int8_t *msk, const double *omega, const double *psi, int nh,
                         int m, int n, double *out, void *stream);

/* ------------------------------------------------ gmg.fortran_multigrid */
/* core/gmg/fortran_multigrid.f90:2-127 smoothtwicewitha(msk,A,x,b,coef,yo), called from
 * core/gmg/level.py:351.  x is updated in place exactly as the Fortran
 * updates it (including the cells its 3-row buffer writes back along the
 * edges).  The reference's yo buffer is replaced by a library scratch
 * array (scratch). */
int f2d_smoothtwicewitha(const int8_t *msk, const double *A, double *x, const double *b,
                         double coef, int m, int n, void *stream);
/* No counterpart in the reference.  The same smoother as f2d_smoothtwicewitha
 * for callers that must not allocate device memory (their memory comes from
 * their own allocator or a fixed budget, or they may not call cudaMalloc or
 * synchronise the device where they smooth): its work array is a fixed
 * 16 MiB static device buffer instead of library-allocated scratch, so
 * m*n may be at most 2^21 points (larger grids: F2D_ERR_LIMIT).  The first
 * call on a device looks up that buffer's device address (no allocation);
 * make that first call before any stream capture.  All calls share the
 * buffer, so calls that overlap on the GPU race with each other. */
int f2d_smoothtwicewitha_noalloc(const int8_t *msk, const double *A, double *x,
                                 const double *b, double coef, int m, int n, void *stream);
/* core/gmg/fortran_multigrid.f90:215-317 smoothtridiag(msk,A,x,b), called from
 * core/gmg/level.py:349 when hydroepsilon*dy/dx <= 0.2: one sweep of vertical
 * line relaxation (Gauss-Seidel across columns, a Thomas solve of rows
 * 3..m-5 per column).  No halo fill (the caller fills it).  m <= 5632.
 * (scratch: the elimination factors) */
int f2d_smoothtridiag(const int8_t *msk, const double *A, double *x, const double *b, int m,
                      int n, void *stream);
/* core/gmg/fortran_multigrid.f90:320-362 computeresidualwitha(msk,A,x,b,y),
 * core/gmg/level.py:374 */
int f2d_computeresidualwitha(const int8_t *msk, const double *A, const double *x,
                             const double *b, double *y, int m, int n, void *stream);
/* core/gmg/fortran_multigrid.f90:365-412 fillhalo(x,nh), core/gmg/halo.py:141 */
int f2d_fillhalo(double *x, int nh, int m, int n, void *stream);
/* core/gmg/fortran_multigrid.f90:415-498 interpolate(msk1,msk2,x2,nh,x1),
 * core/gmg/level.py:460; fine (m1,n1), coarse (m2,n2) */
int f2d_interpolate(const int8_t *msk1, const int8_t *msk2, const double *x2, int nh, int m2,
                    int n2, int m1, int n1, double *x1, void *stream);
/* core/gmg/fortran_multigrid.f90:501-546 restrict(msk2,x1,nh,x2), core/gmg/level.py:483 */
int f2d_restrict(const int8_t *msk2, const double *x1, int nh, int m2, int n2, int m1, int n1,
                 double *x2, void *stream);
/* core/gmg/fortran_multigrid.f90:706-811 Acoarse=coarsenmatrix(Afine,msk1,msk2,nh),
 * core/gmg/level.py:321.  Afine (9,m1,n1), Acoarse (9,m2,n2) planar; only
 * coarse rows/columns nh-1..m2-nh-1 (0-based) are written. */
int f2d_coarsenmatrix(const double *Afine, const int8_t *msk1, const int8_t *msk2, int nh,
                      int m1, int n1, int m2, int n2, double *Acoarse, void *stream);
/* core/gmg/fortran_multigrid.f90:813-839 y=computenorm(msk,x,nh) -> out[0] (sum of squares) */
int f2d_computenorm(const int8_t *msk, const double *x, int nh, int m, int n, double *out,
                    void *stream);
/* core/gmg/fortran_multigrid.f90:841-867 z=computeinner(msk,x,y,nh) -> out[0] */
int f2d_computeinner(const int8_t *msk, const double *x, const double *y, int nh, int m,
                     int n, double *out, void *stream);

/* ------------------------------------------------ device engine -------- */
/* Multigrid hierarchy on caller arrays: core/gmg/hierarchy.py:21-84 (Gmg,
 * setup_hierarchy) built from the corner mask mskp (HOST int8, (ny+6, nx+6)),
 * then twoVcycle (:207-218, operators.py:447) and solve (:154-192,
 * operators.py:470) on DEVICE arrays x (in place) and b.  The solve's
 * iteration count and residual stay on the device (f2d_gmg_solve_stats reads
 * them back, synchronously).  Coarsening stops before a level would have an
 * odd dimension (the reference supports power-of-two grids only, on which
 * nothing changes). */
int f2d_gmg_create(const int8_t *mskp_host, int nx, int ny, double dx, double dy,
                   double hydroepsilon, int qg, double Rd, void **gmg);
int f2d_gmg_destroy(void *gmg);
int f2d_gmg_levels(void *gmg, int *nlev, int *mv, int *nv, int *coarse_level);
int f2d_gmg_twovcycle(void *gmg, double *x, const double *b, void *stream);
int f2d_gmg_solve(void *gmg, double *x, const double *b, int maxite, double tol, void *stream);
int f2d_gmg_solve_stats(void *gmg, int *nite, double *res, int *status);
/* the hierarchy's own arrays of level lev: "msk" (int8), "A" (6 planes:
 * A1..A5 and omega/|A5|, levels >= 1), "x", "b", "r" */
void *f2d_gmg_level_ptr(void *gmg, int lev, const char *which);
/* core/gmg/hierarchy.py:98 Vcycle(lev1) and :131 Fcycle(lev1) on the
 * hierarchy's own x/b arrays */
int f2d_gmg_vcycle(void *gmg, int lev1, void *stream);
int f2d_gmg_fcycle(void *gmg, int lev1, void *stream);

/* Model time stepper: core/euler.py, core/boussinesq.py,
 * core/quasigeostrophic.py with core/timescheme.py:167-180 (RK3_SSP), the
 * Operators of core/operators.py and the loop body of core/fluid2d.py:237-268
 * (set_dt, step, diagnostics), all device-resident. */
#define F2D_EULER 0
#define F2D_BOUSSINESQ 1
#define F2D_QG 2
typedef struct f2d_model_desc {
    int model;           /* F2D_EULER, F2D_BOUSSINESQ or F2D_QG */
    int nx, ny;          /* interior cells (core/grid.py:31-32) */
    double Lx, Ly;
    int perio;           /* geometry 'perio': remove the mean of psi after the full solve */
    int order;           /* advection order (odd: upwind, even: centred) */
    int flux_method;     /* 0 minmax, 1 parabolic (core/operators.py:121-131) */
    double aparab;
    double gravity;      /* Boussinesq */
    double Rd, beta;     /* QG */
    double hydroepsilon;
    int adaptable_dt;    /* core/fluid2d.py:378-391 */
    double dt, cfl, dtmax;
    int precision;       /* 0: float64, 1: mixed (float32 fluxes and multigrid) */
    int diffusion;       /* param.diffusion: add_diffusion at the forcing stage */
    double Kdiff[2];     /* param.Kdiff of the advected tracers: [0] vorticity / pv,
                            [1] buoyancy (core/operators.py:146-152) */
} f2d_model_desc;
/* msk_host: HOST int8 cell mask (ny+6, nx+6) including the geometry's halo */
int f2d_model_create(const f2d_model_desc *d, const int8_t *msk_host, void **model);
int f2d_model_destroy(void *model);
/* state: DEVICE (nvar, ny+6, nx+6) float64, the reference's Var.state layout;
 * diag: DEVICE array of the model's diagnostics (f2d_model_diagname) */
int f2d_model_info(void *model, int *nvar, int *mv, int *nv, int *nlev, int *coarse_level,
                   double **state, double **diag);
/* device bytes the model holds (state, tendencies, hierarchy) */
int f2d_model_bytes(void *model, size_t *bytes);
const char *f2d_model_varname(void *model, int k);
const char *f2d_model_diagname(void *model, int k);
/* internal buffers: "state", "dx0", "dx1", "dx2" (RK tendencies, whose psi
 * planes are the warm starts), "cst", "dt", "diag", "work" */
double *f2d_model_buffer(void *model, const char *which);
/* set_psi_from_vorticity / set_psi_from_pv: full solve and psi -> u, v */
int f2d_model_set_psi(void *model, void *stream);
int f2d_model_diagnostics(void *model, void *stream);
/* nsteps iterations of (set_dt, step, diagnostics) */
int f2d_model_step(void *model, int nsteps, void *stream);
/* the same, replaying one step captured in a CUDA graph (non-default stream) */
int f2d_model_step_graph(void *model, int nsteps, void *stream);

/* nsteps steps of a model whose state lives in host memory: every step
 * uploads the state from `host` (page-locked; the layout of the model's
 * state: nvar planes of (ny+6) x (nx+6) float64), steps and reads it back,
 * the three captured once as one graph for this buffer and replayed on
 * `stream` (non-default).  Asynchronous; the reference's Python holds its
 * state in host arrays and calls the kernels on them every step (no
 * single counterpart: core/fluid2d.py:235-265 over the drop-in modules). */
int f2d_model_step_host(void *model, int nsteps, double *host, void *stream);
int f2d_model_set_dt(void *model, double dt);
int f2d_model_solve_stats(void *model, int *nite, double *res, int *status);
/* The model's status word: F2D_STATUS_* bits that the diagnostics set after
 * every step (and after set_psi) and that stay set until cleared -- what
 * stops the reference's run (core/fluid2d.py:309-314 maxspeed > 1e3,
 * core/gmg/hierarchy.py:182-188 divergence) plus any non-finite value.
 * Reads it on `stream` (synchronous), then clears it if `clear`.  Batched
 * and served runs use it to retire a failing instance alone. */
#define F2D_STATUS_NONFINITE 1 /* NaN or Inf in the fields (diagnostic sums) */
#define F2D_STATUS_BLOWUP 2    /* maxspeed > 1e3 */
#define F2D_STATUS_DIVERGED 4  /* the last full solve diverged */
#define F2D_STATUS_BAD_DT 8    /* dt not a positive finite number */
int f2d_model_status(void *model, int clear, int *status, void *stream);
/* f2d_model_status of n models at once (one synchronisation of `stream`):
 * status[k] for models[k] */
int f2d_models_status(void **models, int n, int clear, int *status, void *stream);
/* Timing probe of the finest-level smoother (one smoothtwicewitha call =
 * the engine's two sweep kernels): enable >= 0 switches it on/off (and drops
 * a captured graph); enable < 0 reads the mean duration in ms over the
 * probed calls of the last step (synchronous). */
int f2d_model_probe(void *model, int enable, int *count, double *avg_ms);
/* number of kernel nodes in the captured step graph */
int f2d_model_graph_kernels(void *model, int *nkernels);

/* ---- no-slip walls: after each step, the vorticity source along the walls
 * that cancels the tangential velocity, then a fast inversion (rhs_noslip,
 * core/operators.py:245-290 with computenoslipsourceterm,
 * core/fortran_operators.f90:221-277; core/euler.py:109-113).  msknoslip:
 * HOST int8 (ny+6, nx+6), the walls that are no-slip (the reference's
 * grid.msknoslip: the geometry's mask before islands are carved). */
int f2d_model_noslip(void *model, const int8_t *msknoslip_host, void *stream);

/* The level from which the multigrid runs in one CTA out of shared memory
 * (default: the finest level whose coarser suffix fits).  Any level from
 * *first to nlev (no CTA) may be chosen; results are identical, only the
 * launch structure (and speed) changes.  level < 0 only queries. */
int f2d_model_coarse_level(void *model, int level, int *current, int *first, int *nlev);

/* The coarse part of the multigrid cycles that start from x = 0 (every
 * V-cycle below the coarse level, and the F-cycle) applied as its dense
 * linear map of the coarse level's right-hand side, built by running the
 * cycle on unit vectors (at most 1024 interior points; product build only:
 * the exact build keeps the reference's order of operations).  enable: 1 on
 * (default), 0 off, < 0 query; *n receives the operator's size (0: none). */
int f2d_model_coarse_op(void *model, int enable, int *n);

/* The float level from which the mixed form's small-level V- and F-cycles
 * run as one thread-block-cluster launch (f2d_set_cluster), -1 if none (no
 * float levels, no coarse operator, fewer than 16 coarse rows, the switch
 * off).  No counterpart in the reference. */
int f2d_model_cluster_level(void *model, int *level);

/* Drop the model's captured step and loop graphs: the next graph run
 * captures again, with the launch settings then current (level tiles and
 * threads, programmatic dependent launch). */
int f2d_model_reset_graphs(void *model);

/* Programmatic dependent launch of the engine kernels (each kernel may be
 * scheduled while its predecessor runs and waits for it before touching
 * memory): 1 on (default), 0 off, < 0 query; returns the previous setting.
 * Graphs captured before a change keep their launches. */
int f2d_set_pdl(int enable);

/* The CTA count the multigrid level kernels (fused smoothing, residual +
 * restriction) aim at when they choose their tile: the largest tile is
 * halved, down to one warp, while the level's grid has fewer CTAs.  -1 twice
 * the SM count, 0 always the largest tile (default), > 0 that count, < -1
 * only queries; returns the previous setting.  Results do not depend on it;
 * graphs captured before a change keep their tiles. */
int f2d_set_level_tiles(int target);

/* The float64 finest level's smoother sweeps and residual (no counterpart in
 * the reference: an arithmetic form): 1 (the product build's default) on
 * grids of at least one CTA per SM, each thread takes a column of four points
 * with their neighbourhood in registers, and a point whose 3x3 block is
 * fluid goes through the separable form of the analytic 9-point operator
 * (8 float64 operations instead of 11 a sweep point, 7 instead of 10 a
 * residual point; the same function, other rounding); 2 the same at every
 * grid size; 0 the sweep and residual kernels in the reference's order of
 * operations.  < 0 queries; returns the previous setting.  The exact build
 * always uses 0; graphs captured before a change keep their kernels. */
int f2d_set_separable(int mode);

/* The mixed form's small levels (no counterpart in the reference: a launch
 * structure): m = 1..8 (product build) a V-cycle from zero or the F-cycle
 * from m levels above the coarse operator's level (fewer where their
 * strips do not fit) runs as one launch of a 16-CTA thread-block cluster
 * holding those levels in distributed shared memory, with the level
 * kernels' arithmetic bit for bit; 0 (the default) the level kernels,
 * which measured faster.  < 0 queries; returns the previous setting.
 * Applies to models created after the change; the exact build keeps 0. */
int f2d_set_cluster(int mode);

/* Persisting L2 windows (no counterpart in the reference: cache control):
 * 1 (default) the multigrid cycles' launches mark the hierarchy's small
 * levels (and the coarse operator's application the operator) for
 * persisting L2 residency, with up to 32 MB of L2 set aside for the
 * process's context; 0 off.  < 0 queries; returns the previous setting.
 * Graphs captured before a change keep their launches. */
int f2d_set_l2_persist(int mode);

/* Threads of the fused level smoother's CTA: 0 one per tile point (the
 * input ring and the first sweep's ring take a second pass; default), 1 one
 * per input point, so that every phase is one pass, for grids of fewer than
 * two CTAs per SM, 2 always one per input point; < 0 only queries; returns
 * the previous setting.  Results do not depend on it. */
int f2d_set_level_threads(int mode);

/* The device's float64 FMA throughput in TFLOP/s, measured (independent FMA
 * chains on every SM, CUDA events, best of three after a warm-up): the
 * FP64-ALU roofline of the float64 kernels.  Synchronises the device. */
int f2d_fp64_peak(double *tflops);

/* ---- batched steps: one step of each of n models (Euler or Boussinesq, float64
 * or mixed, without no-slip walls, islands or line relaxation) recorded and
 * merged into launches that each run one kernel for many models, captured in
 * one CUDA graph.  Each model computes exactly what f2d_model_step computes.
 * Rebuild after changing a model's dt or options. */
/* policy 0: each launch runs the kernel the most models need next; 1: the
 * next kernel of the model with the most work left, joined by every model
 * that needs the same kernel next */
int f2d_batch_create(void **models, int n, int policy, void **batch);
int f2d_batch_step(void *batch, int nsteps, void *stream);
/* launches per batched step and operations recorded over all models */
int f2d_batch_info(void *batch, int *launches, int *ops);
int f2d_batch_destroy(void *batch);

/* ---- islands with a prescribed streamfunction (core/island.py:21-47 gives
 * the two arrays; core/fluid2d.py:110-113 hands them to the operators): the
 * full inversions, the no-slip inversion and QG's stage inversions subtract
 * rhsp from the right-hand side and add psi to the masked solution
 * (core/operators.py:442-444, 482-486).  HOST float64 (ny+6, nx+6) arrays. */
int f2d_model_islands(void *model, const double *rhsp_host, const double *psi_host,
                      void *stream);

/* ---- flux diagnostic: Fluxes.diag_fluxes (core/fluxes.py:100-170), the
 * reversible and irreversible parts of the advective fluxes from one RK3 step
 * forward and one backward of an extended state (state, cell-centred u and v,
 * edge fluxes of every advected quantity), with the model's current dt and
 * umax (the device dt and cst[3] of the last set_dt).  Euler and Boussinesq
 * (the reference has no flux diagnostic for QG). */
int f2d_model_flux_setup(void *model, void *stream);
int f2d_model_diag_fluxes(void *model, void *stream);
/* flx: DEVICE (nfull, ny+6, nx+6) float64 in the order of f2d_model_flux_name
 * (the reference's fullflx_list: rev_x_vorticity, rev_y_vorticity, ...) */
int f2d_model_flux_info(void *model, int *nfull, double **flx);
const char *f2d_model_flux_name(void *model, int k);

/* ---- device time loop.  Replaces the host loop of Fluid2d.loop
 * (core/fluid2d.py:235-314) with its set_dt (:376-397), exact-history-time
 * adjustment (:245-254), blow-up stop (:306-311) and the decisions of
 * Output.do (core/output.py:62-94).  The clock stays on the device; a run is
 * one graph launch (a conditional WHILE node over one step) that stops at
 * tend, on a blow-up, when a record ring is full or after max_steps steps.
 * History records (the interior of the saved planes, float32, the layout of
 * core/output.py:234-243) and diagnostic rows wait in device rings until
 * f2d_model_loop_drain copies them out. */
#define F2D_LOOP_RUNNING 0
#define F2D_LOOP_TEND 1
#define F2D_LOOP_BLOWUP 2
#define F2D_LOOP_BAD_DT 3
typedef struct f2d_loop_desc {
    double tend;                  /* param.tend */
    double freq_his, freq_diag;   /* param.freq_his, param.freq_diag */
    int exacthistime;             /* param.exacthistime (acts with adaptable_dt) */
    int rescaledtime;             /* 0: 'none', 1: 'enstrophy' */
    int nsave;                    /* planes in a history record (<= 8) */
    int save[8];                  /* their state indices (param.var_to_save) */
    int his_cap, diag_cap;        /* ring capacities, in records */
    double t, tnexthis, tnextdiag; /* clock at the start: 0, 0, 0, or a restart's */
    int kt;
    int diag_fluxes;              /* param.diag_fluxes: flux records with the history */
} f2d_loop_desc;
typedef struct f2d_loop_state {
    double t, dt, tnexthis, tnextdiag;
    int kt, status, nhis, ndiag;
} f2d_loop_state;
int f2d_model_loop_setup(void *model, const f2d_loop_desc *ld, void *stream);
/* diagnostics and Output.do at the current time (core/fluid2d.py:199-214) */
int f2d_model_loop_start(void *model, void *stream);
/* asynchronous (the graph is captured once on a private stream) */
int f2d_model_loop_run(void *model, int max_steps, void *stream);
/* synchronous read of the clock */
int f2d_model_loop_state(void *model, f2d_loop_state *st, void *stream);
/* HOST outputs: his nhis x nsave x ny x nx float32, flx nhis x nfull x ny x nx
 * float32 (flux records, with diag_fluxes), his_t/his_kt nhis, diag_rows
 * ndiag x (ndiag_values + 4) float64 = t, kt, the model's diagnostics
 * (f2d_model_diagname order), dkedt, dvdt.  Empties the rings. */
int f2d_model_loop_drain(void *model, float *his, float *flx, double *his_t, int *his_kt,
                         double *diag_rows, int *nhis, int *ndiag, void *stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif /* FLUID2D_GB300_H */
