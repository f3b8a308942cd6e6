// f2d_fused.cuh -- device views and launchers of the engine kernels
// (multigrid levels, single-CTA coarse solve, fused stage kernels).
#pragma once
#include "f2d_common.cuh"

namespace f2d {

constexpr int NH = 3;           // halo width (the reference requires 3)

// call f(offset) for the point (J, I) and each of its periodic halo images:
// rows J, J - m2 (if J is among the last NH interior rows), J + m2 (if among
// the first NH), likewise for columns, every combination (scalars rather than
// small indexed arrays, which would live in local memory)
template <class F>
F2D_DEV void for_images(int J, int I, int mv, int nv, F &&f) {
    const int m2 = mv - 2 * NH, n2 = nv - 2 * NH;
    const int ja = (J >= m2 && J < m2 + NH) ? J - m2 : -1;
    const int jb = (J >= NH && J < 2 * NH) ? J + m2 : -1;
    const int ia = (I >= n2 && I < n2 + NH) ? I - n2 : -1;
    const int ib = (I >= NH && I < 2 * NH) ? I + n2 : -1;
    f(off(J, I, nv));
    if (ia >= 0) f(off(J, ia, nv));
    if (ib >= 0) f(off(J, ib, nv));
    if (ja >= 0) {
        f(off(ja, I, nv));
        if (ia >= 0) f(off(ja, ia, nv));
        if (ib >= 0) f(off(ja, ib, nv));
    }
    if (jb >= 0) {
        f(off(jb, I, nv));
        if (ia >= 0) f(off(jb, ia, nv));
        if (ib >= 0) f(off(jb, ib, nv));
    }
}

constexpr int MAX_LEVELS = 24;  // core/gmg/level.py:112-115 aborts beyond 20

// One multigrid level on the device.  Arrays are (mv, nv) row-major with
// the 3-cell halo.  A holds 6 planes: A1..A5 (SW, S, SE, W, C of the
// symmetric 9-point operator, core/gmg/level.py:332-335) and C3 = omega/|A5|
// (precomputed: the smoother's per-point division of
// core/gmg/fortran_multigrid.f90:67,103, same value).  The finest level has
// no stored A: its operator is analytic in the mask (core/gmg/level.py:261-302).
template <typename T>
struct LevelView {
    int mv, nv;
    const int8_t *msk;
    const T *A;
    T *x, *b, *r, *t;
    // finest level: per point, which of its 8 off-diagonal coefficients
    // (bits 0-7, the order of offdiag) and its diagonal (bit 8) are nonzero,
    // with the periodic-image rule of the analytic operator; else null
    const uint16_t *nb;
};

// Analytic finest-level operator: A_k(J,I) = sc[k] where msk(J',I') and
// msk(J'+dj_k, I'+di_k) are fluid, (J',I') the periodic image of (J,I)
// (the reference fills the halo of A periodically, core/gmg/level.py:297).
template <typename T>
struct AnalyticT {
    T sc[5];  // stencil*coef of planes SW, S, SE, W, C
    T a5;     // A5 on fluid points, after the Helmholtz shift (QG)
    T c3;     // omega / |a5|
};
using Analytic = AnalyticT<double>;

enum CycleMode { CYCLE_V = 0, CYCLE_F = 1 };
// input of a smoothing call: x, zero, x + prolongation of the coarser
// level's x, or the prolongation alone
enum XMode { X_IN = 0, X_ZERO = 1, X_PLUS_INTERP = 2, X_INTERP = 3 };

template <typename T>
struct CoarseArgs {
    int nlev;                    // levels in the CTA: [0, nlev) of lev[]
    LevelView<T> lev[MAX_LEVELS];
    T c1, c2;                    // omega, 1 - omega
    int mode;                    // CYCLE_V or CYCLE_F, started at lev[0]
    int zero_first;              // V-cycle: the first level starts from x = 0
    int ndeepest;                // smoothing calls on the coarsest level
    const int *active;           // skip everything when *active == 0
};

// launchers (kernels_fused.cu)
template <typename T>
int mg_sweep1(const LevelView<T> &L, const AnalyticT<T> *an, T c1, T c2, bool zero_x,
              const int *active, cudaStream_t s);
template <typename T>
int mg_sweep2(const LevelView<T> &L, const AnalyticT<T> *an, T c1, T c2, const int *active,
              cudaStream_t s);
template <typename T>
int mg_residual(const LevelView<T> &L, const AnalyticT<T> *an, const T *x, const T *b, T *r,
                const int *active, cudaStream_t s);
template <typename T>
int mg_restrict(const LevelView<T> &fine, const T *src, const LevelView<T> &coarse, T *dst,
                const int *active, cudaStream_t s);
template <typename T>
int mg_interp(const LevelView<T> &coarse, const T *src, const LevelView<T> &fine, T *dst,
              bool assign, const int *active, cudaStream_t s);
template <typename T>
int mg_coarse(const CoarseArgs<T> &args, size_t smem, cudaStream_t s);
// the coarse part as a linear map: its n x n operator (one CTA per column),
// and its application to the first level's b into x
template <typename T>
int mg_coarse_columns(const CoarseArgs<T> &args, size_t smem, T *op, int n, cudaStream_t s);
template <typename T>
int mg_coarse_apply(const T *op, int n, const LevelView<T> &L, const int *active,
                    cudaStream_t s);
// fused smoothtwicewitha: input per xmode (0 x, 1 zero, 2 x + interp(coarse),
// 3 interp(coarse)), result into `out` (not x)
template <typename T>
int mg_smooth_fused(const LevelView<T> &L, const AnalyticT<T> *an, T c1, T c2, int xmode,
                    const LevelView<T> *coarse, T *out, const int *active, cudaStream_t s);
// the float64 finest level's two sweeps (x or zero -> t -> x and its images)
// in column form (product build); *done = false (nothing launched) when it
// does not apply
template <typename T>
int mg_sweeps_column(const LevelView<T> &L, const AnalyticT<T> &an, T c1, T c2, bool zero_x,
                     const int *active, cudaStream_t s, bool *done);
// a stored level's two sweeps in column form on its uniform-stencil points
// (flags uf, stencil st = (c, ey, ex, c3) from mg_uniform_setup; float64
// product build); call where column_applies(L)
template <typename T>
int mg_sweeps_uniform(const LevelView<T> &L, const uint8_t *uf, const T *st, T c1, T c2,
                      bool zero_x, const int *active, cudaStream_t s);
// a level of L's size takes the column form now: the mode on, no step
// being recorded, (mode 1) a grid of at least one CTA per SM; the finest
// level also needs the analytic 9-point operator and its coefficient bits
template <typename T>
bool column_applies(const LevelView<T> &L);
template <typename T>
bool column_l0_applies(const LevelView<T> &L, const AnalyticT<T> &an);
// set-up of a stored level's uniform stencil: 16 samples (6 doubles each)
// of its stencil into out, the choice on the host, the flags on the device
int mg_stencil_samples(const LevelView<double> &L, double *out, cudaStream_t s);
bool mg_uniform_choose(const double *h, double *st);
int mg_uniform_flags(const LevelView<double> &L, const double *st, uint8_t *uf, cudaStream_t s);
// The mixed form's cluster sub-cycle (a V-cycle from zero or the F-cycle
// from level Ls down to the coarse operator's level, float, one launch of a
// CL_NC-CTA cluster with the levels in distributed shared memory).
constexpr int CL_NC = 16, CL_THREADS = 1024, CL_G = 2, CL_MAXLEV = 8;
constexpr size_t CL_SMEM_MAX = 200 * 1024;

struct ClLevel {
    int mv, nv;
    int rows;                          // local rows: the largest strip + 2 CL_G
    unsigned o_x[2], o_b, o_t;         // shared-memory byte offsets
    const int8_t *msk;
    const float *A;
};

struct ClArgs {
    int nlev;                          // lv[0] = level Ls .. lv[nlev-1] = the operator's level
    ClLevel lv[CL_MAXLEV];
    int p[CL_NC + 1];                  // strips of the operator level's interior rows
    float *x_top;                      // level Ls's x (global): the result
    const float *b_top;                // level Ls's b (global)
    const float *op;                   // the coarse operator of the cycle (V or F)
    const float *op_v;                 // the V-cycle operator (the F-cycle's inner V-cycles)
    int n;                             // operator size
    float c2;                          // 1 - omega
    int mode;                          // CYCLE_V (first smooth from zero) or CYCLE_F
    unsigned o_g;                      // gathered coarse b (n floats)
    const int *active;
};

bool mg_cluster_feasible(size_t smem);
int mg_cluster_cycle(const ClArgs &a, size_t smem, cudaStream_t s);
int &cluster_mode();

// residual of L (x, b) restricted into the coarse b2
template <typename T>
int mg_resres(const LevelView<T> &F, const AnalyticT<T> *an, const LevelView<T> &C, T *b2,
              const int *active, cudaStream_t s, const uint8_t *uf = nullptr,
              const T *ust = nullptr);
template <typename T>
size_t coarse_smem_bytes(const int *mv, const int *nv, int nlev);

// stage kernels (kernels_fused.cu), float64 state
struct AdvStage {
    const int8_t *msk;
    const double *q;          // advected tracer (stage state)
    const double *u, *v;      // stage velocities
    const double *advc;       // device SplitConst derived from cst (written by set_dt)
    double *dq;               // tendency out (interior + periodic halo)
    // torque (Boussinesq, core/operators.py:303-314): dq = dq*msk + g db/dx
    const double *buoy;       // null: no torque
    double torque_coef;       // 0.5*gravity/dx
    // diffusion (core/fortran_operators.f90:125-156 add_diffusion), added after
    // the torque: dq += coef*sum(msk_nb*(q_nb - q)) where msk == 1; 0: none
    double diff_coef;         // Kdiff/(dx*dx), Kdiff already scaled by the stage coef
    // RK combination written in the same pass: out = base + c*(sum of tendencies)
    int rk;                   // 0 none, 1: out = base + dt*dq, 2: out = base + (dt/4)(d0+dq),
                              // 3: out = base + (dt/6)(d0 + d1 + 4 dq)
    const double *base, *d0, *d1;
    double *out;
    const double *dt;         // device scalar
    int kind, method, order;  // flux kind (0 upwind, 1 centred), splitting, order
    int fp32;                 // fluxes computed in float (mixed form)
    int mv, nv;
};
int stage_advection(const AdvStage &a, cudaStream_t s);

struct OrthoStage {
    const int8_t *msk, *mskp;
    double *psi;                 // in/out: psi <- psi*mskp (whole array)
    double *u, *v;               // out: rows/cols 1..m-2
    double zdx, zdy;
    // RK combination of the velocities (rows/cols 1..m-2), as AdvStage::rk,
    // with the current u, v as the newest tendency
    int rk;
    const double *ubase, *vbase, *u0, *v0, *u1, *v1;
    double *uout, *vout;
    // psi_rk != 0: psiout = psibase + (dt/6)*(psi0 + psi1 + 4*psi2) over the
    // whole array; psi1 == null means the current psi is dx1 and dx2 = 0
    // (Euler, whose last stage does not invert), else the current psi is dx2
    int psi_rk;
    const double *psibase, *psi0, *psi1;
    double *psiout;
    const double *dt;
    int mv, nv;
    // psi is already masked (and carries the islands' streamfunction,
    // core/operators.py:482-486): read it as it is
    int premasked;
};
int stage_ortho(const OrthoStage &a, cudaStream_t s);

int vec_add(double *x, const double *y, size_t count, const int *active, cudaStream_t s);
int vec_add_f32(double *x, const float *e, size_t count, const int *active, cudaStream_t s);
int mg_residual_mixed(const LevelView<double> &L, const Analytic &an, const double *x,
                      const double *b, double *r, float *rf, const int *active, cudaStream_t s);
int vec_axpy_const(double *x, double alpha_sub, const double *dev_scalar, size_t count,
                   cudaStream_t s);
// line relaxation (core/gmg/fortran_multigrid.f90:215-317) of a level whose
// operator is analytic (a0, the finest level) or stored: elimination factors
// once, then one sweep per call (no halo fill)
int mg_tri_factor(const LevelView<double> &L, const Analytic *a0, double *gam, double *bet,
                  cudaStream_t s);
int mg_tri_sweep(const LevelView<double> &L, const Analytic *a0, const double *gam,
                 const double *bet, const int *active, cudaStream_t s);
// the finest level's coefficient bits (LevelView::nb) of every point
int mg_nbmask(const LevelView<double> &L, uint16_t *nb, cudaStream_t s);
// x = 0 unless *active == 0
int mg_zero(double *x, size_t n, const int *active, cudaStream_t s);
// x = r (assign) or x += r over the whole array, unless *active == 0
int mg_add(double *x, const double *r, size_t n, bool assign, const int *active,
           cudaStream_t s);

}  // namespace f2d
