// kernels_fused.cu -- engine kernels: multigrid levels, the single-CTA
// coarse solve, and the fused stage kernels of the time step.
//
// Multigrid semantics follow core/gmg/hierarchy.py:98-151 over the routines
// of core/gmg/fortran_multigrid.f90, with every halo fill
// (core/gmg/halo.py:136-141) folded into the kernel that produces the
// interior: a thread that computes an interior value also writes it to the
// halo cells that are its periodic images.  Only the cells each reference
// routine's output depends on are computed:
//   smooth   = sweep 1 on rows/cols 2..m-3 (0-based) into t, sweep 2 on the
//              interior into x, x's halo = periodic images
//              (the Fortran's edge write-backs all land in the halo, which
//              the fill that follows overwrites);
//   residual = interior + periodic halo;
//   restrict = coarse interior + periodic halo;
//   interpolate + (x += r) = fine rows/cols 1..m-2 (what the next smooth
//              reads), so the correction array r is never stored.
#include <cooperative_groups.h>

#include "f2d_common.cuh"
#include "f2d_fused.cuh"
#include "f2d_kernels.cuh"
#include "f2d_adv.cuh"
#include "f2d_tri.cuh"
#include "f2d_batch.cuh"
#include "../../include/fluid2d_gb300.h"

namespace f2d {

// ------------------------------------------------------------ point math
__constant__ int c_dj[5] = {-1, -1, -1, 0, 0};
__constant__ int c_di[5] = {-1, 0, 1, -1, 0};

template <typename T>
F2D_DEV T analytic_coef(const LevelView<T> &L, const AnalyticT<T> &an, int k, int J, int I) {
    const int Jw = wrap(J, L.mv, NH), Iw = wrap(I, L.nv, NH);
    const size_t pc = off(Jw, Iw, L.nv);
    if (L.msk[pc] == 0) return (T)0;
    if (L.msk[off(Jw + c_dj[k], Iw + c_di[k], L.nv)] == 0) return (T)0;
    return k == 4 ? an.a5 : an.sc[k];
}

// the 8 off-diagonal coefficients of point (j, i) in the reference's order
// A1(j,i) A2(j,i) A3(j,i) A4(j,i) A4(j,i+1) A3(j+1,i-1) A2(j+1,i) A1(j+1,i+1)
// For the analytic finest level, the caller guarantees msk(j,i) != 0.  Away
// from the halo no coefficient position needs its periodic image, and each
// coefficient is sc[k] where its neighbour cell is fluid.
template <typename T, bool L0>
F2D_DEV void offdiag(const LevelView<T> &L, const AnalyticT<T> *an, int j, int i, T (&a)[8]) {
    if (L0 && L.nb) {  // the precomputed coefficient bits: one load
        const unsigned b = L.nb[off(j, i, L.nv)];
        a[0] = (b & 1u) ? an->sc[0] : (T)0;
        a[1] = (b & 2u) ? an->sc[1] : (T)0;
        a[2] = (b & 4u) ? an->sc[2] : (T)0;
        a[3] = (b & 8u) ? an->sc[3] : (T)0;
        a[4] = (b & 16u) ? an->sc[3] : (T)0;
        a[5] = (b & 32u) ? an->sc[2] : (T)0;
        a[6] = (b & 64u) ? an->sc[1] : (T)0;
        a[7] = (b & 128u) ? an->sc[0] : (T)0;
    } else if (L0 && j >= NH && j <= L.mv - NH - 2 && i >= NH + 1 && i <= L.nv - NH - 2) {
        const int nv = L.nv;
        const int8_t *m = L.msk + off(j, i, nv);
        a[0] = m[-nv - 1] ? an->sc[0] : (T)0;
        a[1] = m[-nv] ? an->sc[1] : (T)0;
        a[2] = m[-nv + 1] ? an->sc[2] : (T)0;
        a[3] = m[-1] ? an->sc[3] : (T)0;
        a[4] = m[1] ? an->sc[3] : (T)0;
        a[5] = m[nv - 1] ? an->sc[2] : (T)0;
        a[6] = m[nv] ? an->sc[1] : (T)0;
        a[7] = m[nv + 1] ? an->sc[0] : (T)0;
    } else if (L0) {
        a[0] = analytic_coef(L, *an, 0, j, i);
        a[1] = analytic_coef(L, *an, 1, j, i);
        a[2] = analytic_coef(L, *an, 2, j, i);
        a[3] = analytic_coef(L, *an, 3, j, i);
        a[4] = analytic_coef(L, *an, 3, j, i + 1);
        a[5] = analytic_coef(L, *an, 2, j + 1, i - 1);
        a[6] = analytic_coef(L, *an, 1, j + 1, i);
        a[7] = analytic_coef(L, *an, 0, j + 1, i + 1);
    } else {
        const size_t pl = (size_t)L.mv * L.nv, p = off(j, i, L.nv);
        const int nv = L.nv;
        const T *A1 = L.A, *A2 = L.A + pl, *A3 = L.A + 2 * pl, *A4 = L.A + 3 * pl;
        a[0] = A1[p];
        a[1] = A2[p];
        a[2] = A3[p];
        a[3] = A4[p];
        a[4] = A4[p + 1];
        a[5] = A3[p + nv - 1];
        a[6] = A2[p + nv];
        a[7] = A1[p + nv + 1];
    }
}

template <typename T, bool L0>
F2D_DEV T diag_coef(const LevelView<T> &L, const AnalyticT<T> *an, int j, int i) {
    if (L0 && L.nb) return (L.nb[off(j, i, L.nv)] & 256u) ? an->a5 : (T)0;
    if (L0) return analytic_coef(L, *an, 4, j, i);
    return L.A[4 * (size_t)L.mv * L.nv + off(j, i, L.nv)];
}

// omega/|A5| of point (j, i); c3z is its value where A5 = 0, c1/|0|, which
// the host computes once (a division per point costs more than the point)
template <typename T, bool L0>
F2D_DEV T c3_coef(const LevelView<T> &L, const AnalyticT<T> *an, int j, int i, T c3z) {
    if (L0 && L.nb) {  // the diagonal's bit decides a5 != 0 without a float64 compare
        return (L.nb[off(j, i, L.nv)] & 256u) ? an->c3 : c3z;
    }
    if (L0) {
        const T a5 = diag_coef<T, L0>(L, an, j, i);
        return a5 != (T)0 ? an->c3 : c3z;
    }
    return L.A[5 * (size_t)L.mv * L.nv + off(j, i, L.nv)];
}

// c1/|0|: the relaxation factor over a zero diagonal, as the reference's
// smoother computes it for a point without an operator
template <typename T>
inline T c3_zero(T c1) {
    const T zero = (T)0;
    return c1 / fabs(zero);
}

// damped Jacobi (core/gmg/fortran_multigrid.f90:66-85); q == null: x = 0
template <typename T, bool L0>
F2D_DEV T jacobi(const LevelView<T> &L, const AnalyticT<T> *an, const T *q, const T *b, int j,
                 int i, T c3z, T c2) {
    const int nv = L.nv;
    const size_t p = off(j, i, nv);
    if (L.msk[p] == 0) return (T)0;
    const T c3 = c3_coef<T, L0>(L, an, j, i, c3z);
    if (q == nullptr) return c3 * (-b[p]);
    T a[8];
    offdiag<T, L0>(L, an, j, i, a);
    return q[p] * c2 + c3 * (+a[0] * q[p - nv - 1]
                             + a[1] * q[p - nv]
                             + a[2] * q[p - nv + 1]
                             + a[3] * q[p - 1]
                             + a[4] * q[p + 1]
                             + a[5] * q[p + nv - 1]
                             + a[6] * q[p + nv]
                             + a[7] * q[p + nv + 1]
                             - b[p]);
}

// r = b - A x (core/gmg/fortran_multigrid.f90:340-357)
template <typename T, bool L0>
F2D_DEV T residual(const LevelView<T> &L, const AnalyticT<T> *an, const T *x, const T *b, int j,
                   int i) {
    const int nv = L.nv;
    const size_t p = off(j, i, nv);
    if (L.msk[p] == 0) return (T)0;
    T a[8];
    offdiag<T, L0>(L, an, j, i, a);
    const T a5 = diag_coef<T, L0>(L, an, j, i);
    return b[p]
        - a[0] * x[p - nv - 1]
        - a[1] * x[p - nv]
        - a[2] * x[p - nv + 1]
        - a[3] * x[p - 1]
        - a5 * x[p]
        - a[4] * x[p + 1]
        - a[5] * x[p + nv - 1]
        - a[6] * x[p + nv]
        - a[7] * x[p + nv + 1];
}

// full weighting around fine (2*J2-2, 2*I2-2) (core/gmg/fortran_multigrid.f90:531-537)
template <typename T>
F2D_DEV T restrict_value(const int8_t *msk2, int nv2, const T *r, int nv1, int J2, int I2) {
    if (msk2[off(J2, I2, nv2)] == 0) return (T)0;
    const size_t c = off(2 * J2 - 2, 2 * I2 - 2, nv1);
    return (T)0.25 * r[c]
        + (T)0.125 * (r[c - 1] + r[c + 1] + r[c - nv1] + r[c + nv1])
        + (T)0.0625 * (r[c - nv1 - 1] + r[c - nv1 + 1] + r[c + nv1 - 1] + r[c + nv1 + 1]);
}

// the bilinear prolongation of a fine point of parity (dj, di) and mask m1
// from the four coarse points of its cell (masks k.., values x..)
// (core/gmg/fortran_multigrid.f90:449-496)
template <typename T>
F2D_DEV T interp_combine(int m1, int dj, int di, int k00, int k01, int k10, int k11, T x00, T x01,
                         T x10, T x11) {
    if (m1 <= 0) return (T)0;
    if (!dj && !di) return x00;
    if (!dj || !di) {
        const int k = dj ? k00 + k10 : k00 + k01;
        const T c = k == 0 ? (T)0 : (k == 1 ? (T)1 : (T)0.5);
        return (x00 + (dj ? x10 : x01)) * c;
    }
    const int sm4 = k00 + k01 + k10 + k11;
    const T c = sm4 == 0 ? (T)0
                         : sm4 == 1 ? (T)1
                                    : sm4 == 2 ? (T)0.5
                                               : sm4 == 3 ? (T)r4(0.3333333333333333333333333333f)
                                                          : (T)0.25;
    return c * (x00 + x01 + x10 + x11);
}

// bilinear prolongation value at fine (J1, I1), nh = 3
// (core/gmg/fortran_multigrid.f90:449-496)
template <typename T>
F2D_DEV T interp_value(const int8_t *msk1, int nv1, const int8_t *msk2, const T *x2, int nv2,
                       int J1, int I1) {
    const int J2 = (J1 >> 1) + 1, I2 = (I1 >> 1) + 1;
    const int dj = J1 & 1, di = I1 & 1;
    const size_t q = off(J2, I2, nv2);
    // every operand is read up front (one memory round trip; the four coarse
    // points exist for every fine point of rows/cols 1..m-2), and the weight
    // tables are selects rather than indexed local arrays
    const int m1 = msk1[off(J1, I1, nv1)];
    const int k00 = msk2[q], k01 = msk2[q + 1], k10 = msk2[q + nv2], k11 = msk2[q + nv2 + 1];
    const T x00 = x2[q], x01 = x2[q + 1], x10 = x2[q + nv2], x11 = x2[q + nv2 + 1];
    return interp_combine<T>(m1, dj, di, k00, k01, k10, k11, x00, x01, x10, x11);
}

// store an interior value and its periodic halo images
// (core/gmg/fortran_multigrid.f90:365-412)
template <typename T>
F2D_DEV void store_images(T *a, int J, int I, int mv, int nv, T v) {
    for_images(J, I, mv, nv, [&](size_t q) { a[q] = v; });
}

F2D_DEV bool inactive(const int *active) { return active != nullptr && *active == 0; }

// ------------------------------------------------------------ level kernels
constexpr int LV_TX = 32, LV_TY = 8;

// The number of CTAs a level kernel's grid aims at before its tile stops
// shrinking: < 0 twice the SM count, 0 always the largest tile (default:
// a warp's float64 instructions issue at most one per 64 cycles whatever its
// active lanes, so a smaller tile does not shorten a small level's chain and
// measured slower on the 1024^2 step and the ensemble).
int &level_tile_target() {
    static int t = 0;
    return t;
}

static int sm_count() {
    static int n[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!n[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) v = 0;
        n[dev] = v > 0 ? v : 152;
    }
    return n[dev];
}

// The CTA tile of a level kernel over rows x cols points: start from the
// kernel's largest tile (tx, ty) and halve it (the longer side first, down to
// 8 x 4, one warp) while the grid has fewer CTAs than the target.
dim3 level_tile(int rows, int cols, int tx, int ty) {
    int target = level_tile_target();
    if (target == 0) return dim3(tx, ty);
    if (target < 0) target = 2 * sm_count();
    rows = rows > 0 ? rows : 1;
    cols = cols > 0 ? cols : 1;
    while ((long long)((cols + tx - 1) / tx) * ((rows + ty - 1) / ty) < target) {
        if (tx > ty && tx > 8)
            tx /= 2;
        else if (ty > 4)
            ty /= 2;
        else if (tx > 8)
            tx /= 2;
        else
            break;
    }
    return dim3(tx, ty);
}

static inline dim3 lv_grid(int rows, int cols) {
    return grid2d(rows > 0 ? rows : 1, cols > 0 ? cols : 1, dim3(LV_TX, LV_TY));
}

template <typename T>
struct SweepArgs {
    LevelView<T> L;
    AnalyticT<T> an;
    T c1, c2;
    int zero_x;
    const int *active;
    T c3z;  // c1/|0| (c3_zero)
};

template <typename T, bool L0>
F2D_DEV void sweep1_body(const SweepArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const LevelView<T> L = A.L;
    const int i = 2 + vb.x * LV_TX + threadIdx.x;
    const int j = 2 + vb.y * LV_TY + threadIdx.y;
    if (i > L.nv - 3 || j > L.mv - 3) return;
    L.t[off(j, i, L.nv)] = jacobi<T, L0>(L, &A.an, A.zero_x ? nullptr : L.x, L.b, j, i, A.c3z, A.c2);
}

template <typename T, bool L0>
F2D_DEV void sweep2_body(const SweepArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const LevelView<T> L = A.L;
    const int i = NH + vb.x * LV_TX + threadIdx.x;
    const int j = NH + vb.y * LV_TY + threadIdx.y;
    if (i > L.nv - NH - 1 || j > L.mv - NH - 1) return;
    T v = jacobi<T, L0>(L, &A.an, L.t, L.b, j, i, A.c3z, A.c2);
    store_images(L.x, j, i, L.mv, L.nv, v);
}

template <typename T, bool L0>
__global__ void __launch_bounds__(LV_TX *LV_TY) k_sweep1(SweepArgs<T> a) {
    pdl_prologue();
    sweep1_body<T, L0>(a, F2D_VB_NATIVE);
}

template <typename T, bool L0>
__global__ void __launch_bounds__(LV_TX *LV_TY) k_sweep2(SweepArgs<T> a) {
    pdl_prologue();
    sweep2_body<T, L0>(a, F2D_VB_NATIVE);
}

template <typename T>
struct ResidualArgs {
    LevelView<T> L;
    AnalyticT<T> an;
    const T *x, *b;
    T *r;
    float *rf;  // the mixed form's float copy (k_residual_mixed), else unused
    const int *active;
};

// the finest level's residual in column form; false: not launched (the
// residual kernels apply)
template <typename T>
bool residual_column(const LevelView<T> &L, const AnalyticT<T> &an, const T *x, const T *b, T *r,
                     float *rf, const int *active, cudaStream_t s, int *st);

template <typename T, bool L0>
F2D_DEV void residual_body(const ResidualArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const LevelView<T> L = A.L;
    const int i = NH + vb.x * LV_TX + threadIdx.x;
    const int j = NH + vb.y * LV_TY + threadIdx.y;
    if (i > L.nv - NH - 1 || j > L.mv - NH - 1) return;
    store_images(A.r, j, i, L.mv, L.nv, residual<T, L0>(L, &A.an, A.x, A.b, j, i));
}

template <typename T, bool L0>
__global__ void __launch_bounds__(LV_TX *LV_TY) k_residual(ResidualArgs<T> a) {
    pdl_prologue();
    residual_body<T, L0>(a, F2D_VB_NATIVE);
}

// FP64 residual of the finest level with a float copy (the right-hand side
// of the FP32 correction cycles of the mixed form)
F2D_DEV void residual_mixed_body(const ResidualArgs<double> &A, const VB vb) {
    if (inactive(A.active)) return;
    const LevelView<double> L = A.L;
    const int i = NH + vb.x * LV_TX + threadIdx.x;
    const int j = NH + vb.y * LV_TY + threadIdx.y;
    if (i > L.nv - NH - 1 || j > L.mv - NH - 1) return;
    const double v = residual<double, true>(L, &A.an, A.x, A.b, j, i);
    store_images(A.r, j, i, L.mv, L.nv, v);
    store_images(A.rf, j, i, L.mv, L.nv, (float)v);
}

__global__ void __launch_bounds__(LV_TX *LV_TY) k_residual_mixed(ResidualArgs<double> a) {
    pdl_prologue();
    residual_mixed_body(a, F2D_VB_NATIVE);
}

struct BResidualMixed {
    using Args = ResidualArgs<double>;
    static constexpr int THREADS = LV_TX * LV_TY, KIND = BK_ResidualMixed, MIN_BLOCKS = 6;
    F2D_DEV static void run(const Args &a, VB vb) { residual_mixed_body(a, vb); }
};
F2D_BATCH_ENTRY(ResidualMixed, BResidualMixed)

int mg_residual_mixed(const LevelView<double> &L, const Analytic &an, const double *x,
                      const double *b, double *r, float *rf, const int *active, cudaStream_t s) {
    int st = OK;
    if (residual_column<double>(L, an, x, b, r, rf, active, s, &st)) return st;
    dim3 g = lv_grid(L.mv - 2 * NH, L.nv - 2 * NH), bl(LV_TX, LV_TY);
    return launch_body<BResidualMixed>(k_residual_mixed, ResidualArgs<double>{L, an, x, b, r, rf,
                                                                              active},
                                       g, bl, 0, s, "mg_residual_mixed");
}

// x (float64) += e (float32), whole array
struct AddF32Args {
    double *x;
    const float *e;
    size_t n;
    const int *active;
};

F2D_DEV void add_f32_body(const AddF32Args &A, const VB vb) {
    if (inactive(A.active)) return;
    for (size_t q = vb.x * (size_t)blockDim.x + threadIdx.x; q < A.n;
         q += (size_t)vb.gx * blockDim.x)
        A.x[q] = A.x[q] + (double)A.e[q];
}

__global__ void k_add_f32(AddF32Args a) { pdl_prologue();
    add_f32_body(a, F2D_VB_NATIVE); }

struct BAddF32 {
    using Args = AddF32Args;
    static constexpr int THREADS = 256, KIND = BK_AddF32;
    F2D_DEV static void run(const Args &a, VB vb) { add_f32_body(a, vb); }
};
F2D_BATCH_ENTRY(AddF32, BAddF32)

int vec_add_f32(double *x, const float *e, size_t count, const int *active, cudaStream_t s) {
    int blocks = (int)((count + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    return launch_body<BAddF32>(k_add_f32, AddF32Args{x, e, count, active}, dim3(blocks), dim3(256),
                                0, s, "vec_add_f32");
}

template <typename T>
struct RestrictArgs {
    const T *src;
    int nv1;
    const int8_t *msk2;
    int mv2, nv2;
    T *dst;
    const int *active;
};

template <typename T>
F2D_DEV void restrict_body(const RestrictArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const int I2 = NH + vb.x * LV_TX + threadIdx.x;
    const int J2 = NH + vb.y * LV_TY + threadIdx.y;
    if (I2 > A.nv2 - NH - 1 || J2 > A.mv2 - NH - 1) return;
    store_images(A.dst, J2, I2, A.mv2, A.nv2, restrict_value(A.msk2, A.nv2, A.src, A.nv1, J2, I2));
}

template <typename T>
__global__ void __launch_bounds__(LV_TX *LV_TY) k_restrict(RestrictArgs<T> a) {
    pdl_prologue();
    restrict_body<T>(a, F2D_VB_NATIVE);
}

template <typename T>
struct InterpArgs {
    const int8_t *msk1;
    int mv1, nv1;
    const int8_t *msk2;
    const T *x2;
    int nv2;
    T *dst;
    int assign;
    const int *active;
};

// one thread per coarse cell (J, I): its fine points (2J-2+dj, 2I-2+di) in
// rows/cols 1..m-2 share the cell's four coarse values and masks
template <typename T>
F2D_DEV void interp_body(const InterpArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const int I = 1 + vb.x * LV_TX + threadIdx.x;
    const int J = 1 + vb.y * LV_TY + threadIdx.y;
    const int jmax = A.mv1 - 2, imax = A.nv1 - 2;
    if (2 * I - 2 > imax || 2 * J - 2 > jmax) return;
    const int nv2 = A.nv2;
    const size_t p2 = off(J, I, nv2);
    const int k00 = A.msk2[p2], k01 = A.msk2[p2 + 1], k10 = A.msk2[p2 + nv2],
              k11 = A.msk2[p2 + nv2 + 1];
    const T x00 = A.x2[p2], x01 = A.x2[p2 + 1], x10 = A.x2[p2 + nv2], x11 = A.x2[p2 + nv2 + 1];
#pragma unroll
    for (int dj = 0; dj < 2; dj++) {
        const int j = 2 * J - 2 + dj;
        if (j < 1 || j > jmax) continue;
#pragma unroll
        for (int di = 0; di < 2; di++) {
            const int i = 2 * I - 2 + di;
            if (i < 1 || i > imax) continue;
            const size_t p = off(j, i, A.nv1);
            const T v = interp_combine<T>(A.msk1[p], dj, di, k00, k01, k10, k11, x00, x01, x10,
                                          x11);
            A.dst[p] = A.assign ? v : A.dst[p] + v;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(LV_TX *LV_TY) k_interp(InterpArgs<T> a) {
    pdl_prologue();
    interp_body<T>(a, F2D_VB_NATIVE);
}

// the bodies of the level kernels, by type and finest-level flag; KIND is the
// batched kind of the instantiations the batched steps use, else -1
template <typename T, bool L0>
struct BSweep1 {
    using Args = SweepArgs<T>;
    static constexpr int THREADS = LV_TX * LV_TY;
    static constexpr int MIN_BLOCKS = 5;  // near the native kernel's occupancy
    static constexpr int KIND = (sizeof(T) == 8 && L0) ? BK_Sweep1D1 : -1;
    F2D_DEV static void run(const Args &a, VB vb) { sweep1_body<T, L0>(a, vb); }
};
template <typename T, bool L0>
struct BSweep2 {
    using Args = SweepArgs<T>;
    static constexpr int THREADS = LV_TX * LV_TY;
    static constexpr int MIN_BLOCKS = 5;
    static constexpr int KIND = (sizeof(T) == 8 && L0) ? BK_Sweep2D1 : -1;
    F2D_DEV static void run(const Args &a, VB vb) { sweep2_body<T, L0>(a, vb); }
};
template <typename T, bool L0>
struct BResidual {
    using Args = ResidualArgs<T>;
    static constexpr int THREADS = LV_TX * LV_TY;
    static constexpr int MIN_BLOCKS = 5;
    static constexpr int KIND = (sizeof(T) == 8 && L0) ? BK_ResidualD1 : -1;
    F2D_DEV static void run(const Args &a, VB vb) { residual_body<T, L0>(a, vb); }
};
template <typename T>
struct BRestrict {
    using Args = RestrictArgs<T>;
    static constexpr int THREADS = LV_TX * LV_TY;
    static constexpr int KIND = sizeof(T) == 8 ? BK_RestrictD : BK_RestrictF;
    F2D_DEV static void run(const Args &a, VB vb) { restrict_body<T>(a, vb); }
};
template <typename T>
struct BInterp {
    using Args = InterpArgs<T>;
    static constexpr int THREADS = LV_TX * LV_TY;
    static constexpr int KIND = sizeof(T) == 8 ? BK_InterpD : -1;
    F2D_DEV static void run(const Args &a, VB vb) { interp_body<T>(a, vb); }
};
using BSweep1D1 = BSweep1<double, true>;
using BSweep2D1 = BSweep2<double, true>;
using BResidualD1 = BResidual<double, true>;
using BRestrictD = BRestrict<double>;
using BRestrictF = BRestrict<float>;
using BInterpD = BInterp<double>;
F2D_BATCH_ENTRY(Sweep1D1, BSweep1D1)
F2D_BATCH_ENTRY(Sweep2D1, BSweep2D1)
F2D_BATCH_ENTRY(ResidualD1, BResidualD1)
F2D_BATCH_ENTRY(RestrictD, BRestrictD)
F2D_BATCH_ENTRY(RestrictF, BRestrictF)
F2D_BATCH_ENTRY(InterpD, BInterpD)

template <typename T>
int mg_sweep1(const LevelView<T> &L, const AnalyticT<T> *an, T c1, T c2, bool zero_x,
              const int *active, cudaStream_t s) {
    dim3 g = lv_grid(L.mv - 4, L.nv - 4), b(LV_TX, LV_TY);
    SweepArgs<T> a{L, an ? *an : AnalyticT<T>{}, c1, c2, zero_x ? 1 : 0, active, c3_zero(c1)};
    if (an) return launch_body<BSweep1<T, true>>(k_sweep1<T, true>, a, g, b, 0, s, "mg_sweep1");
    return launch_body<BSweep1<T, false>>(k_sweep1<T, false>, a, g, b, 0, s, "mg_sweep1");
}

template <typename T>
int mg_sweep2(const LevelView<T> &L, const AnalyticT<T> *an, T c1, T c2, const int *active,
              cudaStream_t s) {
    dim3 g = lv_grid(L.mv - 2 * NH, L.nv - 2 * NH), b(LV_TX, LV_TY);
    SweepArgs<T> a{L, an ? *an : AnalyticT<T>{}, c1, c2, 0, active, c3_zero(c1)};
    if (an) return launch_body<BSweep2<T, true>>(k_sweep2<T, true>, a, g, b, 0, s, "mg_sweep2");
    return launch_body<BSweep2<T, false>>(k_sweep2<T, false>, a, g, b, 0, s, "mg_sweep2");
}

template <typename T>
int mg_residual(const LevelView<T> &L, const AnalyticT<T> *an, const T *x, const T *b, T *r,
                const int *active, cudaStream_t s) {
    dim3 g = lv_grid(L.mv - 2 * NH, L.nv - 2 * NH), bl(LV_TX, LV_TY);
    ResidualArgs<T> a{L, an ? *an : AnalyticT<T>{}, x, b, r, nullptr, active};
    if constexpr (sizeof(T) == 8) {
        int st = OK;
        if (an && residual_column<T>(L, *an, x, b, r, nullptr, active, s, &st)) return st;
    }
    if (an)
        return launch_body<BResidual<T, true>>(k_residual<T, true>, a, g, bl, 0, s, "mg_residual");
    return launch_body<BResidual<T, false>>(k_residual<T, false>, a, g, bl, 0, s, "mg_residual");
}

template <typename T>
int mg_restrict(const LevelView<T> &fine, const T *src, const LevelView<T> &coarse, T *dst,
                const int *active, cudaStream_t s) {
    dim3 g = lv_grid(coarse.mv - 2 * NH, coarse.nv - 2 * NH), b(LV_TX, LV_TY);
    RestrictArgs<T> a{src, fine.nv, coarse.msk, coarse.mv, coarse.nv, dst, active};
    return launch_body<BRestrict<T>>(k_restrict<T>, a, g, b, 0, s, "mg_restrict");
}

template <typename T>
int mg_interp(const LevelView<T> &coarse, const T *src, const LevelView<T> &fine, T *dst,
              bool assign, const int *active, cudaStream_t s) {
    // coarse cells 1 .. (m-2)/2 + 1 hold the fine rows/cols 1 .. m-2
    dim3 g = lv_grid(((fine.mv - 2) >> 1) + 1, ((fine.nv - 2) >> 1) + 1), b(LV_TX, LV_TY);
    InterpArgs<T> a{fine.msk, fine.mv, fine.nv, coarse.msk, src, coarse.nv, dst,
                    assign ? 1 : 0, active};
    return launch_body<BInterp<T>>(k_interp<T>, a, g, b, 0, s, "mg_interp");
}

// ------------------------------------------------------------ fused level kernels
// One smoothtwicewitha call in one kernel.  The CTA's input values (x, or
// x + prolongation of the coarse correction, or the prolongation alone, or
// zero) on its tile plus a 2-cell ring go to shared memory, the first sweep
// on the tile plus a 1-cell ring goes to shared memory, and the second sweep
// writes the tile (and its periodic halo images) to a separate output array:
// x is read by neighbouring CTAs while they run, so it is never updated in
// place.  Same arithmetic, same order as the unfused kernels.
//
// The tile is the CTA shape (blockDim), chosen per level by level_tile().
constexpr int FS_TX = 32, FS_TY = 16;

// quotient and remainder of a small index by a small divisor through a float
// reciprocal: q < 2^16 and d <= 64 keep the error of (q + 0.5) * (1/d) far
// below the 0.5/d margin to the next integer, so the floor is exact.
F2D_DEV int small_div(int q, float inv) { return (int)(((float)q + 0.5f) * inv); }

// CTA threads: one per tile point (the input ring and the first sweep's ring
// take a second pass), or one per input point so that every phase is a
// single pass (level_one_pass()).
constexpr int FS_THREADS_MAX = ((FS_TX + 4) * (FS_TY + 4) + 31) / 32 * 32;
// two resident CTAs of the largest shape per SM: at most 44 registers, so a
// 512-thread CTA keeps the occupancy (two to three per SM) of a kernel bounded
// for 512 threads alone
constexpr int FS_MIN_BLOCKS = 2;

// 0 (default): one thread per tile point; 1: one per input point when the
// grid has fewer than two CTAs per SM; 2: always one per input point.  On the
// 1024^2 steps and the 96-instance ensemble 1 and 2 measured equal or slower
// than 0 (the small levels' time is not in the second passes).
int &level_one_pass() {
    static int m = 0;
    return m;
}

static inline unsigned smooth_fused_threads(dim3 tile, dim3 grid) {
    const int m = level_one_pass();
    const bool one = m == 2 || (m == 1 && (long long)grid.x * grid.y < 2LL * sm_count());
    if (!one) return tile.x * tile.y;
    return ((tile.x + 4) * (tile.y + 4) + 31) / 32 * 32;
}

template <typename T>
size_t smooth_fused_smem(dim3 b) {
    return sizeof(T) * ((size_t)(b.y + 4) * (b.x + 4) + (size_t)(b.y + 2) * (b.x + 2));
}

template <typename T>
struct CoarseSrc {
    const int8_t *msk;
    const T *x;
    int nv;
};


template <typename T>
struct SmoothFusedArgs {
    LevelView<T> L;
    AnalyticT<T> an;
    T c1, c2;
    int xmode;
    CoarseSrc<T> cs;
    T *out;
    const int *active;
    int tx, ty;  // the tile
    T c3z;       // c3 where the diagonal is 0 (c1/|0|), computed on the host
};

template <typename T, bool L0>
F2D_DEV void smooth_fused_body(const SmoothFusedArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const int TX = A.tx, TY = A.ty, NT = (int)blockDim.x;
    const int XW = TX + 4, XH = TY + 4, TW = TX + 2, TH = TY + 2;
    extern __shared__ __align__(16) unsigned char sm[];
    T *xs = (T *)sm;
    T *ts = xs + XH * XW;
    const LevelView<T> L = A.L;
    const AnalyticT<T> an = A.an;
    const T c1 = A.c1, c2 = A.c2;
    const int xmode = A.xmode;
    const CoarseSrc<T> cs = A.cs;
    T *out = A.out;
    const int mv = L.mv, nv = L.nv;
    const int i0 = NH + vb.x * TX, j0 = NH + vb.y * TY;
    const int tid = (int)threadIdx.x;
    // input x on [j0-2, j0+TY+1] x [i0-2, i0+TX+1], inside rows/cols 1..m-2
    if (xmode == X_IN) {
        const float inv = 1.0f / (float)XW;
        for (int q = tid; q < XH * XW; q += NT) {
            const int qj = small_div(q, inv);
            const int j = j0 - 2 + qj, i = i0 - 2 + (q - qj * XW);
            if (j < 1 || j > mv - 2 || i < 1 || i > nv - 2) continue;
            xs[q] = L.x[off(j, i, nv)];
        }
    } else if (xmode != X_ZERO) {
        // the prolongation by coarse cells (the fine points 2J-2+dj,
        // 2I-2+di of cell (J, I) share its four coarse values and masks)
        const int ja = max(1, j0 - 2), jb = min(mv - 2, j0 + TY + 1);
        const int ia = max(1, i0 - 2), ib = min(nv - 2, i0 + TX + 1);
        const int Ja = (ja >> 1) + 1, Ia = (ia >> 1) + 1;
        const int ch = (jb >> 1) + 1 - Ja + 1, cw = (ib >> 1) + 1 - Ia + 1;
        const int nc2 = cs.nv;
        for (int q = tid; q < ch * cw; q += NT) {
            const int cr = q / cw, J = Ja + cr, I = Ia + q - cr * cw;
            const size_t p2 = off(J, I, nc2);
            const int k00 = cs.msk[p2], k01 = cs.msk[p2 + 1], k10 = cs.msk[p2 + nc2],
                      k11 = cs.msk[p2 + nc2 + 1];
            const T x00 = cs.x[p2], x01 = cs.x[p2 + 1], x10 = cs.x[p2 + nc2],
                    x11 = cs.x[p2 + nc2 + 1];
#pragma unroll
            for (int dj = 0; dj < 2; dj++) {
                const int j = 2 * J - 2 + dj;
                if (j < ja || j > jb) continue;
#pragma unroll
                for (int di = 0; di < 2; di++) {
                    const int i = 2 * I - 2 + di;
                    if (i < ia || i > ib) continue;
                    const size_t p = off(j, i, nv);
                    const T c = interp_combine<T>(L.msk[p], dj, di, k00, k01, k10, k11, x00, x01,
                                                  x10, x11);
                    xs[(j - (j0 - 2)) * XW + (i - (i0 - 2))] =
                        xmode == X_PLUS_INTERP ? L.x[p] + c : c;
                }
            }
        }
    }
    __syncthreads();
    // first sweep on [j0-1, j0+TY] x [i0-1, i0+TX], inside rows/cols 2..m-3
    const float invt = 1.0f / (float)TW;
    for (int q = tid; q < TH * TW; q += NT) {
        const int qj = small_div(q, invt);
        const int j = j0 - 1 + qj, i = i0 - 1 + (q - qj * TW);
        if (j < 2 || j > mv - 3 || i < 2 || i > nv - 3) continue;
        const size_t p = off(j, i, nv);
        T v;
        if (L.msk[p] == 0) {
            v = (T)0;
        } else {
            const T c3 = c3_coef<T, L0>(L, &an, j, i, A.c3z);
            if (xmode == X_ZERO) {
                v = c3 * (-L.b[p]);
            } else {
                T a[8];
                offdiag<T, L0>(L, &an, j, i, a);
                const T *x = xs + (j - (j0 - 2)) * XW + (i - (i0 - 2));
                v = x[0] * c2 + c3 * (+a[0] * x[-XW - 1]
                                      + a[1] * x[-XW]
                                      + a[2] * x[-XW + 1]
                                      + a[3] * x[-1]
                                      + a[4] * x[1]
                                      + a[5] * x[XW - 1]
                                      + a[6] * x[XW]
                                      + a[7] * x[XW + 1]
                                      - L.b[p]);
            }
        }
        ts[q] = v;
    }
    __syncthreads();
    // second sweep on the tile's interior points
    const float invx = 1.0f / (float)TX;
    for (int q = tid; q < TX * TY; q += NT) {
        const int qj = small_div(q, invx);
        const int j = j0 + qj, i = i0 + (q - qj * TX);
        if (j > mv - NH - 1 || i > nv - NH - 1) continue;
        const size_t p = off(j, i, nv);
        T v = (T)0;
        if (L.msk[p] != 0) {
            const T c3 = c3_coef<T, L0>(L, &an, j, i, A.c3z);
            T a[8];
            offdiag<T, L0>(L, &an, j, i, a);
            const T *t = ts + (j - (j0 - 1)) * TW + (i - (i0 - 1));
            v = t[0] * c2 + c3 * (+a[0] * t[-TW - 1]
                                  + a[1] * t[-TW]
                                  + a[2] * t[-TW + 1]
                                  + a[3] * t[-1]
                                  + a[4] * t[1]
                                  + a[5] * t[TW - 1]
                                  + a[6] * t[TW]
                                  + a[7] * t[TW + 1]
                                  - L.b[p]);
        }
        store_images(out, j, i, mv, nv, v);
    }
}

template <typename T, bool L0>
__global__ void __launch_bounds__(FS_THREADS_MAX, FS_MIN_BLOCKS) k_smooth_fused(SmoothFusedArgs<T> a) {
    pdl_prologue();
    smooth_fused_body<T, L0>(a, F2D_VB_NATIVE);
}

template <typename T, bool L0>
struct BSmoothFused {
    using Args = SmoothFusedArgs<T>;
    static constexpr int THREADS = FS_THREADS_MAX;
    static constexpr int MIN_BLOCKS = FS_MIN_BLOCKS;
    // (the float finest level runs smooth_l0_body, batched as SmoothFusedF1)
    static constexpr int KIND = sizeof(T) == 8 ? (L0 ? -1 : BK_SmoothFusedD0)
                                               : (L0 ? -1 : BK_SmoothFusedF0);
    F2D_DEV static void run(const Args &a, VB vb) { smooth_fused_body<T, L0>(a, vb); }
};
using BSmoothFusedD0 = BSmoothFused<double, false>;
using BSmoothFusedF0 = BSmoothFused<float, false>;
F2D_BATCH_ENTRY(SmoothFusedD0, BSmoothFusedD0)
F2D_BATCH_ENTRY(SmoothFusedF0, BSmoothFusedF0)

// The finest level's fused smoother (analytic operator through the
// coefficient bits), for the float form whose kernel is bound by its
// instruction count: a 32 x 32 tile per CTA of 256 threads, each thread a
// column of four points of the tile; x on the tile's 2-ring, and the first
// sweep's inputs (coefficient bits, mask, b) on its 1-ring, are staged in
// shared memory once with 32-bit offsets from the tile's origin, so both
// sweeps read only shared memory.  Same arithmetic in the same order as
// jacobi(); the bits give the coefficients exactly as offdiag() selects them.
constexpr int SL_T = 32, SL_TY = 8, SL_THREADS = SL_T * SL_TY;
constexpr int SL_XW = SL_T + 4, SL_TW = SL_T + 2;

template <typename T>
size_t smooth_l0_smem() {
    return sizeof(T) * (size_t)(SL_XW * SL_XW + 2 * SL_TW * SL_TW) +
           sizeof(uint16_t) * SL_TW * SL_TW + SL_TW * SL_TW;
}

template <typename T>
F2D_DEV T jacobi_bits(unsigned bits, const T *x, int W, T bq, const AnalyticT<T> &an, T c2,
                      T c3z) {
    const T c3 = (bits & 256u) ? an.c3 : c3z;
    const T a0 = (bits & 1u) ? an.sc[0] : (T)0, a1 = (bits & 2u) ? an.sc[1] : (T)0,
            a2 = (bits & 4u) ? an.sc[2] : (T)0, a3 = (bits & 8u) ? an.sc[3] : (T)0,
            a4 = (bits & 16u) ? an.sc[3] : (T)0, a5 = (bits & 32u) ? an.sc[2] : (T)0,
            a6 = (bits & 64u) ? an.sc[1] : (T)0, a7 = (bits & 128u) ? an.sc[0] : (T)0;
    return x[0] * c2 + c3 * (+a0 * x[-W - 1]
                             + a1 * x[-W]
                             + a2 * x[-W + 1]
                             + a3 * x[-1]
                             + a4 * x[1]
                             + a5 * x[W - 1]
                             + a6 * x[W]
                             + a7 * x[W + 1]
                             - bq);
}

// one damped-Jacobi update of a point whose 3x3 block is fluid, through the
// separable form of the analytic 9-point operator (x: the point in a row-major
// array of row width W)
template <typename T>
F2D_DEV T separable9(const T *x, int W, T bq, T c3, T k0, T k1) {
    const T corners = (x[-W - 1] + x[-W + 1]) + (x[W - 1] + x[W + 1]);
    const T edges = (x[-W] + x[W]) + (x[-1] + x[1]);
    const T V = fma((T)4, x[0], fma((T)2, edges, corners));
    return fma(k1, V, fma(k0, x[0], -c3 * bq));
}

// ------------------------------------------------------------ finest-level sweeps, column form
// The float64 finest level's two damped-Jacobi sweeps (product build) with
// each thread taking a column of SC_K = 4 consecutive points: the 3 x
// (SC_K + 2) input values around them (and their b, coefficient bits and
// mask) are loaded up front, one memory round trip, and every point's
// neighbours come from registers.  Where a point's 3x3 block is fluid the
// analytic 9-point operator is (c/4)(V - 4x), V the [1 2 1] x [1 2 1] sum,
// built from row sums shared by three points, so a sweep is
//     x' = k0 x + k1 V - c3 b,   k1 = c3 c/4,  k0 = c2 - 4 k1
// (8 float64 operations a point instead of 11); other points take the
// reference's expression (jacobi_bits).  The same function, another
// rounding: the exact build keeps the sweep kernels.  Same points, inputs and
// outputs as sweep1_body / sweep2_body.
constexpr int SC_K = 4;

template <typename T>
struct SweepCArgs {
    LevelView<T> L;
    AnalyticT<T> an;
    T c1, c2;
    T c3z;         // c3 where the diagonal is 0: c1/|0|, computed on the host
    T k0, k1;      // separable update constants
    int second;    // 0: first sweep (x or zero -> t), 1: second (t -> x and its images)
    int zero_x;
    const int *active;
};

template <typename T>
F2D_DEV void sweepc_body(const SweepCArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const LevelView<T> L = A.L;
    const AnalyticT<T> an = A.an;
    const int mv = L.mv, nv = L.nv, second = A.second;
    const int lo = second ? NH : 2, hj = second ? mv - NH - 1 : mv - 3,
              hi = second ? nv - NH - 1 : nv - 3;
    const int i = lo + vb.x * LV_TX + (int)threadIdx.x;
    const int jb = lo + (vb.y * LV_TY + (int)threadIdx.y) * SC_K;
    if (i > hi || jb > hj) return;
    const T c2 = A.c2, c3z = A.c3z;
    // b, bits and mask of the column's points (mk < 0: beyond the last row)
    T bq[SC_K];
    unsigned bt[SC_K];
    int mk[SC_K];
#pragma unroll
    for (int k = 0; k < SC_K; k++) {
        const int j = jb + k;
        bq[k] = (T)0;
        bt[k] = 0u;
        mk[k] = -1;
        if (j <= hj) {
            const size_t p = off(j, i, nv);
            bq[k] = L.b[p];
            bt[k] = L.nb[p];
            mk[k] = L.msk[p];
        }
    }
    T v[SC_K];
    if (!second && A.zero_x) {
#pragma unroll
        for (int k = 0; k < SC_K; k++)
            v[k] = mk[k] <= 0 ? (T)0 : ((bt[k] & 256u) ? an.c3 : c3z) * (-bq[k]);
    } else {
        const T *__restrict__ q = second ? L.t : L.x;
        // rows jb-1 .. jb+SC_K, columns i-1 .. i+1 (rows past hj + 1 are not needed)
        T w[SC_K + 2][3];
#pragma unroll
        for (int r = 0; r < SC_K + 2; r++) {
            const int j = jb - 1 + r;
            w[r][0] = w[r][1] = w[r][2] = (T)0;
            if (j <= hj + 1) {
                const T *row = q + off(j, i, nv);
                w[r][0] = row[-1];
                w[r][1] = row[0];
                w[r][2] = row[1];
            }
        }
        T h[SC_K + 2];
#pragma unroll
        for (int r = 0; r < SC_K + 2; r++) h[r] = fma((T)2, w[r][1], w[r][0] + w[r][2]);
        bool full = true;
#pragma unroll
        for (int k = 0; k < SC_K; k++) full = full && (mk[k] <= 0 || bt[k] == 511u);
        // the separable form alone for a warp whose points all have fluid
        // blocks (no second expression for the compiler to predicate in)
        if (__all_sync(__activemask(), full)) {
#pragma unroll
            for (int k = 0; k < SC_K; k++) {
                const T V = fma((T)2, h[k + 1], h[k] + h[k + 2]);
                const T u = fma(A.k1, V, fma(A.k0, w[k + 1][1], -an.c3 * bq[k]));
                v[k] = mk[k] > 0 ? u : (T)0;
            }
        } else {
#pragma unroll
        for (int k = 0; k < SC_K; k++) {
            v[k] = (T)0;
            if (mk[k] <= 0) continue;
            const unsigned bits = bt[k];
            if (bits == 511u) {
                const T V = fma((T)2, h[k + 1], h[k] + h[k + 2]);
                v[k] = fma(A.k1, V, fma(A.k0, w[k + 1][1], -an.c3 * bq[k]));
            } else {
                const T c3 = (bits & 256u) ? an.c3 : c3z;
                const T a0 = (bits & 1u) ? an.sc[0] : (T)0, a1 = (bits & 2u) ? an.sc[1] : (T)0,
                        a2 = (bits & 4u) ? an.sc[2] : (T)0, a3 = (bits & 8u) ? an.sc[3] : (T)0,
                        a4 = (bits & 16u) ? an.sc[3] : (T)0, a5 = (bits & 32u) ? an.sc[2] : (T)0,
                        a6 = (bits & 64u) ? an.sc[1] : (T)0, a7 = (bits & 128u) ? an.sc[0] : (T)0;
                v[k] = w[k + 1][1] * c2 + c3 * (+a0 * w[k][0]
                                               + a1 * w[k][1]
                                               + a2 * w[k][2]
                                               + a3 * w[k + 1][0]
                                               + a4 * w[k + 1][2]
                                               + a5 * w[k + 2][0]
                                               + a6 * w[k + 2][1]
                                               + a7 * w[k + 2][2]
                                               - bq[k]);
            }
        }
        }
    }
#pragma unroll
    for (int k = 0; k < SC_K; k++) {
        if (mk[k] < 0) break;
        const int j = jb + k;
        if (second)
            store_images(L.x, j, i, mv, nv, v[k]);
        else
            L.t[off(j, i, nv)] = v[k];
    }
}

template <typename T>
__global__ void __launch_bounds__(LV_TX *LV_TY) k_sweepc(SweepCArgs<T> a) {
    pdl_prologue();
    sweepc_body<T>(a, F2D_VB_NATIVE);
}

int &separable_mode();
// The finest level's residual r = b - A x (core/gmg/fortran_multigrid.f90:
// 340-357) in the same column form: with corners e/2 and edges e, on a fluid
// block A x = (e/2) V + (a5 - 2e) x, so r = b + kv V + kx x with kv = -e/2,
// kx = 2e - a5 (7 float64 operations a point instead of 10); other points
// take the reference's expression.  r is written with its periodic images
// and, for the mixed form, a float copy rf.  Same points, inputs and outputs
// as residual_body / residual_mixed_body.
template <typename T>
struct ResidualCArgs {
    LevelView<T> L;
    AnalyticT<T> an;
    const T *x, *b;
    T *r;
    float *rf;
    T kv, kx;  // on a fluid block: r = b + kv V + kx x
    const int *active;
};

template <typename T>
F2D_DEV void residualc_body(const ResidualCArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const LevelView<T> L = A.L;
    const AnalyticT<T> an = A.an;
    const int mv = L.mv, nv = L.nv;
    const int hj = mv - NH - 1, hi = nv - NH - 1;
    const int i = NH + vb.x * LV_TX + (int)threadIdx.x;
    const int jb = NH + (vb.y * LV_TY + (int)threadIdx.y) * SC_K;
    if (i > hi || jb > hj) return;
    const T *__restrict__ q = A.x;
    T bq[SC_K];
    unsigned bt[SC_K];
    int mk[SC_K];
#pragma unroll
    for (int k = 0; k < SC_K; k++) {
        const int j = jb + k;
        bq[k] = (T)0;
        bt[k] = 0u;
        mk[k] = -1;
        if (j <= hj) {
            const size_t p = off(j, i, nv);
            bq[k] = A.b[p];
            bt[k] = L.nb[p];
            mk[k] = L.msk[p];
        }
    }
    T w[SC_K + 2][3];
#pragma unroll
    for (int r = 0; r < SC_K + 2; r++) {
        const int j = jb - 1 + r;
        w[r][0] = w[r][1] = w[r][2] = (T)0;
        if (j <= hj + 1) {
            const T *row = q + off(j, i, nv);
            w[r][0] = row[-1];
            w[r][1] = row[0];
            w[r][2] = row[1];
        }
    }
    T h[SC_K + 2];
#pragma unroll
    for (int r = 0; r < SC_K + 2; r++) h[r] = fma((T)2, w[r][1], w[r][0] + w[r][2]);
    bool full = true;
#pragma unroll
    for (int k = 0; k < SC_K; k++) full = full && (mk[k] <= 0 || bt[k] == 511u);
    T v[SC_K];
    if (__all_sync(__activemask(), full)) {
#pragma unroll
        for (int k = 0; k < SC_K; k++) {
            const T V = fma((T)2, h[k + 1], h[k] + h[k + 2]);
            const T u = fma(A.kv, V, fma(A.kx, w[k + 1][1], bq[k]));
            v[k] = mk[k] > 0 ? u : (T)0;
        }
    } else {
#pragma unroll
        for (int k = 0; k < SC_K; k++) {
            v[k] = (T)0;
            if (mk[k] <= 0) continue;
            const unsigned bits = bt[k];
            if (bits == 511u) {
                const T V = fma((T)2, h[k + 1], h[k] + h[k + 2]);
                v[k] = fma(A.kv, V, fma(A.kx, w[k + 1][1], bq[k]));
            } else {
                const T a0 = (bits & 1u) ? an.sc[0] : (T)0, a1 = (bits & 2u) ? an.sc[1] : (T)0,
                        a2 = (bits & 4u) ? an.sc[2] : (T)0, a3 = (bits & 8u) ? an.sc[3] : (T)0,
                        a4 = (bits & 16u) ? an.sc[3] : (T)0, a5 = (bits & 32u) ? an.sc[2] : (T)0,
                        a6 = (bits & 64u) ? an.sc[1] : (T)0, a7 = (bits & 128u) ? an.sc[0] : (T)0;
                const T d = (bits & 256u) ? an.a5 : (T)0;
                v[k] = bq[k]
                    - a0 * w[k][0]
                    - a1 * w[k][1]
                    - a2 * w[k][2]
                    - a3 * w[k + 1][0]
                    - d * w[k + 1][1]
                    - a4 * w[k + 1][2]
                    - a5 * w[k + 2][0]
                    - a6 * w[k + 2][1]
                    - a7 * w[k + 2][2];
            }
        }
    }
#pragma unroll
    for (int k = 0; k < SC_K; k++) {
        if (mk[k] < 0) break;
        const int j = jb + k;
        store_images(A.r, j, i, mv, nv, v[k]);
        if (A.rf) store_images(A.rf, j, i, mv, nv, (float)v[k]);
    }
}

template <typename T>
__global__ void __launch_bounds__(LV_TX *LV_TY) k_residualc(ResidualCArgs<T> a) {
    pdl_prologue();
    residualc_body<T>(a, F2D_VB_NATIVE);
}

// false (nothing launched) where the column form does not apply
// (column_l0_applies: the separable mode off, no coefficient bits, not the
// 9-point operator with corners = edges / 2, a step being recorded, a grid
// of fewer CTAs than SMs)
template <typename T>
bool residual_column(const LevelView<T> &L, const AnalyticT<T> &an, const T *x, const T *b, T *r,
                     float *rf, const int *active, cudaStream_t s, int *st) {
    *st = OK;
    if (!column_l0_applies(L, an)) return false;
    const int rows = L.mv - 2 * NH, cols = L.nv - 2 * NH;
    const dim3 g((unsigned)((cols + LV_TX - 1) / LV_TX),
                 (unsigned)((rows + LV_TY * SC_K - 1) / (LV_TY * SC_K)));
    ResidualCArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.L = L;
    a.an = an;
    a.x = x;
    a.b = b;
    a.r = r;
    a.rf = rf;
    a.kv = -an.sc[0];                // -e/2
    a.kx = (T)4 * an.sc[0] - an.a5;  // 2e - a5
    a.active = active;
    *st = cuda_status((cudaError_t)launch_pdl(k_residualc<T>, a, g, dim3(LV_TX, LV_TY), 0, s),
                      "mg_residual column");
    return true;
}

// 1 (the product build's default): the float64 finest level's sweeps and
// residual take the column form where the operator is the 9-point one and
// the grid has at least one CTA per SM; 2: at every grid size; 0: the sweep
// and residual kernels
int &separable_mode() {
#ifdef F2D_EXACT
    static int m = 0;
#else
    static int m = 1;
#endif
    return m;
}

// whether a level of L's size takes the column form now: the mode on, no
// step being recorded, and (mode 1) a grid of at least one CTA per SM
template <typename T>
bool column_applies(const LevelView<T> &L) {
    const int mode = separable_mode();
    if (!mode || recorder() != nullptr) return false;
    const long long tiles = (long long)((L.nv - 4 + LV_TX - 1) / LV_TX) *
                            ((L.mv - 4 + LV_TY * SC_K - 1) / (LV_TY * SC_K));
    return mode == 2 || tiles >= sm_count();
}
template bool column_applies<double>(const LevelView<double> &);
template bool column_applies<float>(const LevelView<float> &);

// the same for the finest level, whose operator must also be the analytic
// 9-point one with corners = edges / 2 and have its coefficient bits
template <typename T>
bool column_l0_applies(const LevelView<T> &L, const AnalyticT<T> &an) {
    if (!L.nb || !column_applies(L)) return false;
    const T e = an.sc[1];
    return e != (T)0 && an.sc[3] == e && an.sc[0] == (T)0.5 * e && an.sc[2] == an.sc[0];
}
template bool column_l0_applies<double>(const LevelView<double> &, const AnalyticT<double> &);

// The finest level's two sweeps in column form; *done = false and nothing
// launched where column_l0_applies does not hold (a step being recorded
// included: a batch takes the sweep kernels, this kernel is not a batched
// body).
template <typename T>
int mg_sweeps_column(const LevelView<T> &L, const AnalyticT<T> &an, T c1, T c2, bool zero_x,
                     const int *active, cudaStream_t s, bool *done) {
    *done = false;
    if (!column_l0_applies(L, an)) return OK;
    const T e = an.sc[1];
    SweepCArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.L = L;
    a.an = an;
    a.c1 = c1;
    a.c2 = c2;
    a.c3z = c3_zero(c1);
    a.k1 = an.c3 * e * (T)0.5;
    a.k0 = c2 - (T)4 * a.k1;
    a.zero_x = zero_x ? 1 : 0;
    a.active = active;
    const dim3 b(LV_TX, LV_TY);
    for (int second = 0; second < 2; second++) {
        a.second = second;
        const int lo = second ? NH : 2;
        const int rows = (second ? L.mv - NH - 1 : L.mv - 3) - lo + 1;
        const int cols = (second ? L.nv - NH - 1 : L.nv - 3) - lo + 1;
        const dim3 g((unsigned)((cols + LV_TX - 1) / LV_TX),
                     (unsigned)((rows + LV_TY * SC_K - 1) / (LV_TY * SC_K)));
        const int st = cuda_status((cudaError_t)launch_pdl(k_sweepc<T>, a, g, b, 0, s),
                                   "mg_sweeps_column");
        if (st) return st;
    }
    *done = true;
    return OK;
}
template bool residual_column<double>(const LevelView<double> &, const AnalyticT<double> &,
                                     const double *, const double *, double *, float *,
                                     const int *, cudaStream_t, int *);
template int mg_sweeps_column<double>(const LevelView<double> &, const AnalyticT<double> &, double,
                                      double, bool, const int *, cudaStream_t, bool *);

// ---- the same column form on a stored level (levels >= 1, float64 product
// build).  Where the stored stencil of a point is the level's uniform one
// (flag uf = 1: corners c, vertical edges ey, horizontal edges ex and c3 as
// chosen at set-up), the sum of its 8 neighbours is
//     c (s[j-1] + s[j+1]) + ey (x[j-1][i] + x[j+1][i]) + ex s[j],
// s[r] = x[r][i-1] + x[r][i+1] shared down the column, and the damped
// Jacobi update x' = c2 x + c3 (sum - b) takes 8.5 float64 operations a point
// instead of 11 (and no coefficient loads); other points take the
// reference's expression (jacobi, core/gmg/fortran_multigrid.f90:66-85).
template <typename T>
struct SweepUArgs {
    LevelView<T> L;
    const uint8_t *uf;
    T kc, key, kex;  // c3 c, c3 ey, c3 ex
    T c2, c3u;       // 1 - omega; the uniform points' c3
    int second, zero_x;
    const int *active;
};

template <typename T>
F2D_DEV void sweepu_body(const SweepUArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const LevelView<T> L = A.L;
    const int mv = L.mv, nv = L.nv, second = A.second;
    const int lo = second ? NH : 2, hj = second ? mv - NH - 1 : mv - 3,
              hi = second ? nv - NH - 1 : nv - 3;
    const int i = lo + vb.x * LV_TX + (int)threadIdx.x;
    const int jb = lo + (vb.y * LV_TY + (int)threadIdx.y) * SC_K;
    if (i > hi || jb > hj) return;
    const T *__restrict__ q = second ? L.t : L.x;
    T bq[SC_K];
    int uq[SC_K], mk[SC_K];
#pragma unroll
    for (int k = 0; k < SC_K; k++) {
        const int j = jb + k;
        bq[k] = (T)0;
        uq[k] = 0;
        mk[k] = -1;
        if (j <= hj) {
            const size_t p = off(j, i, nv);
            bq[k] = L.b[p];
            uq[k] = A.uf[p];
            mk[k] = L.msk[p];
        }
    }
    T v[SC_K];
    bool full = true;
#pragma unroll
    for (int k = 0; k < SC_K; k++) full = full && (mk[k] <= 0 || uq[k]);
    if (!second && A.zero_x) {
#pragma unroll
        for (int k = 0; k < SC_K; k++)
            v[k] = mk[k] < 0 ? (T)0 : jacobi<T, false>(L, nullptr, nullptr, L.b, jb + k, i, (T)0, A.c2);
    } else if (__all_sync(__activemask(), full)) {
        T sr[SC_K + 2], mr[SC_K + 2];
#pragma unroll
        for (int r = 0; r < SC_K + 2; r++) {
            const int j = jb - 1 + r;
            sr[r] = mr[r] = (T)0;
            if (j <= hj + 1) {
                const T *row = q + off(j, i, nv);
                sr[r] = row[-1] + row[1];
                mr[r] = row[0];
            }
        }
#pragma unroll
        for (int k = 0; k < SC_K; k++) {
            const T t1 = sr[k] + sr[k + 2], t2 = mr[k] + mr[k + 2];
            const T u = fma(A.kc, t1, fma(A.key, t2, fma(A.kex, sr[k + 1],
                                                        fma(A.c2, mr[k + 1], -A.c3u * bq[k]))));
            v[k] = mk[k] > 0 ? u : (T)0;
        }
    } else {
#pragma unroll
        for (int k = 0; k < SC_K; k++)
            v[k] = mk[k] < 0 ? (T)0 : jacobi<T, false>(L, nullptr, q, L.b, jb + k, i, (T)0, A.c2);
    }
#pragma unroll
    for (int k = 0; k < SC_K; k++) {
        if (mk[k] < 0) break;
        const int j = jb + k;
        if (second)
            store_images(L.x, j, i, mv, nv, v[k]);
        else
            L.t[off(j, i, nv)] = v[k];
    }
}

template <typename T>
__global__ void __launch_bounds__(LV_TX *LV_TY) k_sweepu(SweepUArgs<T> a) {
    pdl_prologue();
    sweepu_body<T>(a, F2D_VB_NATIVE);
}


template <typename T>
int mg_sweeps_uniform(const LevelView<T> &L, const uint8_t *uf, const T *st, T c1, T c2,
                      bool zero_x, const int *active, cudaStream_t s) {
    (void)c1;
    SweepUArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.L = L;
    a.uf = uf;
    a.c3u = st[3];
    a.kc = st[3] * st[0];
    a.key = st[3] * st[1];
    a.kex = st[3] * st[2];
    a.c2 = c2;
    a.zero_x = zero_x ? 1 : 0;
    a.active = active;
    const dim3 b(LV_TX, LV_TY);
    for (int second = 0; second < 2; second++) {
        a.second = second;
        const int lo = second ? NH : 2;
        const int rows = (second ? L.mv - NH - 1 : L.mv - 3) - lo + 1;
        const int cols = (second ? L.nv - NH - 1 : L.nv - 3) - lo + 1;
        const dim3 g((unsigned)((cols + LV_TX - 1) / LV_TX),
                     (unsigned)((rows + LV_TY * SC_K - 1) / (LV_TY * SC_K)));
        const int st2 = cuda_status((cudaError_t)launch_pdl(k_sweepu<T>, a, g, b, 0, s),
                                    "mg_sweeps_uniform");
        if (st2) return st2;
    }
    return OK;
}
template int mg_sweeps_uniform<double>(const LevelView<double> &, const uint8_t *, const double *,
                                       double, double, bool, const int *, cudaStream_t);
template int mg_sweeps_uniform<float>(const LevelView<float> &, const uint8_t *, const float *,
                                      float, float, bool, const int *, cudaStream_t);

// Set-up of a stored level's uniform stencil: the stencil (c, ey, ex, c3,
// a5) of the points at (1 + 2k) / 8 of the interior, k = 0..3, in both
// directions, where the stencil has the uniform form (4 corners equal,
// vertical and horizontal edges pairwise equal); out[6 * n + 5] = 1 there.
__global__ void k_stencil_samples(const double *A6, const int8_t *msk, int mv, int nv,
                                  double *out) {
    const int n = (int)threadIdx.x;
    if (n >= 16) return;
    const int j = NH + (mv - 2 * NH) * (1 + 2 * (n / 4)) / 8;
    const int i = NH + (nv - 2 * NH) * (1 + 2 * (n % 4)) / 8;
    const size_t pl = (size_t)mv * nv, p = off(j, i, nv);
    const double *A1 = A6, *A2 = A6 + pl, *A3 = A6 + 2 * pl, *A4 = A6 + 3 * pl;
    const double a0 = A1[p], a1 = A2[p], a2 = A3[p], a3 = A4[p], a4 = A4[p + 1],
                 a5 = A3[p + nv - 1], a6 = A2[p + nv], a7 = A1[p + nv + 1];
    const bool ok = msk[p] != 0 && a0 == a2 && a0 == a5 && a0 == a7 && a1 == a6 && a3 == a4;
    out[6 * n + 0] = a0;
    out[6 * n + 1] = a1;
    out[6 * n + 2] = a3;
    out[6 * n + 3] = A6[5 * pl + p];
    out[6 * n + 4] = A6[4 * pl + p];
    out[6 * n + 5] = ok ? 1. : 0.;
}

// uf = 1 where the point is fluid and its stored stencil is (c, ey, ex, c3,
// a5) exactly (rows and columns 1 .. m-2; 0 elsewhere)
__global__ void k_uniform_flags(const double *A6, const int8_t *msk, int mv, int nv, double c,
                                double ey, double ex, double c3, double a5, uint8_t *uf) {
    const size_t pl = (size_t)mv * nv;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < pl;
         p += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(p / nv), i = (int)(p % nv);
        uint8_t f = 0;
        if (j >= 1 && j <= mv - 2 && i >= 1 && i <= nv - 2 && msk[p] != 0) {
            const double *A1 = A6, *A2 = A6 + pl, *A3 = A6 + 2 * pl, *A4 = A6 + 3 * pl;
            f = A1[p] == c && A3[p] == c && A3[p + nv - 1] == c && A1[p + nv + 1] == c &&
                A2[p] == ey && A2[p + nv] == ey && A4[p] == ex && A4[p + 1] == ex &&
                A6[5 * pl + p] == c3 && A6[4 * pl + p] == a5;
        }
        uf[p] = f;
    }
}

int mg_stencil_samples(const LevelView<double> &L, double *out, cudaStream_t s) {
    k_stencil_samples<<<1, 32, 0, s>>>(L.A, L.msk, L.mv, L.nv, out);
    return launch_status("stencil samples");
}

// the level's uniform stencil st = (c, ey, ex, c3, a5): the form most of the
// 16 samples (host copy h of mg_stencil_samples' output) share; false unless
// at least half of them share it (a level whose coarsening rounds the
// stencil out of its symmetric form, or whose samples are mostly next to
// walls, has no uniform stencil, and the column form would take the general
// expression nearly everywhere)
bool mg_uniform_choose(const double *h, double *st) {
    int best = -1, best_n = 0;
    for (int a = 0; a < 16; a++) {
        if (h[6 * a + 5] == 0.) continue;
        int n = 0;
        for (int b = 0; b < 16; b++) {
            bool same = h[6 * b + 5] != 0.;
            for (int k = 0; k < 5; k++) same = same && h[6 * b + k] == h[6 * a + k];
            n += same;
        }
        if (n > best_n) {
            best_n = n;
            best = a;
        }
    }
    if (best < 0 || best_n < 8) return false;
    for (int k = 0; k < 5; k++) st[k] = h[6 * best + k];
    return true;
}

int mg_uniform_flags(const LevelView<double> &L, const double *st, uint8_t *uf, cudaStream_t s) {
    const size_t pl = (size_t)L.mv * L.nv;
    const size_t blocks = (pl + 255) / 256;
    k_uniform_flags<<<(unsigned)(blocks > 4096 ? 4096 : blocks), 256, 0, s>>>(
        L.A, L.msk, L.mv, L.nv, st[0], st[1], st[2], st[3], st[4], uf);
    return launch_status("uniform flags");
}

template <typename T>
F2D_DEV void smooth_l0_body(const SmoothFusedArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    extern __shared__ __align__(16) unsigned char sm[];
    T *xs = (T *)sm;                      // x on [j0-2, j0+33] x [i0-2, i0+33]
    T *ts = xs + SL_XW * SL_XW;           // first sweep on [j0-1, j0+32] x [i0-1, i0+32]
    T *bs = ts + SL_TW * SL_TW;           // b on the first sweep's points
    uint16_t *nbs = (uint16_t *)(bs + SL_TW * SL_TW);
    int8_t *ms = (int8_t *)(nbs + SL_TW * SL_TW);
    const LevelView<T> L = A.L;
    const AnalyticT<T> an = A.an;
    const T c2 = A.c2, c3z = A.c3z;  // c3 where the diagonal is 0
    const int xmode = A.xmode;
    const int mv = L.mv, nv = L.nv;
    const int i0 = NH + vb.x * SL_T, j0 = NH + vb.y * SL_T;
    const int tx = (int)threadIdx.x & (SL_T - 1), ty = (int)threadIdx.x >> 5;
    // the x ring (rows/cols 1..m-2), 32-bit offsets from (j0-2, i0-2)
    const size_t o2 = off(j0 - 2, i0 - 2, nv);
    // the rings are walked as flat index ranges (full warps; the constant
    // widths make the row/column split a multiply-shift)
    const int tid = (int)threadIdx.x;
    if (xmode == X_IN) {
        const T *xg = L.x + o2;
        for (int q = tid; q < SL_XW * SL_XW; q += SL_THREADS) {
            const int r = q / SL_XW, c = q - r * SL_XW;
            const int j = j0 - 2 + r, i = i0 - 2 + c;
            if (j < 1 || j > mv - 2 || i < 1 || i > nv - 2) continue;
            xs[q] = xg[r * nv + c];
        }
    } else if (xmode != X_ZERO) {
        // the prolongation by coarse cells: the fine points (2J-2+dj, 2I-2+di)
        // of cell (J, I) share its four coarse values and masks (one load of
        // each a cell instead of a point); the ring's rows/cols 1..m-2 only
        const T *xg = L.x + o2;
        const int ja = max(1, j0 - 2), jb = min(mv - 2, j0 + SL_XW - 3);
        const int ia = max(1, i0 - 2), ib = min(nv - 2, i0 + SL_XW - 3);
        const int Ja = (ja >> 1) + 1, Ia = (ia >> 1) + 1;
        const int ch = (jb >> 1) + 1 - Ja + 1, cw = (ib >> 1) + 1 - Ia + 1;
        const int nc2 = A.cs.nv;
        for (int q = tid; q < ch * cw; q += SL_THREADS) {
            const int cr = q / cw, J = Ja + cr, I = Ia + q - cr * cw;
            const size_t p2 = off(J, I, nc2);
            const int k00 = A.cs.msk[p2], k01 = A.cs.msk[p2 + 1], k10 = A.cs.msk[p2 + nc2],
                      k11 = A.cs.msk[p2 + nc2 + 1];
            const T x00 = A.cs.x[p2], x01 = A.cs.x[p2 + 1], x10 = A.cs.x[p2 + nc2],
                    x11 = A.cs.x[p2 + nc2 + 1];
#pragma unroll
            for (int dj = 0; dj < 2; dj++) {
                const int j = 2 * J - 2 + dj;
                if (j < ja || j > jb) continue;
#pragma unroll
                for (int di = 0; di < 2; di++) {
                    const int i = 2 * I - 2 + di;
                    if (i < ia || i > ib) continue;
                    const int r = j - (j0 - 2), c = i - (i0 - 2);
                    const T cv = interp_combine<T>(L.msk[off(j, i, nv)], dj, di, k00, k01, k10,
                                                   k11, x00, x01, x10, x11);
                    xs[r * SL_XW + c] = xmode == X_PLUS_INTERP ? xg[r * nv + c] + cv : cv;
                }
            }
        }
    }
    // bits, mask and b of the first sweep's points (rows/cols 2..m-3)
    int mine = 1;  // every point this thread staged has its 3x3 block fluid
    {
        const size_t o1 = off(j0 - 1, i0 - 1, nv);
        const uint16_t *nbg = L.nb + o1;
        const int8_t *mg = L.msk + o1;
        const T *bg = L.b + o1;
        for (int q = tid; q < SL_TW * SL_TW; q += SL_THREADS) {
            const int r = q / SL_TW, c = q - r * SL_TW;
            const int j = j0 - 1 + r, i = i0 - 1 + c;
            if (j < 2 || j > mv - 3 || i < 2 || i > nv - 3) continue;
            const int o = r * nv + c;
            const uint16_t bits = nbg[o];
            nbs[q] = bits;
            ms[q] = mg[o];
            bs[q] = bg[o];
            mine &= bits == 511u;
        }
    }
#ifdef F2D_EXACT
    __syncthreads();
    const bool uni = false;
#else
    // A tile whose first-sweep points all have fluid 3x3 blocks takes the
    // separable form of the 9-point operator (product build): (c/4)(V - 4x)
    // with V the [1 2 1] x [1 2 1] sum, so a sweep is k0 x + k1 V - c3 b
    // (k1 = c3 c/4, k0 = c2 - 4 k1): no coefficient selects, 8 operations
    // for the operator instead of 8 products and 16 selects.  The same
    // function, another rounding; the exact build keeps jacobi_bits().
    const T e = an.sc[1];
    const bool nine = e != (T)0 && an.sc[3] == e && an.sc[0] == (T)0.5 * e && an.sc[2] == an.sc[0];
    const bool uni = __syncthreads_and(mine && nine) != 0;
    const T k1 = an.c3 * e * (T)0.5, k0 = c2 - (T)4 * k1;
#endif
    // first sweep
    for (int q = tid; q < SL_TW * SL_TW; q += SL_THREADS) {
        const int r = q / SL_TW, c = q - r * SL_TW;
        const int j = j0 - 1 + r, i = i0 - 1 + c;
        if (j < 2 || j > mv - 3 || i < 2 || i > nv - 3) continue;
        T v;
        if (ms[q] == 0) {
            v = (T)0;
        } else if (xmode == X_ZERO) {
            v = ((nbs[q] & 256u) ? an.c3 : c3z) * (-bs[q]);
        } else {
            const T *x = xs + (r + 1) * SL_XW + (c + 1);
#ifndef F2D_EXACT
            if (uni)
                v = separable9<T>(x, SL_XW, bs[q], an.c3, k0, k1);
            else
#endif
                v = jacobi_bits<T>(nbs[q], x, SL_XW, bs[q], an, c2, c3z);
        }
        ts[q] = v;
    }
    __syncthreads();
    // second sweep: the tile, each thread rows ty, ty+8, ty+16, ty+24 of column tx
    const int m2 = mv - 2 * NH, n2 = nv - 2 * NH;
    const bool direct = j0 >= 2 * NH && j0 + SL_T <= m2 && i0 >= 2 * NH && i0 + SL_T <= n2;
    T *out = A.out;
    const int i = i0 + tx;
    if (i > nv - NH - 1) return;
    for (int r = ty; r < SL_T; r += SL_TY) {
        const int j = j0 + r;
        if (j > mv - NH - 1) break;
        const int q = (r + 1) * SL_TW + (tx + 1);
        T v = (T)0;
        if (ms[q] != 0)
#ifndef F2D_EXACT
            if (uni)
                v = separable9<T>(ts + q, SL_TW, bs[q], an.c3, k0, k1);
            else
#endif
                v = jacobi_bits<T>(nbs[q], ts + q, SL_TW, bs[q], an, c2, c3z);
        if (direct)
            out[off(j, i, nv)] = v;
        else
            store_images(out, j, i, mv, nv, v);
    }
}

template <typename T>
__global__ void __launch_bounds__(SL_THREADS) k_smooth_l0(SmoothFusedArgs<T> a) {
    pdl_prologue();
    smooth_l0_body<T>(a, F2D_VB_NATIVE);
}

template <typename T>
struct BSmoothL0 {
    using Args = SmoothFusedArgs<T>;
    static constexpr int THREADS = SL_THREADS;
    static constexpr int MIN_BLOCKS = 5;
    static constexpr int KIND = sizeof(T) == 4 ? BK_SmoothFusedF1 : -1;
    F2D_DEV static void run(const Args &a, VB vb) { smooth_l0_body<T>(a, vb); }
};
using BSmoothL0F = BSmoothL0<float>;
F2D_BATCH_ENTRY(SmoothFusedF1, BSmoothL0F)

template <typename T>
int mg_smooth_fused(const LevelView<T> &L, const AnalyticT<T> *an, T c1, T c2, int xmode,
                    const LevelView<T> *coarse, T *out, const int *active, cudaStream_t s) {
    if (an && L.nb && sizeof(T) == 4) {  // the float finest level
        CoarseSrc<T> cs{nullptr, nullptr, 0};
        if (coarse) cs = CoarseSrc<T>{coarse->msk, coarse->x, coarse->nv};
        SmoothFusedArgs<T> a{L, *an, c1, c2, xmode, cs, out, active, SL_T, SL_T, c3_zero(c1)};
        const dim3 g = grid2d(L.mv - 2 * NH, L.nv - 2 * NH, dim3(SL_T, SL_T));
        return launch_body<BSmoothL0<T>>(k_smooth_l0<T>, a, g, dim3(SL_THREADS),
                                         smooth_l0_smem<T>(), s, "mg_smooth_l0");
    }
    const dim3 tile = level_tile(L.mv - 2 * NH, L.nv - 2 * NH, FS_TX, FS_TY);
    const dim3 g = grid2d(L.mv - 2 * NH, L.nv - 2 * NH, tile);
    const dim3 b(smooth_fused_threads(tile, g));
    const size_t smem = smooth_fused_smem<T>(tile);
    CoarseSrc<T> cs{nullptr, nullptr, 0};
    if (coarse) cs = CoarseSrc<T>{coarse->msk, coarse->x, coarse->nv};
    SmoothFusedArgs<T> a{L,   an ? *an : AnalyticT<T>{}, c1, c2, xmode, cs, out, active,
                         (int)tile.x, (int)tile.y, c3_zero(c1)};
    if (an)
        return launch_body<BSmoothFused<T, true>>(k_smooth_fused<T, true>, a, g, b, smem, s,
                                                  "mg_smooth_fused");
    return launch_body<BSmoothFused<T, false>>(k_smooth_fused<T, false>, a, g, b, smem, s,
                                               "mg_smooth_fused");
}

// residual + full-weighting restriction: the fine residuals a coarse tile
// needs (fine halo positions through their periodic images, as the
// reference's halo fill of r makes them) are computed once into shared
// memory, then restricted.  The CTA has one thread per fine residual of its
// region ((2ty+1) x (2tx+1) for a coarse tile tx x ty, rounded up to whole
// warps): each thread waits for its loads once, and its float64 chain is one
// residual plus at most one restriction.
constexpr int RR_TX = 16, RR_TY = 8;
constexpr int RR_THREADS = ((2 * RR_TX + 1) * (2 * RR_TY + 1) + 31) / 32 * 32;
constexpr int RR_MIN_BLOCKS = 2;  // at most 56 registers: two CTAs of 576 per SM

static inline unsigned resres_threads(dim3 tile) {
    return ((2 * tile.x + 1) * (2 * tile.y + 1) + 31) / 32 * 32;
}

template <typename T>
size_t resres_smem(dim3 tile) {
    return sizeof(T) * (size_t)(2 * tile.y + 1) * (2 * tile.x + 1);
}

template <typename T>
struct ResresArgs {
    LevelView<T> F;
    AnalyticT<T> an;
    const int8_t *msk2;
    int mv2, nv2;
    T *b2;
    const int *active;
    int tx, ty;  // the coarse tile
    // a stored level's uniform stencil (product build; uf null: none): the
    // flagged points' residual b - (c corners + ey vertical + ex horizontal
    // + a5 x), without the coefficient loads
    const uint8_t *uf;
    T uc, uey, uex, ua5;
};

template <typename T, bool L0>
F2D_DEV void resres_body(const ResresArgs<T> &A, const VB vb) {
    if (inactive(A.active)) return;
    const int TX = A.tx, TY = A.ty, NT = (int)blockDim.x;
    const int RW = 2 * TX + 1, RH = 2 * TY + 1;
    extern __shared__ __align__(16) unsigned char sm[];
    T *rs = (T *)sm;
    const LevelView<T> F = A.F;
    const AnalyticT<T> an = A.an;
    const int8_t *msk2 = A.msk2;
    const int mv2 = A.mv2, nv2 = A.nv2;
    T *b2 = A.b2;
    const int I2a = NH + vb.x * TX, J2a = NH + vb.y * TY;
    const int jf0 = 2 * J2a - 3, if0 = 2 * I2a - 3;
    const int tid = (int)threadIdx.x;
    const int mv = F.mv, nv = F.nv;
    const float inv = 1.0f / (float)RW;
#ifndef F2D_EXACT
    // the analytic finest level (product build): a warp whose points all
    // have fluid 3x3 blocks takes the separable form of the 9-point operator,
    // r = b + kv V + kx x (kv = -e/2, kx = 2e - a5 for edges e and corners
    // e/2), without the coefficient selects
    const T e = an.sc[1];
    const bool nine = L0 && F.nb && e != (T)0 && an.sc[3] == e && an.sc[0] == (T)0.5 * e &&
                      an.sc[2] == an.sc[0];
    const T kv = -an.sc[0], kx = (T)4 * an.sc[0] - an.a5;
#endif
    for (int q = tid; q < RH * RW; q += NT) {
        const int qj = small_div(q, inv);
        const int jf = jf0 + qj, iff = if0 + (q - qj * RW);
        const bool in = jf <= mv - 3 && iff <= nv - 3;  // within the last coarse point's stencil
#ifndef F2D_EXACT
        if (nine) {
            const int jw = in ? wrap(jf, mv, NH) : NH, iw = in ? wrap(iff, nv, NH) : NH;
            const size_t p = off(jw, iw, nv);
            const bool full = !in || F.nb[p] == 511u;
            if (__all_sync(__activemask(), full)) {
                if (in) {
                    const T *x = F.x + p;
                    const T corners = (x[-nv - 1] + x[-nv + 1]) + (x[nv - 1] + x[nv + 1]);
                    const T edges = (x[-nv] + x[nv]) + (x[-1] + x[1]);
                    const T V = fma((T)4, x[0], fma((T)2, edges, corners));
                    rs[q] = fma(kv, V, fma(kx, x[0], F.b[p]));
                }
                continue;
            }
        }
#endif
        if (!in) continue;
        const int jw = wrap(jf, mv, NH), iw = wrap(iff, nv, NH);
        if (!L0 && A.uf) {
            const size_t p = off(jw, iw, nv);
            if (A.uf[p]) {
                const T *x = F.x + p;
                const T corners = (x[-nv - 1] + x[-nv + 1]) + (x[nv - 1] + x[nv + 1]);
                const T vert = x[-nv] + x[nv], horiz = x[-1] + x[1];
                rs[q] = F.b[p] - fma(A.uc, corners, fma(A.uey, vert, fma(A.uex, horiz, A.ua5 * x[0])));
                continue;
            }
        }
        rs[q] = residual<T, L0>(F, &an, F.x, F.b, jw, iw);
    }
    __syncthreads();
    const float invt = 1.0f / (float)TX;
    for (int c = tid; c < TX * TY; c += NT) {
        const int cj = small_div(c, invt);
        const int J2 = J2a + cj, I2 = I2a + (c - cj * TX);
        if (J2 > mv2 - NH - 1 || I2 > nv2 - NH - 1) continue;
        T v = (T)0;
        if (msk2[off(J2, I2, nv2)] != 0) {
            const T *r = rs + (2 * J2 - 2 - jf0) * RW + (2 * I2 - 2 - if0);
            v = (T)0.25 * r[0]
                + (T)0.125 * (r[-1] + r[1] + r[-RW] + r[RW])
                + (T)0.0625 * (r[-RW - 1] + r[-RW + 1] + r[RW - 1] + r[RW + 1]);
        }
        store_images(b2, J2, I2, mv2, nv2, v);
    }
}

template <typename T, bool L0>
__global__ void __launch_bounds__(RR_THREADS, RR_MIN_BLOCKS) k_resres(ResresArgs<T> a) {
    pdl_prologue();
    resres_body<T, L0>(a, F2D_VB_NATIVE);
}

template <typename T, bool L0>
struct BResres {
    using Args = ResresArgs<T>;
    static constexpr int THREADS = RR_THREADS;
    static constexpr int MIN_BLOCKS = RR_MIN_BLOCKS;
    static constexpr int KIND = sizeof(T) == 8 ? (L0 ? -1 : BK_ResresD0)
                                               : (L0 ? BK_ResresF1 : BK_ResresF0);
    F2D_DEV static void run(const Args &a, VB vb) { resres_body<T, L0>(a, vb); }
};
using BResresD0 = BResres<double, false>;
using BResresF0 = BResres<float, false>;
using BResresF1 = BResres<float, true>;
F2D_BATCH_ENTRY(ResresD0, BResresD0)
F2D_BATCH_ENTRY(ResresF0, BResresF0)
F2D_BATCH_ENTRY(ResresF1, BResresF1)

template <typename T>
int mg_resres(const LevelView<T> &F, const AnalyticT<T> *an, const LevelView<T> &C, T *b2,
              const int *active, cudaStream_t s, const uint8_t *uf, const T *ust) {
    const dim3 tile = level_tile(C.mv - 2 * NH, C.nv - 2 * NH, RR_TX, RR_TY);
    const dim3 g = grid2d(C.mv - 2 * NH, C.nv - 2 * NH, tile);
    const dim3 b(resres_threads(tile));
    const size_t smem = resres_smem<T>(tile);
    ResresArgs<T> a{F,  an ? *an : AnalyticT<T>{}, C.msk, C.mv, C.nv, b2, active,
                    (int)tile.x, (int)tile.y, nullptr, (T)0, (T)0, (T)0, (T)0};
    // float64 levels of at least one CTA per SM (measured: 1024^2 step -1.4 %;
    // on the small levels of a 128^2 hierarchy the flag's extra load made the
    // step 5 % slower, and the float levels of the mixed form gained nothing)
    if (uf && ust && !an && sizeof(T) == 8 && column_applies(F)) {
        a.uf = uf;
        a.uc = ust[0];
        a.uey = ust[1];
        a.uex = ust[2];
        a.ua5 = ust[4];
    }
    if (an)
        return launch_body<BResres<T, true>>(k_resres<T, true>, a, g, b, smem, s, "mg_resres");
    return launch_body<BResres<T, false>>(k_resres<T, false>, a, g, b, smem, s, "mg_resres");
}

// ------------------------------------------------------------ coarse CTA
// All levels below a size threshold are processed by one CTA out of shared
// memory: the recursion of core/gmg/hierarchy.py:98-151 runs as a sequence
// of block-wide phases separated by __syncthreads().  Each level's arrays
// are addressed from a descriptor table in shared memory, so every access
// compiles to a shared-memory access; threads cover a level in 32 x 32
// blocks of (row, column).
constexpr int CO_TX = 32, CO_TY = 32;
constexpr int COARSE_SMEM_MAX = 220 * 1024;
constexpr int CO_THREADS = CO_TX * CO_TY;

F2D_HD size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

template <typename T>
size_t coarse_smem_bytes(const int *mv, const int *nv, int nlev) {
    size_t tot = 0;
    for (int l = 0; l < nlev; l++) {
        size_t pts = (size_t)mv[l] * nv[l];
        tot += align16(pts) + align16(sizeof(T) * pts * 10);  // msk, A(6), x, b, r, t
    }
    return tot;
}

struct CoLv {
    int mv, nv;
    unsigned o_msk, o_A, o_x, o_b, o_r, o_t;
};

template <typename T>
F2D_DEV LevelView<T> co_view(unsigned char *sm, const CoLv &d) {
    LevelView<T> L;
    L.mv = d.mv;
    L.nv = d.nv;
    L.msk = (const int8_t *)(sm + d.o_msk);
    L.A = (const T *)(sm + d.o_A);
    L.x = (T *)(sm + d.o_x);
    L.b = (T *)(sm + d.o_b);
    L.r = (T *)(sm + d.o_r);
    L.t = (T *)(sm + d.o_t);
    L.nb = nullptr;
    return L;
}

// Phases on small levels (at most CO_SMALL_PTS points, halo included) run on
// the first CO_GROUP threads only -- one warp per SM sub-partition, so that
// float64 work still reaches every FP64 unit -- and synchronise with a named
// barrier; the other warps skip them.  A block-wide barrier is placed only
// where a large-level phase follows small-level ones.
constexpr int CO_GROUP = 128;
constexpr int CO_SMALL_PTS = 256;

struct CoSched {
    bool prev_small;
};

// enter a phase on a level of `pts` points: returns whether this thread works
F2D_DEV bool co_enter(CoSched &sc, int pts, int &nthreads) {
    const bool small = pts <= CO_SMALL_PTS;
    if (!small && sc.prev_small) __syncthreads();
    sc.prev_small = small;
    nthreads = small ? CO_GROUP : CO_THREADS;
    const int tid = threadIdx.y * CO_TX + threadIdx.x;
    return tid < nthreads;
}

F2D_DEV void co_leave(int nthreads) {
    if (nthreads == CO_THREADS)
        __syncthreads();
    else
        asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// rows [j0, j1] x cols [i0, i1] strided over the phase's threads
#define CO_FOR(j0, j1, i0, i1, nthreads)                                               \
    for (int _q = threadIdx.y * CO_TX + threadIdx.x,                                   \
             _w = (i1) - (i0) + 1, _n = _w * ((j1) - (j0) + 1);                        \
         _q < _n; _q += (nthreads))                                                    \
        for (int j = (j0) + _q / _w, i = (i0) + _q % _w, _once = 1; _once; _once = 0)

template <typename T>
F2D_DEV void co_smooth(unsigned char *sm, const CoLv &d, T c1, T c2, bool zero_x, CoSched &sc) {
    const LevelView<T> L = co_view<T>(sm, d);
    int nt;
    if (co_enter(sc, L.mv * L.nv, nt)) {
        CO_FOR(2, L.mv - 3, 2, L.nv - 3, nt)
        L.t[off(j, i, L.nv)] = jacobi<T, false>(L, nullptr, zero_x ? nullptr : L.x, L.b, j, i,
                                                c1, c2);  // stored level: c3 from its A plane
        co_leave(nt);
        CO_FOR(NH, L.mv - NH - 1, NH, L.nv - NH - 1, nt)
        store_images(L.x, j, i, L.mv, L.nv, jacobi<T, false>(L, nullptr, L.t, L.b, j, i, c1, c2));
        co_leave(nt);
    }
}

template <typename T>
F2D_DEV void co_residual(unsigned char *sm, const CoLv &d, CoSched &sc) {
    const LevelView<T> L = co_view<T>(sm, d);
    int nt;
    if (co_enter(sc, L.mv * L.nv, nt)) {
        CO_FOR(NH, L.mv - NH - 1, NH, L.nv - NH - 1, nt)
        store_images(L.r, j, i, L.mv, L.nv, residual<T, false>(L, nullptr, L.x, L.b, j, i));
        co_leave(nt);
    }
}

template <typename T>
F2D_DEV void co_restrict(unsigned char *sm, const CoLv &df, bool from_b, const CoLv &dc,
                         CoSched &sc) {
    const LevelView<T> F = co_view<T>(sm, df), Cl = co_view<T>(sm, dc);
    const T *src = from_b ? F.b : F.r;
    int nt;
    if (co_enter(sc, F.mv * F.nv, nt)) {
        CO_FOR(NH, Cl.mv - NH - 1, NH, Cl.nv - NH - 1, nt)
        store_images(Cl.b, j, i, Cl.mv, Cl.nv, restrict_value(Cl.msk, Cl.nv, src, F.nv, j, i));
        co_leave(nt);
    }
}

template <typename T>
F2D_DEV void co_interp(unsigned char *sm, const CoLv &dc, const CoLv &df, bool assign,
                       CoSched &sc) {
    const LevelView<T> Cl = co_view<T>(sm, dc), F = co_view<T>(sm, df);
    int nt;
    if (co_enter(sc, F.mv * F.nv, nt)) {
        CO_FOR(1, F.mv - 2, 1, F.nv - 2, nt) {
            T v = interp_value(F.msk, F.nv, Cl.msk, Cl.x, Cl.nv, j, i);
            size_t p = off(j, i, F.nv);
            F.x[p] = assign ? v : F.x[p] + v;
        }
        co_leave(nt);
    }
}

template <typename T>
F2D_DEV void co_vcycle(unsigned char *sm, const CoLv *lv, int l1, int deep, bool zero_first,
                       T c1, T c2, int ndeepest, CoSched &sc) {
    for (int l = l1; l < deep; l++) {
        co_smooth<T>(sm, lv[l], c1, c2, zero_first || l > l1, sc);
        co_residual<T>(sm, lv[l], sc);
        co_restrict<T>(sm, lv[l], false, lv[l + 1], sc);
    }
    for (int k = 0; k < ndeepest; k++) co_smooth<T>(sm, lv[deep], c1, c2, k == 0, sc);
    for (int l = deep - 1; l >= l1; l--) {
        co_interp<T>(sm, lv[l + 1], lv[l], false, sc);
        co_smooth<T>(sm, lv[l], c1, c2, false, sc);
    }
}

// shared-memory layout of the levels (thread 0 writes the table)
template <typename T>
F2D_DEV void coarse_layout(const CoarseArgs<T> &a, CoLv *lv) {
    unsigned o = 0;
    for (int l = 0; l < a.nlev; l++) {
        const unsigned pts = (unsigned)(a.lev[l].mv * a.lev[l].nv);
        CoLv d;
        d.mv = a.lev[l].mv;
        d.nv = a.lev[l].nv;
        d.o_msk = o;
        o += (unsigned)align16(pts);
        d.o_A = o;
        d.o_x = o + 6 * pts * sizeof(T);
        d.o_b = o + 7 * pts * sizeof(T);
        d.o_r = o + 8 * pts * sizeof(T);
        d.o_t = o + 9 * pts * sizeof(T);
        o += (unsigned)align16(sizeof(T) * pts * 10);
        lv[l] = d;
    }
}

// masks and operators of every level into shared memory; the first level's
// b and x from the arrays (unit < 0), or b = the unit vector of interior
// point `unit` (with its periodic images) and x = 0
template <typename T>
F2D_DEV void coarse_load(const CoarseArgs<T> &a, const CoLv *lv, unsigned char *sm, int unit) {
    const int tid = threadIdx.y * CO_TX + threadIdx.x;
    for (int l = 0; l < a.nlev; l++) {
        const LevelView<T> &g = a.lev[l];
        const LevelView<T> s = co_view<T>(sm, lv[l]);
        const int pts = g.mv * g.nv;
        for (int q = tid; q < pts; q += CO_THREADS) ((int8_t *)s.msk)[q] = g.msk[q];
        for (int q = tid; q < 6 * pts; q += CO_THREADS) ((T *)s.A)[q] = g.A[q];
        if (l == 0)
            for (int q = tid; q < pts; q += CO_THREADS) {
                s.b[q] = unit < 0 ? g.b[q] : (T)0;
                s.x[q] = (unit < 0 && a.mode == CYCLE_V && !a.zero_first) ? g.x[q] : (T)0;
            }
    }
    if (unit >= 0) {
        __syncthreads();
        if (tid == 0) {
            const LevelView<T> s = co_view<T>(sm, lv[0]);
            const int n2 = s.nv - 2 * NH;
            store_images(s.b, NH + unit / n2, NH + unit % n2, s.mv, s.nv, (T)1);
        }
    }
}

// core/gmg/hierarchy.py:98-151 on the levels in shared memory
template <typename T>
F2D_DEV void coarse_cycle(const CoarseArgs<T> &a, const CoLv *lv, unsigned char *sm) {
    const int deep = a.nlev - 1;
    CoSched sc{false};
    if (a.mode == CYCLE_V) {
        co_vcycle<T>(sm, lv, 0, deep, a.zero_first != 0, a.c1, a.c2, a.ndeepest, sc);
    } else {
        for (int l = 0; l < deep; l++) co_restrict<T>(sm, lv[l], true, lv[l + 1], sc);
        for (int k = 0; k < a.ndeepest; k++) co_smooth<T>(sm, lv[deep], a.c1, a.c2, k == 0, sc);
        for (int l = deep - 1; l >= 0; l--) {
            co_interp<T>(sm, lv[l + 1], lv[l], true, sc);
            co_vcycle<T>(sm, lv, l, deep, false, a.c1, a.c2, a.ndeepest, sc);
        }
    }
}

template <typename T>
F2D_DEV void coarse_body(const CoarseArgs<T> &a, const VB) {
    if (inactive(a.active)) return;
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ CoLv lv[MAX_LEVELS];
    const int tid = threadIdx.y * CO_TX + threadIdx.x;
    if (tid == 0) coarse_layout(a, lv);
    __syncthreads();
    coarse_load(a, lv, sm, -1);
    __syncthreads();
    coarse_cycle(a, lv, sm);
    __syncthreads();
    const LevelView<T> s0 = co_view<T>(sm, lv[0]);
    const int pts0 = a.lev[0].mv * a.lev[0].nv;
    for (int q = tid; q < pts0; q += CO_THREADS) a.lev[0].x[q] = s0.x[q];
}

// The coarse part of a cycle started from x = 0 (a V-cycle with zero_first,
// or the F-cycle) is a fixed linear map of the first level's right-hand
// side.  CTA k runs it on the unit vector of interior point k and writes the
// resulting interior values into column k of op (row-major, n x n).
template <typename T>
__global__ void __launch_bounds__(CO_THREADS) k_coarse_columns(CoarseArgs<T> a, T *op, int n) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ CoLv lv[MAX_LEVELS];
    const int tid = threadIdx.y * CO_TX + threadIdx.x;
    const int k = (int)blockIdx.x;
    if (k >= n) return;
    if (tid == 0) coarse_layout(a, lv);
    __syncthreads();
    coarse_load(a, lv, sm, k);
    __syncthreads();
    coarse_cycle(a, lv, sm);
    __syncthreads();
    const LevelView<T> s0 = co_view<T>(sm, lv[0]);
    const int n2 = s0.nv - 2 * NH;
    for (int i = tid; i < n; i += CO_THREADS)
        op[(size_t)i * n + k] = s0.x[off(NH + i / n2, NH + i % n2, s0.nv)];
}

template <typename T>
__global__ void __launch_bounds__(CO_THREADS) k_coarse(CoarseArgs<T> a) {
    pdl_prologue();
    coarse_body<T>(a, F2D_VB_NATIVE);
}

template <typename T>
struct BCoarse {
    using Args = CoarseArgs<T>;
    static constexpr int THREADS = CO_THREADS;
    static constexpr int KIND = sizeof(T) == 8 ? BK_CoarseD : BK_CoarseF;
    F2D_DEV static void run(const Args &a, VB vb) { coarse_body<T>(a, vb); }
};
using BCoarseD = BCoarse<double>;
using BCoarseF = BCoarse<float>;
F2D_BATCH_ENTRY(CoarseD, BCoarseD)
F2D_BATCH_ENTRY(CoarseF, BCoarseF)

// the batched coarse kernels need the same opt-in shared memory
int configure_batched_coarse() {
    int st = cuda_status(cudaFuncSetAttribute(k_batch<BCoarseD>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              COARSE_SMEM_MAX),
                         "batched coarse smem");
    if (st) return st;
    return cuda_status(cudaFuncSetAttribute(k_batch<BCoarseF>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            COARSE_SMEM_MAX),
                       "batched coarse smem");
}

namespace {
// per library and device: the opt-in shared-memory size of k_coarse
bool g_coarse_configured[2][64];
}

template <typename T>
int mg_coarse(const CoarseArgs<T> &args, size_t smem, cudaStream_t s) {
    int idx = sizeof(T) == 8 ? 0 : 1, dev = 0;
    int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    if (dev < 0 || dev >= 64 || !g_coarse_configured[idx][dev]) {
        // 227 KB per CTA minus the kernel's static shared memory (the level table)
        st = cuda_status(cudaFuncSetAttribute(k_coarse<T>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              COARSE_SMEM_MAX),
                         "coarse smem attribute");
        if (st) return st;
        if (dev >= 0 && dev < 64) g_coarse_configured[idx][dev] = true;
    }
    return launch_body<BCoarse<T>>(k_coarse<T>, args, dim3(1), dim3(CO_TX, CO_TY), smem, s,
                                   "mg_coarse");
}

// The coarse part applied as its linear map: x(interior i) = sum_k op[i][k]
// b(interior k), written with its periodic images (every halo point of the
// first level is the image of an interior point, as the cycle leaves it).
// One warp per interior point; the first level's interior b is staged in
// shared memory.  The same function as the cycle on the levels, summed in a
// different order: used by the product build only.
constexpr int CA_WARPS = 8;

template <typename T>
struct CoarseApplyArgs {
    const T *op;
    int n, n2, mv, nv;
    const T *b;
    T *x;
    const int *active;
};

template <typename T>
F2D_DEV void coarse_apply_body(const CoarseApplyArgs<T> &a, const VB vb) {
    if (inactive(a.active)) return;
    extern __shared__ __align__(16) unsigned char sm[];
    T *bs = (T *)sm;
    const int tid = (int)threadIdx.x, n = a.n, n2 = a.n2;
    for (int k = tid; k < n; k += CA_WARPS * 32) {
        const int qj = k / n2;
        bs[k] = a.b[off(NH + qj, NH + (k - qj * n2), a.nv)];
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const int i = vb.x * CA_WARPS + warp;
    if (i >= n) return;
    const T *row = a.op + (size_t)i * n;
    T s0 = (T)0, s1 = (T)0;
    int k = lane;
    for (; k + 32 < n; k += 64) {
        s0 = fma(row[k], bs[k], s0);
        s1 = fma(row[k + 32], bs[k + 32], s1);
    }
    if (k < n) s0 = fma(row[k], bs[k], s0);
    T v = s0 + s1;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) {
        const int qj = i / n2;
        store_images(a.x, NH + qj, NH + (i - qj * n2), a.mv, a.nv, v);
    }
}

template <typename T>
__global__ void __launch_bounds__(CA_WARPS * 32) k_coarse_apply(CoarseApplyArgs<T> a) {
    pdl_prologue();
    coarse_apply_body<T>(a, F2D_VB_NATIVE);
}

template <typename T>
struct BCoarseApply {
    using Args = CoarseApplyArgs<T>;
    static constexpr int THREADS = CA_WARPS * 32;
    static constexpr int KIND = sizeof(T) == 8 ? BK_CoarseApplyD : BK_CoarseApplyF;
    F2D_DEV static void run(const Args &a, VB vb) { coarse_apply_body<T>(a, vb); }
};
using BCoarseApplyD = BCoarseApply<double>;
using BCoarseApplyF = BCoarseApply<float>;
F2D_BATCH_ENTRY(CoarseApplyD, BCoarseApplyD)
F2D_BATCH_ENTRY(CoarseApplyF, BCoarseApplyF)

template <typename T>
int mg_coarse_columns(const CoarseArgs<T> &args, size_t smem, T *op, int n, cudaStream_t s) {
    int st = cuda_status(cudaFuncSetAttribute(k_coarse_columns<T>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              COARSE_SMEM_MAX),
                         "coarse columns smem attribute");
    if (st) return st;
    k_coarse_columns<T><<<n, dim3(CO_TX, CO_TY), smem, s>>>(args, op, n);
    return launch_status("mg_coarse_columns");
}

template <typename T>
int mg_coarse_apply(const T *op, int n, const LevelView<T> &L, const int *active,
                    cudaStream_t s) {
    CoarseApplyArgs<T> a{op, n, L.nv - 2 * NH, L.mv, L.nv, L.b, L.x, active};
    const dim3 g((unsigned)((n + CA_WARPS - 1) / CA_WARPS)), b(CA_WARPS * 32);
    return launch_body<BCoarseApply<T>>(k_coarse_apply<T>, a, g, b, sizeof(T) * (size_t)n, s,
                                        "mg_coarse_apply");
}

// ------------------------------------------------------------ stage kernels
// dt6 = dt/6, divided once a CTA (a float64 division costs a point's worth
// of FMAs, and a warp pays it whatever its active lanes)
F2D_DEV double rk_combine(int rk, double base, double d0, double d1, double dq, double dt,
                          double dt6) {
    if (rk == 1) return base + dt * dq;                                  // x + dt*dx0
    if (rk == 2) return base + (0.25 * dt) * (d0 + dq);                  // x + (dt/4)(dx0+dx1)
    return base + dt6 * (d0 + d1 + 4 * dq);                              // x + (dt/6)(...)
}

// Advection of one tracer with the halo fill, the Boussinesq torque and the
// RK combination fused (core/operators.py:214-236,303-314,
// core/timescheme.py:167-180).  TC is the type the fluxes are computed in
// (double, or float in the mixed form); loads, tendency and RK combination
// stay float64.
template <typename TC>
F2D_DEV void stage_adv_body(const AdvStage &a, const VB vb) {
    __shared__ TC sfx[8][33];
    __shared__ TC sfy[9][32];
    __shared__ double sdt6;
    const int tx = threadIdx.x, ty = threadIdx.y;
    if (tx == 0 && ty == 0 && a.rk == 3) sdt6 = *a.dt / 6.;
    const int nv = a.nv, mv = a.mv;
    const int I = NH + vb.x * 32 + tx;
    const int J = NH + vb.y * 8 + ty;
    const bool in = (I <= nv - NH - 1) && (J <= mv - NH - 1);
    const SplitT<TC> c = split_cast<TC>(*(const SplitConst *)a.advc);
    if (in) {
        const size_t p = off(J, I, nv);
        sfx[ty][tx + 1] = edge_flux_rt_t<TC>(a.kind, a.msk, a.q, a.u, p, 1, a.method, a.order, c);
        sfy[ty + 1][tx] = edge_flux_rt_t<TC>(a.kind, a.msk, a.q, a.v, p, nv, a.method, a.order, c);
        // the tile's south faces: warp 0, one face per lane
        if (ty == 0)
            sfy[0][tx] = edge_flux_rt_t<TC>(a.kind, a.msk, a.q, a.v, p - nv, nv, a.method, a.order, c);
    }
    // the tile's west faces: lanes 0-7 of warp 1, one row each (a warp
    // issues a float64 instruction for all its lanes, so one warp per ring
    // instead of lane 0 of every row's warp)
    if (ty == 1 && tx < 8) {
        const int Jr = NH + vb.y * 8 + tx, I0 = NH + vb.x * 32;
        if (I0 <= nv - NH - 1 && Jr <= mv - NH - 1)
            sfx[tx][0] = edge_flux_rt_t<TC>(a.kind, a.msk, a.q, a.u, off(Jr, I0, nv) - 1, 1,
                                            a.method, a.order, c);
    }
    __syncthreads();
    if (!in) return;
    const size_t p = off(J, I, nv);
    TC yc = -(c.zdx * (sfx[ty][tx + 1] - sfx[ty][tx])) - c.zdy * (sfy[ty + 1][tx] - sfy[ty][tx]);
    double y = (double)yc;
    if (a.buoy) {
        const int mc = a.msk[p];
        y = y * (double)mc;
        const int sl = mc + a.msk[p - 1], sr = a.msk[p + 1] + mc;
        const int ml = sl > 1 ? sl : 1, mr = sr > 1 ? sr : 1;
        if (ml + mr == 4) y = y + (a.buoy[p + 1] - a.buoy[p - 1]) * a.torque_coef * (double)mc;
    }
    if (a.diff_coef != 0. && a.msk[p] == 1) {  // add_diffusion, Fortran term order
        const double t = a.q[p];
        const double lap = (double)a.msk[p - 1] * (a.q[p - 1] - t) +
                           (double)a.msk[p + 1] * (a.q[p + 1] - t) +
                           (double)a.msk[p - nv] * (a.q[p - nv] - t) +
                           (double)a.msk[p + nv] * (a.q[p + nv] - t);
        y = y + a.diff_coef * lap;
    }
    const double dt = a.rk ? *a.dt : 0., dt6 = a.rk == 3 ? sdt6 : 0.;
    // the point and its periodic halo images (store_images' positions)
    auto put = [&](size_t q) {
        a.dq[q] = y;
        if (a.rk)
            a.out[q] = rk_combine(a.rk, a.base[q], a.d0 ? a.d0[q] : 0., a.d1 ? a.d1[q] : 0., y, dt,
                                  dt6);
    };
    for_images(J, I, mv, nv, put);
}

template <typename TC>
__global__ void __launch_bounds__(256) k_stage_adv(AdvStage a) {
    pdl_prologue();
    stage_adv_body<TC>(a, F2D_VB_NATIVE);
}

template <typename TC>
struct BStageAdv {
    using Args = AdvStage;
    static constexpr int THREADS = 256;
    static constexpr int MIN_BLOCKS = 4;
    static constexpr int KIND = sizeof(TC) == 8 ? BK_StageAdv64 : -1;
    F2D_DEV static void run(const Args &a, VB vb) { stage_adv_body<TC>(a, vb); }
};
using BStageAdv64 = BStageAdv<double>;
F2D_BATCH_ENTRY(StageAdv64, BStageAdv64)

int stage_advection(const AdvStage &a, cudaStream_t s) {
    dim3 b(32, 8);
    dim3 g = grid2d(a.mv - 2 * NH, a.nv - 2 * NH, b);
    if (a.fp32)
        return launch_body<BStageAdv<float>>(k_stage_adv<float>, a, g, b, 0, s,
                                             "stage_advection");
    return launch_body<BStageAdv<double>>(k_stage_adv<double>, a, g, b, 0, s, "stage_advection");
}

// psi <- psi*mskp (whole array, core/operators.py:481) and
// u,v = orthogradient(psi) (core/fortran_operators.f90:22-37), with the RK
// combinations of u, v (rows/cols 1..m-2) and of psi fused.
F2D_DEV void stage_ortho_body(const OrthoStage &a, const VB vb) {
    __shared__ double sdt6;
    if (threadIdx.x == 0 && threadIdx.y == 0 && (a.rk == 3 || a.psi_rk)) sdt6 = *a.dt / 6.;
    __syncthreads();
    const int i = vb.x * 32 + threadIdx.x;
    const int j = vb.y * 8 + threadIdx.y;
    const int nv = a.nv, mv = a.mv;
    if (i >= nv || j >= mv) return;
    const size_t p = off(j, i, nv);
    // masking is idempotent, so neighbours read before or after their own
    // thread masks them give the same value
    const double pc = (a.premasked || a.mskp[p]) ? a.psi[p] : 0.;
    const double dt = (a.rk || a.psi_rk) ? *a.dt : 0.;
    const double dt6 = (a.rk == 3 || a.psi_rk) ? sdt6 : 0.;
    if (!a.premasked) a.psi[p] = pc;
    if (a.psi_rk) {
        // x += (dt/6)*(dx0 + dx1 + 4*dx2) (core/timescheme.py:180)
        const double d1 = a.psi1 ? a.psi1[p] : pc;
        const double d2 = a.psi1 ? pc : 0.;
        a.psiout[p] = a.psibase[p] + dt6 * (a.psi0[p] + d1 + 4 * d2);
    }
    if (i < 1 || j < 1 || i > nv - 2 || j > mv - 2) return;
    const double ps = (a.premasked || a.mskp[p - nv]) ? a.psi[p - nv] : 0.;
    const double pw = (a.premasked || a.mskp[p - 1]) ? a.psi[p - 1] : 0.;
    const int mc = a.msk[p];
    const double u = (mc + a.msk[p + 1] == 2) ? a.zdy * (ps - pc) : 0.;
    const double v = (mc + a.msk[p + nv] == 2) ? a.zdx * (pc - pw) : 0.;
    a.u[p] = u;
    a.v[p] = v;
    if (a.rk) {
        a.uout[p] = rk_combine(a.rk, a.ubase[p], a.u0 ? a.u0[p] : 0., a.u1 ? a.u1[p] : 0., u, dt,
                               dt6);
        a.vout[p] = rk_combine(a.rk, a.vbase[p], a.v0 ? a.v0[p] : 0., a.v1 ? a.v1[p] : 0., v, dt,
                               dt6);
    }
}

__global__ void __launch_bounds__(256) k_stage_ortho(OrthoStage a) {
    pdl_prologue();
    stage_ortho_body(a, F2D_VB_NATIVE);
}

struct BStageOrtho {
    using Args = OrthoStage;
    static constexpr int THREADS = 256, KIND = BK_StageOrtho, MIN_BLOCKS = 6;
    F2D_DEV static void run(const Args &a, VB vb) { stage_ortho_body(a, vb); }
};
F2D_BATCH_ENTRY(StageOrtho, BStageOrtho)

int stage_ortho(const OrthoStage &a, cudaStream_t s) {
    dim3 b(32, 8);
    return launch_body<BStageOrtho>(k_stage_ortho, a, grid2d(a.mv, a.nv, b), b, 0, s,
                                    "stage_ortho");
}

struct VecAddArgs {
    double *x;
    const double *y;
    size_t n;
    const int *active;
};

F2D_DEV void vec_add_body(const VecAddArgs &A, const VB vb) {
    if (inactive(A.active)) return;
    for (size_t q = vb.x * (size_t)blockDim.x + threadIdx.x; q < A.n;
         q += (size_t)vb.gx * blockDim.x)
        A.x[q] = A.x[q] + A.y[q];
}

__global__ void k_vec_add(VecAddArgs a) { pdl_prologue();
    vec_add_body(a, F2D_VB_NATIVE); }

struct BVecAdd {
    using Args = VecAddArgs;
    static constexpr int THREADS = 256, KIND = BK_VecAdd;
    F2D_DEV static void run(const Args &a, VB vb) { vec_add_body(a, vb); }
};
F2D_BATCH_ENTRY(VecAdd, BVecAdd)

int vec_add(double *x, const double *y, size_t count, const int *active, cudaStream_t s) {
    int blocks = (int)((count + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    return launch_body<BVecAdd>(k_vec_add, VecAddArgs{x, y, count, active}, dim3(blocks),
                                dim3(256), 0, s, "vec_add");
}

// x -= dev_scalar[0] / area (core/operators.py:474-477)
struct SubMeanArgs {
    double *x;
    double area;
    const double *sum;
    size_t n;
};

F2D_DEV void sub_mean_body(const SubMeanArgs &A, const VB vb) {
    const double m = *A.sum / A.area;
    for (size_t q = vb.x * (size_t)blockDim.x + threadIdx.x; q < A.n;
         q += (size_t)vb.gx * blockDim.x)
        A.x[q] = A.x[q] - m;
}

__global__ void k_sub_mean(SubMeanArgs a) { pdl_prologue();
    sub_mean_body(a, F2D_VB_NATIVE); }

struct BSubMean {
    using Args = SubMeanArgs;
    static constexpr int THREADS = 256, KIND = BK_SubMean;
    F2D_DEV static void run(const Args &a, VB vb) { sub_mean_body(a, vb); }
};
F2D_BATCH_ENTRY(SubMean, BSubMean)

int vec_axpy_const(double *x, double area, const double *sum, size_t count, cudaStream_t s) {
    int blocks = (int)((count + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    return launch_body<BSubMean>(k_sub_mean, SubMeanArgs{x, area, sum, count}, dim3(blocks),
                                 dim3(256), 0, s, "sub_mean");
}

// explicit instantiations
#define F2D_INST(T)                                                                              \
    template int mg_sweep1<T>(const LevelView<T> &, const AnalyticT<T> *, T, T, bool,            \
                              const int *, cudaStream_t);                                        \
    template int mg_sweep2<T>(const LevelView<T> &, const AnalyticT<T> *, T, T, const int *,     \
                              cudaStream_t);                                                     \
    template int mg_residual<T>(const LevelView<T> &, const AnalyticT<T> *, const T *, const T *, \
                                T *, const int *, cudaStream_t);                                 \
    template int mg_restrict<T>(const LevelView<T> &, const T *, const LevelView<T> &, T *,      \
                                const int *, cudaStream_t);                                      \
    template int mg_interp<T>(const LevelView<T> &, const T *, const LevelView<T> &, T *, bool,  \
                              const int *, cudaStream_t);                                        \
    template int mg_coarse<T>(const CoarseArgs<T> &, size_t, cudaStream_t);                     \
    template int mg_coarse_columns<T>(const CoarseArgs<T> &, size_t, T *, int, cudaStream_t);    \
    template int mg_coarse_apply<T>(const T *, int, const LevelView<T> &, const int *,           \
                                    cudaStream_t);                                               \
    template int mg_smooth_fused<T>(const LevelView<T> &, const AnalyticT<T> *, T, T, int,       \
                                    const LevelView<T> *, T *, const int *, cudaStream_t);       \
    template int mg_resres<T>(const LevelView<T> &, const AnalyticT<T> *, const LevelView<T> &,  \
                              T *, const int *, cudaStream_t, const uint8_t *, const T *);       \
    template size_t coarse_smem_bytes<T>(const int *, const int *, int);
F2D_INST(double)
F2D_INST(float)

// ------------------------------------------------------------ line relaxation
// the finest level's analytic operator as a tridiagonal-smoother accessor
struct AAnalytic {
    LevelView<double> L;
    Analytic an;
    F2D_DEV double operator()(int k, int j, int i) const { return analytic_coef(L, an, k, j, i); }
};

int mg_tri_factor(const LevelView<double> &L, const Analytic *a0, double *gam, double *bet,
                  cudaStream_t s) {
    const unsigned g = (unsigned)((L.nv - 2 + 127) / 128);
    if (a0)
        k_tri_factor<AAnalytic><<<g, 128, 0, s>>>(L.msk, AAnalytic{L, *a0}, gam, bet, L.mv, L.nv);
    else
        k_tri_factor<AStored><<<g, 128, 0, s>>>(L.msk, AStored{L.A, (size_t)L.mv * L.nv, L.nv},
                                                gam, bet, L.mv, L.nv);
    return launch_status("tri_factor");
}

namespace {
// per library and device: the opt-in shared memory of the two sweep kernels
bool g_tri_configured[2][64];
}

int mg_tri_sweep(const LevelView<double> &L, const Analytic *a0, const double *gam,
                 const double *bet, const int *active, cudaStream_t s) {
    const size_t smem = tri_smem_bytes(L.mv);
    int dev = 0;
    int st0 = cuda_status(cudaGetDevice(&dev), "tri device");
    if (st0) return st0;
    if (smem > 48 * 1024 && dev < 64 && !g_tri_configured[a0 ? 1 : 0][dev]) {
        int st = a0 ? cuda_status(cudaFuncSetAttribute(k_tri_sweep<AAnalytic>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       220 * 1024),
                                  "tri smem")
                    : cuda_status(cudaFuncSetAttribute(k_tri_sweep<AStored>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       220 * 1024),
                                  "tri smem");
        if (st) return st;
        g_tri_configured[a0 ? 1 : 0][dev] = true;
    }
    if (a0)
        k_tri_sweep<AAnalytic><<<1, TRI_THREADS, smem, s>>>(L.msk, AAnalytic{L, *a0}, L.x, L.b,
                                                            gam, bet, L.mv, L.nv, active);
    else
        k_tri_sweep<AStored><<<1, TRI_THREADS, smem, s>>>(
            L.msk, AStored{L.A, (size_t)L.mv * L.nv, L.nv}, L.x, L.b, gam, bet, L.mv, L.nv,
            active);
    return launch_status("tri_sweep");
}

// the coefficient bits of the analytic finest level, from the same rule as
// analytic_coef (a coefficient is nonzero when the point's and the
// neighbour's periodic-image cells are fluid)
__global__ void k_nbmask(LevelView<double> L, uint16_t *nb) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= L.nv || j >= L.mv) return;
    AnalyticT<double> one;
    for (int k = 0; k < 5; k++) one.sc[k] = 1.;
    one.a5 = 1.;
    one.c3 = 1.;
    const double c[9] = {analytic_coef(L, one, 0, j, i),         analytic_coef(L, one, 1, j, i),
                         analytic_coef(L, one, 2, j, i),         analytic_coef(L, one, 3, j, i),
                         analytic_coef(L, one, 3, j, i + 1),     analytic_coef(L, one, 2, j + 1, i - 1),
                         analytic_coef(L, one, 1, j + 1, i),     analytic_coef(L, one, 0, j + 1, i + 1),
                         analytic_coef(L, one, 4, j, i)};
    unsigned b = 0;
    for (int k = 0; k < 9; k++)
        if (c[k] != 0.) b |= 1u << k;
    nb[off(j, i, L.nv)] = (uint16_t)b;
}

int mg_nbmask(const LevelView<double> &L, uint16_t *nb, cudaStream_t s) {
    dim3 b(32, 8);
    k_nbmask<<<grid2d(L.mv, L.nv, b), b, 0, s>>>(L, nb);
    return launch_status("nbmask");
}

__global__ void k_zero_active(double *x, size_t n, const int *active) {
    if (active && *active == 0) return;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        x[q] = 0.;
}

__global__ void k_add_active(double *x, const double *r, size_t n, int assign,
                             const int *active) {
    if (active && *active == 0) return;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        x[q] = assign ? r[q] : x[q] + r[q];
}

int mg_add(double *x, const double *r, size_t n, bool assign, const int *active,
           cudaStream_t s) {
    size_t b = (n + 255) / 256;
    k_add_active<<<(unsigned)(b > 4096 ? 4096 : b), 256, 0, s>>>(x, r, n, assign ? 1 : 0, active);
    return launch_status("mg_add");
}

int mg_zero(double *x, size_t n, const int *active, cudaStream_t s) {
    size_t b = (n + 255) / 256;
    k_zero_active<<<(unsigned)(b > 4096 ? 4096 : b), 256, 0, s>>>(x, n, active);
    return launch_status("mg_zero");
}


// ------------------------------------------------------------ cluster sub-cycle
// The float levels of the mixed form from a level Ls down to the coarse
// operator's level, held in the distributed shared memory of one cluster
// of CL_NC CTAs: a V-cycle (or the F-cycle) from Ls in one launch instead of
// two to three launches a level visit (the small levels' launches are the
// mixed step's latency-bound part).  Each CTA owns a strip of the interior
// rows of every level (the coarse level's rows split evenly, doubled on
// each finer level, so a coarse strip covers exactly its fine strip) plus
// CL_G ghost rows a side; ghost rows are copied from their owners through
// distributed shared memory after a cluster barrier, halo rows as the
// periodic images of interior rows (the reference's halo fill).  Every
// phase evaluates the reference's expressions with the level kernels'
// device functions (jacobi, residual, restrict_value, interp_value, the
// coarse operator's dot product in its order), so the result is the launch
// sequence's bit for bit.  All CTAs run the same sequence of phases and
// barriers; no CTA leaves early.
namespace cgx = cooperative_groups;

struct ClCtx {
    const ClArgs *a;
    unsigned char *sm;
    int rank;
    int cur[CL_MAXLEV];                // x buffer in use, per level
};

F2D_DEV int cl_r0(const ClArgs &a, int k, int c) { return NH + (a.p[c] << (a.nlev - 1 - k)); }

F2D_DEV int cl_owner(const ClArgs &a, int k, int j) {
    int q = 0;
    while (q + 1 < CL_NC && cl_r0(a, k, q + 1) <= j) q++;
    return q;
}

// array at byte offset o of level k in this CTA, indexed by global (j, i)
F2D_DEV float *cl_view(const ClCtx &c, int k, unsigned o) {
    const ClLevel &L = c.a->lv[k];
    return (float *)(c.sm + o) - (ptrdiff_t)(cl_r0(*c.a, k, c.rank) - CL_G) * L.nv;
}

F2D_DEV LevelView<float> cl_level(const ClCtx &c, int k, const float *x, const float *b) {
    const ClLevel &L = c.a->lv[k];
    LevelView<float> v;
    v.mv = L.mv;
    v.nv = L.nv;
    v.msk = L.msk;
    v.A = L.A;
    v.x = (float *)x;
    v.b = (float *)b;
    v.r = nullptr;
    v.t = nullptr;
    v.nb = nullptr;
    return v;
}

// ghost rows [r0-lo, r0) and [r1, r1+hi) of array o of level k from their
// owners (rows outside [0, mv) are skipped; halo rows take their images)
F2D_DEV void cl_fill(const ClCtx &c, cgx::cluster_group &cl, int k, unsigned o, int lo, int hi) {
    const ClArgs &a = *c.a;
    const ClLevel &L = a.lv[k];
    const int nv = L.nv, r0 = cl_r0(a, k, c.rank), r1 = cl_r0(a, k, c.rank + 1);
    float *loc = cl_view(c, k, o);
    const int n = (lo + hi) * nv;
    for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
        const int rr = q / nv, i = q - rr * nv;
        const int j = rr < lo ? r0 - lo + rr : r1 + rr - lo;
        if (j < 0 || j >= L.mv) continue;
        const int src = wrap(j, L.mv, NH);
        const int w = cl_owner(a, k, src);
        const float *rem = cl.map_shared_rank((float *)(c.sm + o), w);
        loc[off(j, i, nv)] = rem[off(src - (cl_r0(a, k, w) - CL_G), i, nv)];
    }
}

// value v at (j, i) of a strip array and its images in the same row
F2D_DEV void cl_put(float *x, int j, int i, int nv, float v) {
    const int n2 = nv - 2 * NH;
    x[off(j, i, nv)] = v;
    if (i >= n2 && i < n2 + NH) x[off(j, i - n2, nv)] = v;
    if (i >= NH && i < 2 * NH) x[off(j, i + n2, nv)] = v;
}

// one smoothtwicewitha call on level k: x (the level's current buffer,
// rows r0-2 .. r1+1 valid) or zero -> t -> the other buffer (strip rows and
// their row images); b rows r0-1 .. r1 valid
F2D_DEV void cl_smooth(ClCtx &c, int k, bool zero_x) {
    const ClArgs &a = *c.a;
    const ClLevel &L = a.lv[k];
    const int mv = L.mv, nv = L.nv, r0 = cl_r0(a, k, c.rank), r1 = cl_r0(a, k, c.rank + 1);
    const float *x = cl_view(c, k, L.o_x[c.cur[k]]);
    float *t = cl_view(c, k, L.o_t), *y = cl_view(c, k, L.o_x[c.cur[k] ^ 1]);
    const float *b = cl_view(c, k, L.o_b);
    const LevelView<float> V = cl_level(c, k, x, b);
    if (r1 > r0) {
        const int ja = max(2, r0 - 1), jb = min(mv - 3, r1), w = nv - 4;
        const int n = (jb - ja + 1) * w;
        for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
            const int rr = q / w, j = ja + rr, i = 2 + q - rr * w;
            t[off(j, i, nv)] = jacobi<float, false>(V, nullptr, zero_x ? nullptr : x, b, j, i, 0.f,
                                                    a.c2);
        }
    }
    __syncthreads();
    {
        const LevelView<float> W = cl_level(c, k, t, b);
        const int w = nv - 2 * NH, n = (r1 - r0) * w;
        for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
            const int rr = q / w, j = r0 + rr, i = NH + q - rr * w;
            cl_put(y, j, i, nv, jacobi<float, false>(W, nullptr, t, b, j, i, 0.f, a.c2));
        }
    }
    c.cur[k] ^= 1;
}

// x of level k (rows r0-2 .. r1+1, columns 1 .. nv-2) = prolongation of
// level k+1's x (plus x itself unless assign); level k+1's x rows valid
// from its r0-2 to its r1+1
F2D_DEV void cl_interp(ClCtx &c, int k, bool assign) {
    const ClArgs &a = *c.a;
    const ClLevel &F = a.lv[k], &C = a.lv[k + 1];
    const int mv = F.mv, nv = F.nv, r0 = cl_r0(a, k, c.rank), r1 = cl_r0(a, k, c.rank + 1);
    float *x = cl_view(c, k, F.o_x[c.cur[k]]);
    const float *xc = cl_view(c, k + 1, C.o_x[c.cur[k + 1]]);
    const int ja = max(1, r0 - CL_G), jb = min(mv - 2, r1 + CL_G - 1), w = nv - 2;
    const int n = r1 > r0 ? (jb - ja + 1) * w : 0;
    for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
        const int rr = q / w, j = ja + rr, i = 1 + q - rr * w;
        const float v = interp_value(F.msk, nv, C.msk, xc, C.nv, j, i);
        x[off(j, i, nv)] = assign ? v : x[off(j, i, nv)] + v;
    }
}

// residual of level k (strip rows and the row above: the restriction's
// reach) into t, then full weighting into level k+1's b (its strip rows)
F2D_DEV void cl_resres(ClCtx &c, int k) {
    const ClArgs &a = *c.a;
    const ClLevel &F = a.lv[k], &C = a.lv[k + 1];
    const int mv = F.mv, nv = F.nv, r0 = cl_r0(a, k, c.rank), r1 = cl_r0(a, k, c.rank + 1);
    const int m2 = mv - 2 * NH, n2 = nv - 2 * NH;
    const float *x = cl_view(c, k, F.o_x[c.cur[k]]);
    const float *b = cl_view(c, k, F.o_b);
    float *r = cl_view(c, k, F.o_t);
    if (r1 > r0) {
        // rows r0 .. r1 at interior columns; the row above the top strip is
        // the halo row whose image is row NH: its operator and mask are row
        // NH's (the view shifted by m2 rows), its x and b the images here
        const int w = n2, n = (r1 - r0 + 1) * w;
        for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
            const int rr = q / w, j = r0 + rr, i = NH + q - rr * w;
            LevelView<float> V = cl_level(c, k, x, b);
            if (j >= mv - NH) {
                V.msk -= (ptrdiff_t)m2 * nv;
                V.A -= (ptrdiff_t)m2 * nv;
            }
            cl_put(r, j, i, nv, residual<float, false>(V, nullptr, x, b, j, i));
        }
    }
    __syncthreads();
    const int R0 = cl_r0(a, k + 1, c.rank), R1 = cl_r0(a, k + 1, c.rank + 1);
    float *b2 = cl_view(c, k + 1, C.o_b);
    const int w2 = C.nv - 2 * NH, n = (R1 - R0) * w2;
    for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
        const int rr = q / w2, J = R0 + rr, I = NH + q - rr * w2;
        cl_put(b2, J, I, C.nv, restrict_value(C.msk, C.nv, r, nv, J, I));
    }
}

// level k+1's b (strip rows) = full weighting of level k's b (the
// F-cycle's coarsening of the right-hand side); level k's b rows valid to r1
F2D_DEV void cl_restrict_b(ClCtx &c, int k) {
    const ClArgs &a = *c.a;
    const ClLevel &F = a.lv[k], &C = a.lv[k + 1];
    const float *b = cl_view(c, k, F.o_b);
    const int R0 = cl_r0(a, k + 1, c.rank), R1 = cl_r0(a, k + 1, c.rank + 1);
    float *b2 = cl_view(c, k + 1, C.o_b);
    const int w2 = C.nv - 2 * NH, n = (R1 - R0) * w2;
    for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
        const int rr = q / w2, J = R0 + rr, I = NH + q - rr * w2;
        cl_put(b2, J, I, C.nv, restrict_value(C.msk, C.nv, b, F.nv, J, I));
    }
}

// the coarse level's x = op . (its interior b), one warp per point, summed
// in k_coarse_apply's order
F2D_DEV void cl_coarse(ClCtx &c, cgx::cluster_group &cl, const float *op) {
    const ClArgs &a = *c.a;
    const int k = a.nlev - 1;
    const ClLevel &L = a.lv[k];
    const int nv = L.nv, n2 = nv - 2 * NH, n = a.n;
    float *g = (float *)(c.sm + a.o_g);
    for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
        const int qj = q / n2, j = NH + qj, i = NH + q - qj * n2;
        const int w = cl_owner(a, k, j);
        const float *rem = cl.map_shared_rank((float *)(c.sm + L.o_b), w);
        g[q] = rem[off(j - (cl_r0(a, k, w) - CL_G), i, nv)];
    }
    __syncthreads();
    float *x = cl_view(c, k, L.o_x[c.cur[k]]);
    const int r0 = cl_r0(a, k, c.rank), r1 = cl_r0(a, k, c.rank + 1);
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    const int np = (r1 - r0) * n2;
    for (int pt = warp; pt < np; pt += CL_THREADS / 32) {
        const int rr = pt / n2, j = r0 + rr, i = NH + pt - rr * n2;
        const int row = (j - NH) * n2 + (i - NH);
        const float *orow = op + (size_t)row * n;
        float s0 = 0.f, s1 = 0.f;
        int q = lane;
        for (; q + 32 < n; q += 64) {
            s0 = fma(orow[q], g[q], s0);
            s1 = fma(orow[q + 32], g[q + 32], s1);
        }
        if (q < n) s0 = fma(orow[q], g[q], s0);
        float v = s0 + s1;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) cl_put(x, j, i, nv, v);
    }
}

// a V-cycle from level k0 (its b rows r0-1 .. r1 valid): the first smooth
// from zero, or (f_interp) from the prolongation of level k0+1's x
F2D_DEV void cl_vcycle(ClCtx &c, cgx::cluster_group &cl, int k0, bool f_interp) {
    const ClArgs &a = *c.a;
    const int K = a.nlev - 1;
    for (int k = k0; k < K; k++) {
        if (k == k0 && f_interp) {
            cl_interp(c, k, true);
            __syncthreads();
            cl_smooth(c, k, false);
        } else {
            cl_smooth(c, k, true);
        }
        cl.sync();
        cl_fill(c, cl, k, a.lv[k].o_x[c.cur[k]], CL_G, CL_G);
        __syncthreads();
        cl_resres(c, k);
        cl.sync();
        cl_fill(c, cl, k + 1, a.lv[k + 1].o_b, 1, 1);
        __syncthreads();
    }
    cl_coarse(c, cl, a.op_v);
    for (int k = K - 1; k >= k0; k--) {
        cl.sync();
        cl_fill(c, cl, k + 1, a.lv[k + 1].o_x[c.cur[k + 1]], CL_G, CL_G);
        __syncthreads();
        cl_interp(c, k, false);
        __syncthreads();
        cl_smooth(c, k, false);
    }
}

F2D_DEV void cl_body(const ClArgs &a) {
    cgx::cluster_group cl = cgx::this_cluster();
    extern __shared__ __align__(16) unsigned char cl_sm[];
    ClCtx c;
    c.a = &a;
    c.sm = cl_sm;
    c.rank = (int)cl.block_rank();
    for (int k = 0; k < CL_MAXLEV; k++) c.cur[k] = 0;
    const bool skip = inactive(a.active);  // the same in every CTA: no barrier is skipped alone
    if (skip) return;
    const ClLevel &L0 = a.lv[0];
    {   // level Ls's b, strip rows and CL_G ghost rows a side, from global memory
        const int r0 = cl_r0(a, 0, c.rank), r1 = cl_r0(a, 0, c.rank + 1);
        const int ja = max(0, r0 - CL_G), jb = min(L0.mv - 1, r1 + CL_G - 1), nv = L0.nv;
        float *b = cl_view(c, 0, L0.o_b);
        const int n = (jb - ja + 1) * nv;
        for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) b[(size_t)ja * nv + q] = a.b_top[(size_t)ja * nv + q];
    }
    __syncthreads();
    const int K = a.nlev - 1;
    if (a.mode == CYCLE_V) {
        cl_vcycle(c, cl, 0, false);
    } else {
        for (int k = 0; k < K; k++) {
            cl_restrict_b(c, k);
            cl.sync();
            cl_fill(c, cl, k + 1, a.lv[k + 1].o_b, 1, 1);
            __syncthreads();
        }
        cl_coarse(c, cl, a.op);
        for (int k = K - 1; k >= 0; k--) {
            cl.sync();
            cl_fill(c, cl, k + 1, a.lv[k + 1].o_x[c.cur[k + 1]], CL_G, CL_G);
            __syncthreads();
            cl_vcycle(c, cl, k, true);
        }
    }
    // level Ls's x: strip rows with their images, to global memory
    const int r0 = cl_r0(a, 0, c.rank), r1 = cl_r0(a, 0, c.rank + 1), nv = L0.nv;
    const float *x = cl_view(c, 0, L0.o_x[c.cur[0]]);
    const int w = nv - 2 * NH, n = (r1 - r0) * w;
    for (int q = (int)threadIdx.x; q < n; q += CL_THREADS) {
        const int rr = q / w, j = r0 + rr, i = NH + q - rr * w;
        store_images(a.x_top, j, i, L0.mv, nv, x[off(j, i, nv)]);
    }
    // no CTA leaves while another may still read its shared memory
    cl.sync();
}

__global__ void __launch_bounds__(CL_THREADS, 1) k_cluster_cycle(const __grid_constant__ ClArgs a) {
    pdl_prologue();
    cl_body(a);
}

// cluster launch attributes of k_cluster_cycle (CL_NC CTAs: a non-portable
// cluster size) and `smem` bytes of dynamic shared memory
static int cl_config(size_t smem, cudaStream_t s, cudaLaunchConfig_t *cfg,
                     cudaLaunchAttribute *attr) {
    // the function attributes once (set-up time, outside any stream capture),
    // for every layout up to CL_SMEM_MAX bytes
    static int attrs = -1;
    if (attrs < 0) {
        int st = cuda_status(cudaFuncSetAttribute(k_cluster_cycle,
                                                  cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                             "cluster size attribute");
        if (!st)
            st = cuda_status(cudaFuncSetAttribute(k_cluster_cycle,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)CL_SMEM_MAX),
                             "cluster shared memory attribute");
        attrs = st;
    }
    if (attrs) return attrs;
    if (smem > CL_SMEM_MAX) return ERR_ARG;
    memset(cfg, 0, sizeof(*cfg));
    cfg->gridDim = dim3(CL_NC);
    cfg->blockDim = dim3(CL_THREADS);
    cfg->dynamicSmemBytes = smem;
    cfg->stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL_NC;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg->attrs = attr;
    cfg->numAttrs = pdl_enabled() ? 2 : 1;
    return OK;
}

// whether a cluster of k_cluster_cycle with `smem` bytes can be resident
bool mg_cluster_feasible(size_t smem) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[2];
    if (cl_config(smem, nullptr, &cfg, attr) != OK) {
        (void)cudaGetLastError();
        return false;
    }
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_cluster_cycle, &cfg) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return n > 0;
}

int mg_cluster_cycle(const ClArgs &a, size_t smem, cudaStream_t s) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[2];
    int st = cl_config(smem, s, &cfg, attr);
    if (st) return st;
    return cuda_status(cudaLaunchKernelEx(&cfg, k_cluster_cycle, a), "mg_cluster_cycle");
}

// the mixed form's cluster sub-cycle: 0 (the default) off, the level
// kernels; m >= 1 (product build) one cluster launch a sub-cycle from m
// levels above the coarse operator's level (fewer if they do not fit).
// Measured slower than the level kernels at every m on the GB300.
int &cluster_mode() {
    static int m = 0;
    return m;
}
}  // namespace f2d

extern "C" {

// the mixed form's cluster sub-cycle: 0 off (the default), m = 1..8 from m
// levels above the coarse operator's level (product build; the exact build
// keeps 0); < 0 only queries; returns the previous setting.  It applies to
// models created after the change.
int f2d_set_cluster(int mode) {
    const int prev = f2d::cluster_mode();
#ifndef F2D_EXACT
    if (mode >= 0 && mode <= 8) f2d::cluster_mode() = mode;
#endif
    return prev;
}

// the CTA count the multigrid level kernels aim at when they choose their
// tile: -1 twice the SM count, 0 always the largest tile (the default), > 0
// that count, < -1 only queries; returns the previous setting.
int f2d_set_level_tiles(int target) {
    const int prev = f2d::level_tile_target();
    if (target >= -1) f2d::level_tile_target() = target;
    return prev;
}

// the float64 finest level's sweeps and residual: 1 the column form where
// the operator allows on grids of at least one CTA per SM (the product
// build's default), 2 at every grid size, 0 the sweep and residual kernels
// in the reference's order; < 0 only queries; returns the previous setting.
// The exact build always takes the reference's order (0).
int f2d_set_separable(int mode) {
    const int prev = f2d::separable_mode();
#ifndef F2D_EXACT
    if (mode >= 0 && mode <= 2) f2d::separable_mode() = mode;
#endif
    return prev;
}

// threads of the fused smoother: 0 one per tile point (the default), 1 one per
// input point for grids of fewer than two CTAs per SM, 2 always one per input
// point; < 0 only queries; returns the previous setting.
int f2d_set_level_threads(int mode) {
    const int prev = f2d::level_one_pass();
    if (mode >= 0 && mode <= 2) f2d::level_one_pass() = mode;
    return prev;
}

}  // extern "C"
