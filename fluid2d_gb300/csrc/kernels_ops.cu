// kernels_ops.cu -- grid operators and masked diagnostics.
//
// Drop-in kernels for
//   fortran_operators.computeorthogradient  (core/fortran_operators.f90:2-39)
//   fortran_operators.celltocorner          (:44-64)
//   fortran_operators.cornertocell          (:102-122)
//   fortran_operators.add_diffusion         (:125-156)
//   fortran_operators.add_torque            (:330-381)
//   fortran_diag.*                          (core/fortran_diag.f90)
//   gmg.fortran_multigrid.computenorm/computeinner
//                                           (core/gmg/fortran_multigrid.f90:813-867)
// Each kernel covers exactly the Fortran loop range; cells outside it are
// left as they are.  The diagnostics are deterministic fixed-order tree
// reductions (the reference sums sequentially, so sums agree to rounding;
// maxima agree exactly).
#include "f2d_common.cuh"
#include "f2d_kernels.cuh"

#include "f2d_batch.cuh"

namespace f2d {

constexpr int OP_TX = 32, OP_TY = 8;

// u(j,i) = zdy*(psi(j-1,i)-psi(j,i)) where msk(j,i)+msk(j,i+1)==2,
// v(j,i) = zdx*(psi(j,i)-psi(j,i-1)) where msk(j,i)+msk(j+1,i)==2,
// j,i in 2..m-1 (1-based).
__global__ void k_orthogradient(const int8_t *__restrict__ msk, const double *__restrict__ psi,
                                double zdx, double zdy, int m, int n,
                                double *__restrict__ u, double *__restrict__ v) {
    int i = 1 + blockIdx.x * OP_TX + threadIdx.x;
    int j = 1 + blockIdx.y * OP_TY + threadIdx.y;
    if (i > n - 2 || j > m - 2) return;
    size_t p = off(j, i, n);
    int mc = msk[p];
    u[p] = (mc + msk[p + 1] == 2) ? zdy * (psi[p - n] - psi[p]) : 0.;
    v[p] = (mc + msk[p + n] == 2) ? zdx * (psi[p] - psi[p - 1]) : 0.;
}

int launch_orthogradient(const int8_t *msk, const double *psi, double dx, double dy,
                         int m, int n, double *u, double *v, cudaStream_t s) {
    if (m < 3 || n < 3) return OK;
    double zdx = 1. / dx, zdy = 1. / dy;
    dim3 b(OP_TX, OP_TY);
    k_orthogradient<<<grid2d(m - 2, n - 2, b), b, 0, s>>>(msk, psi, zdx, zdy, m, n, u, v);
    return launch_status("computeorthogradient");
}

// xp(j,i) = 0.25*(xr(j,i)+xr(j,i+1)+xr(j+1,i)+xr(j+1,i+1)), j,i in 1..m-1
struct CellToCornerArgs {
    const double *xr;
    double *xp;
    int m, n;
};

F2D_DEV void celltocorner_body(const CellToCornerArgs &a, const VB vb) {
    const int m = a.m, n = a.n;
    int i = vb.x * OP_TX + threadIdx.x;
    int j = vb.y * OP_TY + threadIdx.y;
    if (i > n - 2 || j > m - 2) return;
    size_t p = off(j, i, n);
    const double *xr = a.xr;
    a.xp[p] = 0.25 * (xr[p] + xr[p + 1] + xr[p + n] + xr[p + n + 1]);
}

__global__ void k_celltocorner(CellToCornerArgs a) { pdl_prologue();
    celltocorner_body(a, F2D_VB_NATIVE); }

struct BCellToCorner {
    using Args = CellToCornerArgs;
    static constexpr int THREADS = OP_TX * OP_TY, KIND = BK_CellToCorner;
    F2D_DEV static void run(const Args &a, VB vb) { celltocorner_body(a, vb); }
};
F2D_BATCH_ENTRY(CellToCorner, BCellToCorner)

int launch_celltocorner(const double *xr, double *xp, int m, int n, cudaStream_t s) {
    if (m < 2 || n < 2) return OK;
    dim3 b(OP_TX, OP_TY);
    return launch_body<BCellToCorner>(k_celltocorner, CellToCornerArgs{xr, xp, m, n},
                                      grid2d(m - 1, n - 1, b), b, 0, s, "celltocorner");
}

// xr(j,i) = 0.25*(xp(j,i)+xp(j,i-1)+xp(j-1,i)+xp(j-1,i-1)), j,i in 2..m
__global__ void k_cornertocell(const double *__restrict__ xp, double *__restrict__ xr, int m, int n) {
    int i = 1 + blockIdx.x * OP_TX + threadIdx.x;
    int j = 1 + blockIdx.y * OP_TY + threadIdx.y;
    if (i > n - 1 || j > m - 1) return;
    size_t p = off(j, i, n);
    xr[p] = 0.25 * (xp[p] + xp[p - 1] + xp[p - n] + xp[p - n - 1]);
}

int launch_cornertocell(const double *xp, double *xr, int m, int n, cudaStream_t s) {
    if (m < 2 || n < 2) return OK;
    dim3 b(OP_TX, OP_TY);
    k_cornertocell<<<grid2d(m - 1, n - 1, b), b, 0, s>>>(xp, xr, m, n);
    return launch_status("cornertocell");
}

// dtrac += Kdiff/dx^2 * sum_nb msk(nb)*(trac(nb)-trac), where msk==1, j,i in 2..m-1
__global__ void k_add_diffusion(const int8_t *__restrict__ msk, const double *__restrict__ trac,
                                double coef, int m, int n, double *__restrict__ dtrac) {
    int i = 1 + blockIdx.x * OP_TX + threadIdx.x;
    int j = 1 + blockIdx.y * OP_TY + threadIdx.y;
    if (i > n - 2 || j > m - 2) return;
    size_t p = off(j, i, n);
    if (msk[p] != 1) return;
    double t = trac[p];
    dtrac[p] = dtrac[p] + coef * (+(double)msk[p - 1] * (trac[p - 1] - t)
                                  + (double)msk[p + 1] * (trac[p + 1] - t)
                                  + (double)msk[p - n] * (trac[p - n] - t)
                                  + (double)msk[p + n] * (trac[p + n] - t));
}

int launch_add_diffusion(const int8_t *msk, const double *trac, double dx, double Kdiff,
                         double *dtrac, int m, int n, cudaStream_t s) {
    if (m < 3 || n < 3) return OK;
    double coef = Kdiff / (dx * dx);
    dim3 b(OP_TX, OP_TY);
    k_add_diffusion<<<grid2d(m - 2, n - 2, b), b, 0, s>>>(msk, trac, coef, m, n, dtrac);
    return launch_status("add_diffusion");
}

// domega += (b(i+1)-b(i-1))*coef*msk where max(1,m(i)+m(i-1)) + max(1,m(i+1)+m(i)) == 4,
// interior cells (core/fortran_operators.f90:351-377)
__global__ void k_add_torque(const int8_t *__restrict__ msk, const double *__restrict__ b,
                             double coef, int nh, int m, int n, double *__restrict__ w) {
    int i = nh + blockIdx.x * OP_TX + threadIdx.x;
    int j = nh + blockIdx.y * OP_TY + threadIdx.y;
    if (i > n - nh - 1 || j > m - nh - 1) return;
    size_t p = off(j, i, n);
    int mc = msk[p];
    int sl = mc + msk[p - 1], sr = msk[p + 1] + mc;
    int ml = sl > 1 ? sl : 1, mr = sr > 1 ? sr : 1;
    if (ml + mr == 4) w[p] = w[p] + (b[p + 1] - b[p - 1]) * coef * (double)mc;
}

int launch_add_torque(const int8_t *msk, const double *b, double dx, int nh, double gravity,
                      double *w, int m, int n, cudaStream_t s) {
    if (m <= 2 * nh || n <= 2 * nh) return OK;
    double coef = 0.5 * gravity / dx;
    dim3 bl(OP_TX, OP_TY);
    k_add_torque<<<grid2d(m - 2 * nh, n - 2 * nh, bl), bl, 0, s>>>(msk, b, coef, nh, m, n, w);
    return launch_status("add_torque");
}

// ---------------------------------------------------------------- reductions
// Per-point contributions of each diagnostic over interior cells.
enum RedKind {
    R_DOT = 0,        // sum x*y, msk != 0        (computedotprod, computeinner)
    R_MAX = 1,        // max |x|, msk != 0        (computemax)
    R_SUM = 2,        // sum x, msk != 0          (computesum)
    R_SUMNORM = 3,    // sum x, sum x^2, msk == 1 (computesumandnorm)
    R_NORMMAXU = 4,   // sum x^2, max|x|, msk(i)+msk(i+1)==2 (computenormmaxu)
    R_KEMAXU = 5,     // ke, maxu                 (computekemaxu)
    R_KEMAXUV = 6,    // ke, maxu, maxv           (computekemaxuv)
    R_KEWITHPSI = 7,  // -0.125*(4 psi corners)*omega (computekewithpsi)
    R_NORM = 8,       // sum x^2, msk != 0        (computenorm)
};

struct RedSpec {
    int nv;
    bool is_max[RED_MAX_VALUES];
};

__host__ __device__ constexpr RedSpec red_spec(int kind) {
    return kind == R_MAX       ? RedSpec{1, {true, false, false, false}}
           : kind == R_SUMNORM ? RedSpec{2, {false, false, false, false}}
           : kind == R_NORMMAXU || kind == R_KEMAXU ? RedSpec{2, {false, true, false, false}}
           : kind == R_KEMAXUV ? RedSpec{3, {false, true, true, false}}
                               : RedSpec{1, {false, false, false, false}};
}

template <int KIND>
F2D_DEV void red_point(const int8_t *msk, const double *x, const double *y, size_t p, int n,
                       double (&acc)[RED_MAX_VALUES]) {
    int mc = msk[p];
    if (KIND == R_DOT) {
        if (mc != 0) acc[0] += x[p] * y[p];
    } else if (KIND == R_MAX) {
        if (mc != 0) { double a = fabs(x[p]); acc[0] = acc[0] > a ? acc[0] : a; }
    } else if (KIND == R_SUM) {
        if (mc != 0) acc[0] += x[p];
    } else if (KIND == R_SUMNORM) {
        if (mc == 1) { double a = x[p]; acc[0] += a; acc[1] += a * a; }
    } else if (KIND == R_NORMMAXU) {
        if (mc + msk[p + 1] == 2) {
            double a = x[p];
            acc[0] += a * a;
            double b = fabs(a);
            acc[1] = acc[1] > b ? acc[1] : b;
        }
    } else if (KIND == R_KEMAXU) {
        if (mc == 1) {
            double a = x[p], b = x[p - 1], c = y[p], d = y[p - n];
            double zu = a * a + b * b;
            double zv = c * c + d * d;
            acc[0] += zu + zv;
            double s = fabs(a + b) + fabs(c + d);
            acc[1] = acc[1] > s ? acc[1] : s;
        }
    } else if (KIND == R_KEMAXUV) {
        if (mc == 1) {
            double a = x[p], b = x[p - 1], c = y[p], d = y[p - n];
            double zu = a * a + b * b;
            double zv = c * c + d * d;
            acc[0] += zu + zv;
            acc[1] = acc[1] > zu ? acc[1] : zu;
            acc[2] = acc[2] > zv ? acc[2] : zv;
        }
    } else if (KIND == R_KEWITHPSI) {
        // x = omega, y = psi
        if (mc == 1) acc[0] -= 0.125 * (y[p] + y[p - n] + y[p - n - 1] + y[p - 1]) * x[p];
    } else if (KIND == R_NORM) {
        if (mc != 0) acc[0] += x[p] * x[p];
    }
}

// Stage 1: block b reduces interior rows [b*rpb, (b+1)*rpb) (threads stride
// over the row-major cells of those rows), writes NV partials.
struct ReducePartialArgs {
    const int8_t *msk;
    const double *x, *y;
    int nh, m, n, rpb;
    double *part;
};

template <int KIND>
F2D_DEV void reduce_partial_body(const ReducePartialArgs &a, const VB vb) {
    __shared__ double sh[RED_MAX_VALUES * RED_THREADS];
    constexpr RedSpec spec = red_spec(KIND);
    const int8_t *msk = a.msk;
    const double *x = a.x, *y = a.y;
    const int nh = a.nh, m = a.m, n = a.n, rpb = a.rpb;
    double *part = a.part;
    double acc[RED_MAX_VALUES] = {0., 0., 0., 0.};
    const int rows = m - 2 * nh, cols = n - 2 * nh;
    const int r0 = vb.x * rpb;
    const int r1 = min(rows, r0 + rpb);
    // thread t takes cells t, t + RED_THREADS, ... of the block's rows in
    // row-major order; its (row, column) advances without a division per cell
    const int cells = (r1 - r0) * cols;
    int jr = (int)threadIdx.x / cols, ic = (int)threadIdx.x - jr * cols;
    for (int q = threadIdx.x; q < cells; q += RED_THREADS) {
        red_point<KIND>(msk, x, y, off(nh + r0 + jr, nh + ic, n), n, acc);
        ic += RED_THREADS;
        while (ic >= cols) {
            ic -= cols;
            jr++;
        }
    }
    double v[RED_MAX_VALUES];
    bool mx[RED_MAX_VALUES];
#pragma unroll
    for (int k = 0; k < RED_MAX_VALUES; k++) { v[k] = acc[k]; mx[k] = spec.is_max[k]; }
    block_reduce<RED_MAX_VALUES>(v, mx, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < spec.nv; k++) part[k * RED_MAX_BLOCKS + vb.x] = v[k];
}

template <int KIND>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_partial(ReducePartialArgs a) {
    pdl_prologue();
    reduce_partial_body<KIND>(a, F2D_VB_NATIVE);
}

// Stage 2: one block reduces the partials in block order and applies the
// routine's final scaling.
struct ReduceFinalArgs {
    const double *part;
    int nblocks;
    double *out;
};

template <int KIND>
F2D_DEV void reduce_final_body(const ReduceFinalArgs &a, const VB) {
    const double *part = a.part;
    const int nblocks = a.nblocks;
    double *out = a.out;
    __shared__ double sh[RED_MAX_VALUES * RED_THREADS];
    constexpr RedSpec spec = red_spec(KIND);
    double acc[RED_MAX_VALUES] = {0., 0., 0., 0.};
    for (int b = threadIdx.x; b < nblocks; b += RED_THREADS)
        for (int k = 0; k < spec.nv; k++) {
            double a = part[k * RED_MAX_BLOCKS + b];
            acc[k] = spec.is_max[k] ? (acc[k] > a ? acc[k] : a) : acc[k] + a;
        }
    double v[RED_MAX_VALUES];
    bool mx[RED_MAX_VALUES];
#pragma unroll
    for (int k = 0; k < RED_MAX_VALUES; k++) { v[k] = acc[k]; mx[k] = spec.is_max[k]; }
    block_reduce<RED_MAX_VALUES>(v, mx, sh);
    if (threadIdx.x == 0) {
        if (KIND == R_KEMAXU) {  // core/fortran_diag.f90:192-193
            out[0] = v[0] * 0.25;
            out[1] = v[1] * 0.5;
        } else if (KIND == R_KEMAXUV) {  // :232-234
            out[0] = v[0] * 0.25;
            out[1] = sqrt(v[1] / 2.);
            out[2] = sqrt(v[2] / 2.);
        } else {
            for (int k = 0; k < spec.nv; k++) out[k] = v[k];
        }
    }
}

template <int KIND>
__global__ void __launch_bounds__(RED_THREADS) k_reduce_final(ReduceFinalArgs a) {
    pdl_prologue();
    reduce_final_body<KIND>(a, F2D_VB_NATIVE);
}

template <int RK>
struct BReducePartial {
    using Args = ReducePartialArgs;
    static constexpr int THREADS = RED_THREADS;
    static constexpr int KIND = RK == R_NORM ? BK_Reduce8P : (RK == R_SUM ? BK_Reduce2P : -1);
    F2D_DEV static void run(const Args &a, VB vb) { reduce_partial_body<RK>(a, vb); }
};
template <int RK>
struct BReduceFinal {
    using Args = ReduceFinalArgs;
    static constexpr int THREADS = RED_THREADS;
    static constexpr int KIND = RK == R_NORM ? BK_Reduce8F : (RK == R_SUM ? BK_Reduce2F : -1);
    F2D_DEV static void run(const Args &a, VB vb) { reduce_final_body<RK>(a, vb); }
};
using BReduce8P = BReducePartial<R_NORM>;
using BReduce8F = BReduceFinal<R_NORM>;
using BReduce2P = BReducePartial<R_SUM>;
using BReduce2F = BReduceFinal<R_SUM>;
F2D_BATCH_ENTRY(Reduce8P, BReduce8P)
F2D_BATCH_ENTRY(Reduce8F, BReduce8F)
F2D_BATCH_ENTRY(Reduce2P, BReduce2P)
F2D_BATCH_ENTRY(Reduce2F, BReduce2F)

int reduce_blocks(int rows) {
    if (rows <= 0) return 1;
    int rpb = (rows + RED_MAX_BLOCKS - 1) / RED_MAX_BLOCKS;
    if (rpb < 1) rpb = 1;
    return (rows + rpb - 1) / rpb;
}

template <int KIND>
static int launch_reduce_t(const int8_t *msk, const double *x, const double *y, int nh,
                           int m, int n, double *out, double *work, cudaStream_t s) {
    int rows = m - 2 * nh;
    if (rows < 0) rows = 0;
    int nb = reduce_blocks(rows);
    int rpb = rows > 0 ? (rows + nb - 1) / nb : 1;
    nb = rows > 0 ? (rows + rpb - 1) / rpb : 1;
    int st = launch_body<BReducePartial<KIND>>(k_reduce_partial<KIND>,
                                               ReducePartialArgs{msk, x, y, nh, m, n, rpb, work},
                                               dim3(nb), dim3(RED_THREADS), 0, s, "reduction");
    if (st) return st;
    return launch_body<BReduceFinal<KIND>>(k_reduce_final<KIND>, ReduceFinalArgs{work, nb, out},
                                           dim3(1), dim3(RED_THREADS), 0, s, "reduction");
}

int launch_reduce(int kind, const int8_t *msk, const double *x, const double *y, int nh,
                  int m, int n, double *out, double *work, cudaStream_t s) {
    if (!msk || !x || !out) {
        set_error("reduction: null pointer");
        return ERR_ARG;
    }
    int st = OK;
    if (!work) {
        work = reduce_workspace(&st);
        if (st) return st;
    }
    switch (kind) {
        case R_DOT: return launch_reduce_t<R_DOT>(msk, x, y, nh, m, n, out, work, s);
        case R_MAX: return launch_reduce_t<R_MAX>(msk, x, y, nh, m, n, out, work, s);
        case R_SUM: return launch_reduce_t<R_SUM>(msk, x, y, nh, m, n, out, work, s);
        case R_SUMNORM: return launch_reduce_t<R_SUMNORM>(msk, x, y, nh, m, n, out, work, s);
        case R_NORMMAXU: return launch_reduce_t<R_NORMMAXU>(msk, x, y, nh, m, n, out, work, s);
        case R_KEMAXU: return launch_reduce_t<R_KEMAXU>(msk, x, y, nh, m, n, out, work, s);
        case R_KEMAXUV: return launch_reduce_t<R_KEMAXUV>(msk, x, y, nh, m, n, out, work, s);
        case R_KEWITHPSI: return launch_reduce_t<R_KEWITHPSI>(msk, x, y, nh, m, n, out, work, s);
        case R_NORM: return launch_reduce_t<R_NORM>(msk, x, y, nh, m, n, out, work, s);
        default: set_error("reduction: bad kind %d", kind); return ERR_ARG;
    }
}

}  // namespace f2d
