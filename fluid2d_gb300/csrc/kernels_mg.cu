// kernels_mg.cu -- drop-in kernels of the geometric multigrid.
//
//   smoothtwicewitha      core/gmg/fortran_multigrid.f90:2-127
//   computeresidualwitha  :320-362
//   fillhalo              :365-412
//   interpolate           :415-498
//   restrict              :501-546
//   coarsenmatrix         :706-811
//
// Stencil storage: the reference's A(j,i,k) (5 planes: SW, S, SE, W, C of a
// symmetric 9-point operator) is stored here plane by plane, A[k][j][i]
// (k = 0..4), so that every plane is coalesced along i.  The 9-plane
// arrays of coarsenmatrix are stored the same way with 9 planes.
#include "f2d_common.cuh"
#include "f2d_kernels.cuh"
#include "f2d_tri.cuh"

namespace f2d {

constexpr int MG_TX = 32, MG_TY = 8;

// One damped-Jacobi update at (j, i) of the array q (row stride n), with
// the symmetric-storage neighbours of core/gmg/fortran_multigrid.f90:66-85:
//   c2*q(j,i) + (c1/|A5(j,i)|)*( A1(j,i)q(j-1,i-1) + A2(j,i)q(j-1,i)
//     + A3(j,i)q(j-1,i+1) + A4(j,i)q(j,i-1) + A4(j,i+1)q(j,i+1)
//     + A3(j+1,i-1)q(j+1,i-1) + A2(j+1,i)q(j+1,i) + A1(j+1,i+1)q(j+1,i+1)
//     - b(j,i) )
// Masked points give 0.
F2D_DEV double jacobi_point(const int8_t *msk, const double *A, size_t plane,
                            const double *q, const double *b, size_t p, int n,
                            double c1, double c2) {
    if (msk[p] == 0) return 0.;
    const double *A1 = A, *A2 = A + plane, *A3 = A + 2 * plane, *A4 = A + 3 * plane,
                 *A5 = A + 4 * plane;
    double c3 = c1 / fabs(A5[p]);
    return q[p] * c2 + c3 * (+A1[p] * q[p - n - 1]
                             + A2[p] * q[p - n]
                             + A3[p] * q[p - n + 1]
                             + A4[p] * q[p - 1]
                             + A4[p + 1] * q[p + 1]
                             + A3[p + n - 1] * q[p + n - 1]
                             + A2[p + n] * q[p + n]
                             + A1[p + n + 1] * q[p + n + 1]
                             - b[p]);
}

// First sweep of smoothtwicewitha: t = J(x) on rows/cols 1..m-2 (0-based).
__global__ void k_smooth_sweep1(const int8_t *__restrict__ msk, const double *__restrict__ A,
                                const double *__restrict__ x, const double *__restrict__ b,
                                double c1, double c2, int m, int n, double *__restrict__ t) {
    int i = 1 + blockIdx.x * MG_TX + threadIdx.x;
    int j = 1 + blockIdx.y * MG_TY + threadIdx.y;
    if (i > n - 2 || j > m - 2) return;
    size_t p = off(j, i, n);
    t[p] = jacobi_point(msk, A, (size_t)m * n, x, b, p, n, c1, c2);
}

// Second sweep: x = J(t) on rows/cols 2..m-3, plus the cells the Fortran's
// 3-row buffer writes back along the edges (fortran_multigrid.f90:92-95):
// column 1 (0-based) on rows 1..m-3 and column n-2 on rows 1..m-4 receive
// the first-sweep value.  Every other cell of x keeps its content.
__global__ void k_smooth_sweep2(const int8_t *__restrict__ msk, const double *__restrict__ A,
                                const double *__restrict__ t, const double *__restrict__ b,
                                double c1, double c2, int m, int n, double *__restrict__ x) {
    int i = 1 + blockIdx.x * MG_TX + threadIdx.x;
    int j = 1 + blockIdx.y * MG_TY + threadIdx.y;
    if (i > n - 2 || j > m - 2) return;
    size_t p = off(j, i, n);
    if (j >= 2 && j <= m - 3 && i >= 2 && i <= n - 3) {
        x[p] = jacobi_point(msk, A, (size_t)m * n, t, b, p, n, c1, c2);
    } else if (i == 1 && j <= m - 3) {
        x[p] = t[p];
    } else if (i == n - 2 && j <= m - 4) {
        x[p] = t[p];
    }
}

int launch_smoothtwice(const int8_t *msk, const double *A, double *x, const double *b,
                       double coef, int m, int n, double *tmp, cudaStream_t s) {
    if (m < 3 || n < 3) return OK;
    double c1 = coef;
    double c2 = 1. - c1;
    dim3 bl(MG_TX, MG_TY);
    dim3 g = grid2d(m - 2, n - 2, bl);
    k_smooth_sweep1<<<g, bl, 0, s>>>(msk, A, x, b, c1, c2, m, n, tmp);
    k_smooth_sweep2<<<g, bl, 0, s>>>(msk, A, tmp, b, c1, c2, m, n, x);
    return launch_status("smoothtwicewitha");
}

// smoothtridiag (core/gmg/fortran_multigrid.f90:215-317): factors into
// `work` (2 m n doubles), then one sweep
int launch_smoothtridiag(const int8_t *msk, const double *A, double *x, const double *b, int m,
                         int n, double *work, cudaStream_t s) {
    if (m < 8 || n < 3) return OK;  // no row in 3..m-5
    const size_t smem = tri_smem_bytes(m);
    if (smem > 220 * 1024) {
        set_error("smoothtridiag: %d rows exceed the shared-memory column buffers", m);
        return ERR_LIMIT;
    }
    AStored acc{A, (size_t)m * n, n};
    double *gam = work, *bet = work + (size_t)m * n;
    k_tri_factor<AStored><<<(n - 2 + 127) / 128, 128, 0, s>>>(msk, acc, gam, bet, m, n);
    int st = launch_status("smoothtridiag factor");
    if (st) return st;
    if (smem > 48 * 1024) {
        st = cuda_status(cudaFuncSetAttribute(k_tri_sweep<AStored>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem),
                         "smoothtridiag smem");
        if (st) return st;
    }
    k_tri_sweep<AStored><<<1, TRI_THREADS, smem, s>>>(msk, acc, x, b, gam, bet, m, n, nullptr);
    return launch_status("smoothtridiag");
}

// r = b - A x on rows/cols 1..m-2 (0-based), masked -> 0
// (core/gmg/fortran_multigrid.f90:338-359)
F2D_DEV double residual_point(const int8_t *msk, const double *A, size_t plane,
                              const double *x, const double *b, size_t p, int n) {
    if (msk[p] == 0) return 0.;
    const double *A1 = A, *A2 = A + plane, *A3 = A + 2 * plane, *A4 = A + 3 * plane,
                 *A5 = A + 4 * plane;
    return b[p]
        - A1[p] * x[p - n - 1]
        - A2[p] * x[p - n]
        - A3[p] * x[p - n + 1]
        - A4[p] * x[p - 1]
        - A5[p] * x[p]
        - A4[p + 1] * x[p + 1]
        - A3[p + n - 1] * x[p + n - 1]
        - A2[p + n] * x[p + n]
        - A1[p + n + 1] * x[p + n + 1];
}

__global__ void k_residual(const int8_t *__restrict__ msk, const double *__restrict__ A,
                           const double *__restrict__ x, const double *__restrict__ b,
                           int m, int n, double *__restrict__ r) {
    int i = 1 + blockIdx.x * MG_TX + threadIdx.x;
    int j = 1 + blockIdx.y * MG_TY + threadIdx.y;
    if (i > n - 2 || j > m - 2) return;
    size_t p = off(j, i, n);
    r[p] = residual_point(msk, A, (size_t)m * n, x, b, p, n);
}

int launch_residual(const int8_t *msk, const double *A, const double *x, const double *b,
                    double *r, int m, int n, cudaStream_t s) {
    if (m < 3 || n < 3) return OK;
    dim3 bl(MG_TX, MG_TY);
    k_residual<<<grid2d(m - 2, n - 2, bl), bl, 0, s>>>(msk, A, x, b, m, n, r);
    return launch_status("computeresidualwitha");
}

// Periodic wrap of the 8 halo blocks.  Thread q enumerates the halo cells:
// first the nh bottom and nh top rows (full width), then the left and right
// nh columns of the interior rows.  Every source is an interior cell, so
// the order of the copies does not matter.
__global__ void k_fillhalo(double *__restrict__ x, int nh, int m, int n, long long total) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= total) return;
    int j, i;
    long long band = 2LL * nh * n;
    if (q < band) {
        int r = (int)(q / n);
        i = (int)(q % n);
        j = r < nh ? r : m - 2 * nh + r;  // rows 0..nh-1, then m-nh..m-1
    } else {
        long long q2 = q - band;
        int r = (int)(q2 / (2 * nh));
        int c = (int)(q2 % (2 * nh));
        j = nh + r;
        i = c < nh ? c : n - 2 * nh + c;
    }
    x[off(j, i, n)] = x[off(wrap(j, m, nh), wrap(i, n, nh), n)];
}

int launch_fillhalo(double *x, int nh, int m, int n, cudaStream_t s) {
    if (nh <= 0) return OK;
    if (m < 2 * nh || n < 2 * nh) {
        set_error("fillhalo: (%d, %d) smaller than two halos", m, n);
        return ERR_SHAPE;
    }
    long long total = 2LL * nh * n + 2LL * nh * (m - 2 * nh);
    int threads = 256;
    long long blocks = (total + threads - 1) / threads;
    k_fillhalo<<<(unsigned)blocks, threads, 0, s>>>(x, nh, m, n, total);
    return launch_status("fillhalo");
}

// Full-weighting restriction (core/gmg/fortran_multigrid.f90:525-544):
// coarse (J2, I2), J2 in [nh-1, m2-nh-1], from fine (2*J2+1-nh, 2*I2+1-nh).
__global__ void k_restrict(const int8_t *__restrict__ msk2, const double *__restrict__ x1,
                           int nh, int m2, int n2, int n1, double *__restrict__ x2) {
    int I2 = nh - 1 + blockIdx.x * MG_TX + threadIdx.x;
    int J2 = nh - 1 + blockIdx.y * MG_TY + threadIdx.y;
    if (I2 > n2 - nh - 1 || J2 > m2 - nh - 1) return;
    size_t p2 = off(J2, I2, n2);
    if (msk2[p2] == 0) {
        x2[p2] = 0.;
        return;
    }
    size_t p = off(2 * J2 + 1 - nh, 2 * I2 + 1 - nh, n1);
    x2[p2] = 0.25 * x1[p]
        + 0.125 * (x1[p - 1] + x1[p + 1] + x1[p - n1] + x1[p + n1])
        + 0.0625 * (x1[p - n1 - 1] + x1[p - n1 + 1] + x1[p + n1 - 1] + x1[p + n1 + 1]);
}

int launch_restrict(const int8_t *msk2, const double *x1, int nh, int m2, int n2, int m1,
                    int n1, double *x2, cudaStream_t s) {
    if (m2 - 2 * nh + 1 <= 0 || n2 - 2 * nh + 1 <= 0) return OK;
    // the finest point read is fine row 2*(m2-nh-1)+1-nh+1
    if (2 * (m2 - nh - 1) + 2 - nh > m1 - 1 || 2 * (n2 - nh - 1) + 2 - nh > n1 - 1 || nh < 1) {
        set_error("restrict: coarse (%d, %d) does not fit fine (%d, %d)", m2, n2, m1, n1);
        return ERR_SHAPE;
    }
    dim3 bl(MG_TX, MG_TY);
    k_restrict<<<grid2d(m2 - 2 * nh + 1, n2 - 2 * nh + 1, bl), bl, 0, s>>>(msk2, x1, nh, m2, n2,
                                                                           n1, x2);
    return launch_status("restrict");
}

// Mask-aware bilinear prolongation (core/gmg/fortran_multigrid.f90:437-496):
// coarse (J2, I2), J2 in [1, m2-3], fills the 2x2 fine cells starting at
// (2*J2-2, 2*I2-2) for nh=3 (2*J2-1 for nh=2).  Fine cells outside the fine
// array (only possible when the arrays do not form a 2:1 pair) are skipped.
__global__ void k_interpolate(const int8_t *__restrict__ msk1, const int8_t *__restrict__ msk2,
                              const double *__restrict__ x2, int shift, int m2, int n2, int m1,
                              int n1, double *__restrict__ x1) {
    int I2 = 1 + blockIdx.x * MG_TX + threadIdx.x;
    int J2 = 1 + blockIdx.y * MG_TY + threadIdx.y;
    if (I2 > n2 - 3 || J2 > m2 - 3) return;
    // the weight tables as selects (an indexed local array lives in local memory)
    auto c2 = [](int k) { return k == 0 ? 0. : (k == 1 ? 1. : 0.5); };
    auto c3 = [](int k) {
        return k == 0 ? 0. : k == 1 ? 1. : k == 2 ? 0.5 : k == 3 ? r4(0.3333333333333333333333333333f)
                                                                 : 0.25;
    };
    int J1 = 2 * J2 - shift, I1 = 2 * I2 - shift;
    size_t q = off(J2, I2, n2);
    double a = x2[q], bx = x2[q + 1], by = x2[q + n2], bxy = x2[q + n2 + 1];
    int ma = msk2[q], mbx = msk2[q + 1], mby = msk2[q + n2], mbxy = msk2[q + n2 + 1];
    if (J1 < m1 && I1 < n1) {
        size_t p = off(J1, I1, n1);
        x1[p] = msk1[p] > 0 ? a : 0.;
    }
    if (J1 < m1 && I1 + 1 < n1) {
        size_t p = off(J1, I1 + 1, n1);
        x1[p] = msk1[p] > 0 ? (a + bx) * c2(ma + mbx) : 0.;
    }
    if (J1 + 1 < m1 && I1 < n1) {
        size_t p = off(J1 + 1, I1, n1);
        x1[p] = msk1[p] > 0 ? (a + by) * c2(ma + mby) : 0.;
    }
    if (J1 + 1 < m1 && I1 + 1 < n1) {
        size_t p = off(J1 + 1, I1 + 1, n1);
        x1[p] = msk1[p] > 0 ? c3(ma + mbx + mby + mbxy) * (a + bx + by + bxy) : 0.;
    }
}

int launch_interpolate(const int8_t *msk1, const int8_t *msk2, const double *x2, int nh,
                       int m2, int n2, int m1, int n1, double *x1, cudaStream_t s) {
    int shift;
    if (nh == 3) shift = 2;
    else if (nh == 2) shift = 1;
    else {
        set_error("interpolate: nh must be 2 or 3 (got %d)", nh);
        return ERR_NH;
    }
    if (m2 < 4 || n2 < 4) return OK;
    dim3 bl(MG_TX, MG_TY);
    k_interpolate<<<grid2d(m2 - 3, n2 - 3, bl), bl, 0, s>>>(msk1, msk2, x2, shift, m2, n2, m1,
                                                            n1, x1);
    return launch_status("interpolate");
}

// Galerkin coarse operator (core/gmg/fortran_multigrid.f90:735-808), one
// thread per coarse point, 9 outputs, same accumulation order.
__global__ void k_coarsenmatrix(const double *__restrict__ Af, const int8_t *__restrict__ msk1,
                                const int8_t *__restrict__ msk2, int nh, int m1, int n1, int m2,
                                int n2, double *__restrict__ Ac) {
    int I2 = nh - 1 + blockIdx.x * MG_TX + threadIdx.x;
    int J2 = nh - 1 + blockIdx.y * MG_TY + threadIdx.y;
    if (I2 > n2 - nh - 1 || J2 > m2 - nh - 1) return;
    const size_t pl1 = (size_t)m1 * n1, pl2 = (size_t)m2 * n2;
    const size_t p2 = off(J2, I2, n2);
    // coef(ki, kj) = 2 w(ki) w(kj), w = (1/4, 1/2, 1/4): the DATA statement values
    const double cw[3] = {0.125, 0.25, 0.125};
    const double cc[3] = {0.25, 0.5, 0.25};
#define COEF(ki, kj) ((kj) == 0 ? cc[(ki) + 1] : cw[(ki) + 1])
    if (msk2[p2] != 1) {
        for (int l = 0; l < 9; l++) Ac[l * pl2 + p2] = 0.;
        return;
    }
    // 1-based j2 = J2 + 1; i1 = 2*(i2-nh)+nh -> 0-based I1 = 2*(I2+1-nh)+nh-1
    const int I1 = 2 * (I2 + 1 - nh) + nh - 1, J1 = 2 * (J2 + 1 - nh) + nh - 1;
    for (int l = 1; l <= 9; l++) {
        int di2 = (l - 1) % 3 - 1, dj2 = (l - 1) / 3 - 1;
        double z5[5][5];
        for (int a = 0; a < 5; a++)
            for (int c = 0; c < 5; c++) z5[a][c] = 0.;
        for (int kj = -1; kj <= 1; kj++)
            for (int ki = -1; ki <= 1; ki++) {
                int i = 2 * di2 + ki, j = 2 * dj2 + kj;
                if (abs(i) <= 2 && abs(j) <= 2 && msk1[off(J1 + j, I1 + i, n1)] == 1)
                    z5[i + 2][j + 2] = 2. * COEF(ki, kj);
            }
        double z3[3][3];
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) z3[a][c] = 0.;
        for (int jj = -1; jj <= 1; jj++)
            for (int ii = -1; ii <= 1; ii++) {
                size_t pf = off(J1 + jj, I1 + ii, n1);
                if (msk1[pf] != 1) continue;
                double z = z3[ii + 1][jj + 1];
                for (int kj = -1; kj <= 1; kj++)
                    for (int ki = -1; ki <= 1; ki++) {
                        int k = (ki + 1) + (kj + 1) * 3;
                        z = z + Af[k * pl1 + pf] * z5[ii + ki + 2][jj + kj + 2];
                    }
                z3[ii + 1][jj + 1] = z;
            }
        double w = 0.;
        for (int jj = -1; jj <= 1; jj++)
            for (int ii = -1; ii <= 1; ii++) w = w + 0.5 * COEF(ii, jj) * z3[ii + 1][jj + 1];
        Ac[(l - 1) * pl2 + p2] = w;
    }
#undef COEF
}

int launch_coarsenmatrix(const double *Af, const int8_t *msk1, const int8_t *msk2, int nh,
                         int m1, int n1, int m2, int n2, double *Ac, cudaStream_t s) {
    if (m2 - 2 * nh + 1 <= 0 || n2 - 2 * nh + 1 <= 0) return OK;
    // finest fine cell touched: 0-based 2*(m2-2nh)+nh-1 (+2 for the stencil)
    int I1max = 2 * (n2 - 2 * nh) + nh - 1, J1max = 2 * (m2 - 2 * nh) + nh - 1;
    if (J1max + 2 > m1 - 1 || I1max + 2 > n1 - 1) {
        set_error("coarsenmatrix: coarse (%d, %d) does not fit fine (%d, %d)", m2, n2, m1, n1);
        return ERR_SHAPE;
    }
    dim3 bl(MG_TX, MG_TY);
    k_coarsenmatrix<<<grid2d(m2 - 2 * nh + 1, n2 - 2 * nh + 1, bl), bl, 0, s>>>(
        Af, msk1, msk2, nh, m1, n1, m2, n2, Ac);
    return launch_status("coarsenmatrix");
}

}  // namespace f2d
