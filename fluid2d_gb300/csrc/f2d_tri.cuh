// f2d_tri.cuh -- the vertical line relaxation smoothtridiag
// (core/gmg/fortran_multigrid.f90:215-317), shared by the drop-in entry point
// and the engine.
//
// One sweep visits the columns i = 1..n-2 in order (Gauss-Seidel across
// columns: column i reads column i-1 as this sweep left it) and solves, on
// each column whose row 3 is fluid, the tridiagonal system of its rows
// 3..m-5 by the Thomas algorithm.  The elimination factors (gam, bet) depend
// on the operator only, so they are computed once per level (tri_factor,
// one thread per column, the Fortran's operations in its order); a sweep is
// one CTA that forms a column's right-hand side in parallel and runs the
// two recurrences on one thread, from shared memory.
//
// The operator is read through an accessor A(k, j, i), k = 0..4 for the
// reference's planes A(j,i,1..5).
#pragma once
#include "f2d_common.cuh"

namespace f2d {

constexpr int TRI_THREADS = 256;
// five shared arrays of m doubles
inline size_t tri_smem_bytes(int mv) { return sizeof(double) * 5 * (size_t)mv; }

template <typename Acc>
__global__ void k_tri_factor(const int8_t *msk, Acc A, double *gam, double *bet, int mv, int nv) {
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i > nv - 2 || msk[off(3, i, nv)] == 0) return;
    // d(j) = A(j,i,5), dd(j) = ud(j) = A(j+1,i,2)
    double b = 1. / A(4, 3, i);
    bet[off(3, i, nv)] = b;
    for (int k = 4; k <= mv - 5; k++) {
        const double dd = A(1, k, i);
        const double g = dd * b;
        gam[off(k, i, nv)] = g;
        b = 1. / (A(4, k, i) - dd * g);
        bet[off(k, i, nv)] = b;
    }
}

template <typename Acc>
__global__ void __launch_bounds__(TRI_THREADS)
    k_tri_sweep(const int8_t *msk, Acc A, double *x, const double *rhsb, const double *gam,
                const double *bet, int mv, int nv, const int *active) {
    if (active && *active == 0) return;
    extern __shared__ __align__(16) unsigned char tri_sm[];
    double *rhs = (double *)tri_sm;
    double *xc = rhs + mv;
    double *sg = xc + mv;
    double *sb = sg + mv;
    double *sd = sb + mv;
    const int tid = threadIdx.x;
    for (int i = 1; i <= nv - 2; i++) {
        if (msk[off(3, i, nv)] == 0) continue;
        for (int j = 3 + tid; j <= mv - 5; j += TRI_THREADS) {
            const size_t p = off(j, i, nv);
            // y = b - A x without the column's own (vertical) couplings
            rhs[j] = rhsb[p] - A(0, j, i) * x[p - nv - 1] - A(2, j, i) * x[p - nv + 1] -
                     A(3, j, i) * x[p - 1] - A(3, j, i + 1) * x[p + 1] -
                     A(2, j + 1, i - 1) * x[p + nv - 1] - A(0, j + 1, i + 1) * x[p + nv + 1];
            sg[j] = gam[p];
            sb[j] = bet[p];
            sd[j] = A(1, j + 1, i);
        }
        __syncthreads();
        if (tid == 0) {
            double c = rhs[3] * sb[3];
            xc[3] = c;
            for (int k = 4; k <= mv - 5; k++) {
                c = (rhs[k] - sd[k - 1] * c) * sb[k];
                xc[k] = c;
            }
            for (int k = mv - 6; k >= 3; k--) {
                c = xc[k] - sg[k + 1] * c;
                xc[k] = c;
            }
        }
        __syncthreads();
        for (int j = 3 + tid; j <= mv - 5; j += TRI_THREADS) x[off(j, i, nv)] = xc[j];
        __syncthreads();
    }
}

// the reference's stored operator: 5 (or more) planes of m*n values
struct AStored {
    const double *A;
    size_t pl;
    int nv;
    F2D_DEV double operator()(int k, int j, int i) const { return A[k * pl + off(j, i, nv)]; }
};

}  // namespace f2d
