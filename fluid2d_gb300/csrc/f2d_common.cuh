// f2d_common.cuh -- shared helpers of the fluid2d_gb300 CUDA kernels.
//
// Array convention (the reference's numpy/f2py layout): a field of the
// reference is a row-major (m, n) array, row j (y) and column i (x), both
// 0-based here.  The Fortran loop "do j=a,b" over 1-based rows becomes
// j in [a-1, b-1] over 0-based rows.  The halo is nh = 3 cells wide.
//
// Arithmetic: every kernel writes each expression in the reference's
// evaluation order.  The product build lets nvcc contract a*b+c into FMA;
// the exact build (-DF2D_EXACT together with -fmad=false) rounds every
// operation separately, so that its results can be compared bit for bit
// with the CPU oracle.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#define F2D_DEV __device__ __forceinline__
#define F2D_HD __host__ __device__ __forceinline__

namespace f2d {

// ---------------------------------------------------------------- status
enum Status {
    OK = 0,
    ERR_NH = 1,        // nh != 3 where the reference stops (fortran_advection.f90:30-34)
    ERR_SHAPE = 2,     // array dimensions the routine cannot handle
    ERR_ARG = 3,       // bad argument (null pointer, bad method/order, ...)
    ERR_CUDA = 4,      // a CUDA call failed
    ERR_DIVERGED = 5,  // multigrid not converging (core/gmg/hierarchy.py:182-188)
    ERR_LIMIT = 6,     // a size beyond a fixed capacity of the library
};

void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *where);
int launch_status(const char *where);

// REAL*4 literals of the Fortran source, widened to REAL*8
F2D_HD double r4(float x) { return (double)x; }

// 1-based Fortran (j, i) -> 0-based row-major offset
F2D_HD size_t off(int j, int i, int n) { return (size_t)j * (size_t)n + (size_t)i; }

// periodic image of a halo index (core/gmg/fortran_multigrid.f90:365-412):
// indices [0, nh) map to [len-2nh, len-nh), [len-nh, len) to [nh, 2nh)
F2D_HD int wrap(int k, int len, int nh) {
    const int inner = len - 2 * nh;
    if (k < nh) return k + inner;
    if (k >= len - nh) return k - inner;
    return k;
}

inline dim3 grid2d(int rows, int cols, dim3 block) {
    return dim3((unsigned)((cols + (int)block.x - 1) / (int)block.x),
                (unsigned)((rows + (int)block.y - 1) / (int)block.y), 1);
}

// ---------------------------------------------------------------- reductions
// Deterministic two-level reductions: every block reduces a fixed set of
// rows in a fixed order, then one block reduces the per-block partials in
// block order.  The result depends only on (m, n), never on scheduling.
constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 1024;
constexpr int RED_MAX_VALUES = 4;

int reduce_blocks(int rows);
// device workspace of at least RED_MAX_BLOCKS * RED_MAX_VALUES doubles,
// owned by the library (one per device, allocated on first use)
double *reduce_workspace(int *status);

template <int NV>
F2D_DEV void block_reduce(double (&v)[NV], const bool (&is_max)[NV], double *sh) {
    // sh: NV * RED_THREADS doubles; fixed pairwise tree over the threads
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NV; k++) sh[k * RED_THREADS + t] = v[k];
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (t < s) {
#pragma unroll
            for (int k = 0; k < NV; k++) {
                double a = sh[k * RED_THREADS + t], b = sh[k * RED_THREADS + t + s];
                sh[k * RED_THREADS + t] = is_max[k] ? (a > b ? a : b) : a + b;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = sh[k * RED_THREADS];
}

}  // namespace f2d
