// noalloc.cu -- an allocation-free variant of smoothtwicewitha.
//
// f2d_smoothtwicewitha needs a work array as large as the grid (the first
// Jacobi sweep is written there before the second one reads it).  It gets
// that array from the library, which calls cudaMalloc the first time and
// again, after a device-wide synchronisation and cudaFree, whenever a
// larger grid comes along.  Some callers cannot let that happen: programs
// whose device memory is handed out by their own allocator or a fixed
// budget, and programs that may not synchronise the whole device or call
// cudaMalloc/cudaFree at the point where they smooth.  For them,
// f2d_smoothtwicewitha_noalloc takes its work array from a fixed
// statically allocated device buffer instead and never allocates.
//
// The buffer, NOALLOC_SCRATCH_DOUBLES float64 values (16 MiB), is part of
// the library's device image: every GPU on which the library is used holds
// it until the process exits.  Grids with m*n above that are rejected.
#include <mutex>

#include "../../include/fluid2d_gb300.h"
#include "f2d_common.cuh"
#include "f2d_kernels.cuh"

namespace f2d {

constexpr size_t NOALLOC_SCRATCH_DOUBLES = (size_t)2 << 20;  // 2^21 doubles = 16 MiB

// The work array.  In host code this name is only a host-side stand-in for
// the device variable: the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
double *g_scratch_ptr[MAX_DEVICES] = {};

// Device address of the work array on the current device, looked up once
// per device (the lookup is the only set-up; it allocates nothing).
int scratch_address(double **out) {
    int dev = 0;
    int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    if (dev < 0 || dev >= MAX_DEVICES) {
        set_error("smoothtwicewitha_noalloc: device index %d beyond %d", dev, MAX_DEVICES);
        return ERR_LIMIT;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                         "cudaGetSymbolAddress(g_noalloc_scratch)");
        if (st) return st;
        g_scratch_ptr[dev] = (double *)p;
    }
    *out = g_scratch_ptr[dev];
    return OK;
}
}  // namespace

}  // namespace f2d

using namespace f2d;

extern "C" int f2d_smoothtwicewitha_noalloc(const int8_t *msk, const double *A, double *x,
                                            const double *b, double coef, int m, int n,
                                            void *stream) {
    if (!msk || !A || !x || !b) {
        set_error("smoothtwicewitha_noalloc: null pointer");
        return ERR_ARG;
    }
    if (m < 0 || n < 0 || (size_t)m * (size_t)n > NOALLOC_SCRATCH_DOUBLES) {
        set_error("smoothtwicewitha_noalloc: grid %d x %d = %zu points exceeds the fixed work "
                  "array of %zu points; use f2d_smoothtwicewitha",
                  m, n, (size_t)(m < 0 ? 0 : m) * (size_t)(n < 0 ? 0 : n),
                  NOALLOC_SCRATCH_DOUBLES);
        return ERR_LIMIT;
    }
    double *tmp = nullptr;
    int st = scratch_address(&tmp);
    if (st) return st;
    // The first sweep writes every work cell the second sweep reads, so the
    // previous call's contents never leak into this one; nothing needs
    // clearing.
    return launch_smoothtwice(msk, A, x, b, coef, m, n, tmp, (cudaStream_t)stream);
}
