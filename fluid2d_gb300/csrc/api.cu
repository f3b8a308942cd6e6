// api.cu -- extern "C" entry points of the per-routine kernels, error state
// and the library-owned device scratch.
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/fluid2d_gb300.h"
#include "f2d_common.cuh"
#include "f2d_kernels.cuh"
#include "f2d_walls.cuh"

namespace f2d {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return OK;
    set_error("%s: %s", where, cudaGetErrorString(e));
    // clear a non-sticky error so that it is not reported again by the next
    // launch check of an unrelated kernel
    cudaGetLastError();
    return ERR_CUDA;
}

int launch_status(const char *where) { return cuda_status(cudaGetLastError(), where); }

// One growable device scratch per device and purpose.
struct Scratch {
    void *ptr = nullptr;
    size_t bytes = 0;
};
static std::mutex g_scratch_mu;
static std::vector<Scratch> g_scratch[2];  // [0] general, [1] reduction partials

static void *device_scratch(int which, size_t bytes, int *status) {
    int dev = 0;
    *status = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (*status) return nullptr;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    auto &v = g_scratch[which];
    if ((int)v.size() <= dev) v.resize(dev + 1);
    Scratch &s = v[dev];
    if (s.bytes < bytes) {
        // the old buffer may still be in use by queued work on some stream
        if (s.ptr) {
            *status = cuda_status(cudaDeviceSynchronize(), "scratch grow sync");
            if (*status) return nullptr;
            cudaFree(s.ptr);
            s.ptr = nullptr;
            s.bytes = 0;
        }
        size_t nb = bytes + bytes / 4 + 4096;
        *status = cuda_status(cudaMalloc(&s.ptr, nb), "scratch cudaMalloc");
        if (*status) return nullptr;
        s.bytes = nb;
    }
    return s.ptr;
}

void *scratch_buffer(size_t bytes, int *status) { return device_scratch(0, bytes, status); }

double *reduce_workspace(int *status) {
    return (double *)device_scratch(1, sizeof(double) * RED_MAX_BLOCKS * RED_MAX_VALUES, status);
}

}  // namespace f2d

using namespace f2d;

#define STREAM(s) ((cudaStream_t)(s))

extern "C" {

int f2d_version(void) { return 100; }

const char *f2d_last_error(void) { return g_err; }

int f2d_exact_arithmetic(void) {
#ifdef F2D_EXACT
    return 1;
#else
    return 0;
#endif
}

int f2d_adv_upwind(const int8_t *msk, const double *x, double *y, const double *u,
                   const double *v, const double *cst, int nh, int method, int order, int m,
                   int n, void *stream) {
    return launch_advection(0, msk, x, y, u, v, nullptr, nullptr, cst, nh, method, order, m, n,
                            STREAM(stream));
}

int f2d_adv_centered(const int8_t *msk, const double *x, double *y, const double *u,
                     const double *v, const double *cst, int nh, int method, int order, int m,
                     int n, void *stream) {
    return launch_advection(1, msk, x, y, u, v, nullptr, nullptr, cst, nh, method, order, m, n,
                            STREAM(stream));
}

int f2d_flx_adv_upwind(const int8_t *msk, const double *x, double *y, const double *u,
                       const double *v, double *xflx, double *yflx, const double *cst, int nh,
                       int method, int order, int m, int n, void *stream) {
    if (!xflx || !yflx) {
        set_error("flux outputs must not be null");
        return ERR_ARG;
    }
    return launch_advection(0, msk, x, y, u, v, xflx, yflx, cst, nh, method, order, m, n,
                            STREAM(stream));
}

int f2d_flx_adv_centered(const int8_t *msk, const double *x, double *y, const double *u,
                         const double *v, double *xflx, double *yflx, const double *cst,
                         int nh, int method, int order, int m, int n, void *stream) {
    if (!xflx || !yflx) {
        set_error("flux outputs must not be null");
        return ERR_ARG;
    }
    return launch_advection(2, msk, x, y, u, v, xflx, yflx, cst, nh, method, order, m, n,
                            STREAM(stream));
}

int f2d_computeorthogradient(const int8_t *msk, const double *psi, double dx, double dy,
                             int nh, int m, int n, double *u, double *v, void *stream) {
    (void)nh;
    return launch_orthogradient(msk, psi, dx, dy, m, n, u, v, STREAM(stream));
}

int f2d_celltocorner(const double *xr, double *xp, int m, int n, void *stream) {
    return launch_celltocorner(xr, xp, m, n, STREAM(stream));
}

int f2d_cornertocell(const double *xp, double *xr, int m, int n, void *stream) {
    return launch_cornertocell(xp, xr, m, n, STREAM(stream));
}

int f2d_add_diffusion(const int8_t *msk, const double *trac, double dx, int nh, double Kdiff,
                      double *dtrac, int m, int n, void *stream) {
    (void)nh;
    return launch_add_diffusion(msk, trac, dx, Kdiff, dtrac, m, n, STREAM(stream));
}

int f2d_add_torque(const int8_t *msk, const double *buoy, double dx, int nh, double gravity,
                   double *domega, int m, int n, void *stream) {
    return launch_add_torque(msk, buoy, dx, nh, gravity, domega, m, n, STREAM(stream));
}

int f2d_computenoslipsourceterm(const int8_t *msk, const double *x, double *y, double dx,
                                double dy, int nh, int m, int n, double *total, void *stream) {
    return launch_noslip_dropin(msk, x, y, dx, dy, nh, m, n, total, STREAM(stream));
}

// reduction kinds, see kernels_ops.cu
int f2d_computedotprod(const int8_t *msk, const double *x, const double *y, int nh, int m,
                       int n, double *out, void *stream) {
    return launch_reduce(0, msk, x, y, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computemax(const int8_t *msk, const double *x, int nh, int m, int n, double *out,
                   void *stream) {
    return launch_reduce(1, msk, x, nullptr, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computesum(const int8_t *msk, const double *x, int nh, int m, int n, double *out,
                   void *stream) {
    return launch_reduce(2, msk, x, nullptr, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computesumandnorm(const int8_t *msk, const double *x, int nh, int m, int n,
                          double *out, void *stream) {
    return launch_reduce(3, msk, x, nullptr, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computenormmaxu(const int8_t *msk, const double *x, int nh, int m, int n, double *out,
                        void *stream) {
    return launch_reduce(4, msk, x, nullptr, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computekemaxu(const int8_t *msk, const double *u, const double *v, int nh, int m,
                      int n, double *out, void *stream) {
    if (!v) {
        set_error("computekemaxu: null v");
        return ERR_ARG;
    }
    return launch_reduce(5, msk, u, v, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computekemaxuv(const int8_t *msk, const double *u, const double *v, int nh, int m,
                       int n, double *out, void *stream) {
    if (!v) {
        set_error("computekemaxuv: null v");
        return ERR_ARG;
    }
    return launch_reduce(6, msk, u, v, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computekewithpsi(const int8_t *msk, const double *omega, const double *psi, int nh,
                         int m, int n, double *out, void *stream) {
    if (!psi) {
        set_error("computekewithpsi: null psi");
        return ERR_ARG;
    }
    return launch_reduce(7, msk, omega, psi, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computenorm(const int8_t *msk, const double *x, int nh, int m, int n, double *out,
                    void *stream) {
    return launch_reduce(8, msk, x, nullptr, nh, m, n, out, nullptr, STREAM(stream));
}
int f2d_computeinner(const int8_t *msk, const double *x, const double *y, int nh, int m, int n,
                     double *out, void *stream) {
    if (!y) {
        set_error("computeinner: null y");
        return ERR_ARG;
    }
    return launch_reduce(0, msk, x, y, nh, m, n, out, nullptr, STREAM(stream));
}

int f2d_smoothtwicewitha(const int8_t *msk, const double *A, double *x, const double *b,
                         double coef, int m, int n, void *stream) {
    if (!msk || !A || !x || !b) {
        set_error("smoothtwicewitha: null pointer");
        return ERR_ARG;
    }
    int st = OK;
    double *tmp = (double *)scratch_buffer(sizeof(double) * (size_t)m * n, &st);
    if (st) return st;
    return launch_smoothtwice(msk, A, x, b, coef, m, n, tmp, STREAM(stream));
}

int f2d_smoothtridiag(const int8_t *msk, const double *A, double *x, const double *b, int m,
                      int n, void *stream) {
    if (!msk || !A || !x || !b) {
        set_error("smoothtridiag: null pointer");
        return ERR_ARG;
    }
    int st = OK;
    double *work = (double *)scratch_buffer(2 * sizeof(double) * (size_t)m * n, &st);
    if (st) return st;
    return launch_smoothtridiag(msk, A, x, b, m, n, work, STREAM(stream));
}

int f2d_computeresidualwitha(const int8_t *msk, const double *A, const double *x,
                             const double *b, double *y, int m, int n, void *stream) {
    if (!msk || !A || !x || !b || !y) {
        set_error("computeresidualwitha: null pointer");
        return ERR_ARG;
    }
    return launch_residual(msk, A, x, b, y, m, n, STREAM(stream));
}

int f2d_fillhalo(double *x, int nh, int m, int n, void *stream) {
    return launch_fillhalo(x, nh, m, n, STREAM(stream));
}

int f2d_interpolate(const int8_t *msk1, const int8_t *msk2, const double *x2, int nh, int m2,
                    int n2, int m1, int n1, double *x1, void *stream) {
    return launch_interpolate(msk1, msk2, x2, nh, m2, n2, m1, n1, x1, STREAM(stream));
}

int f2d_restrict(const int8_t *msk2, const double *x1, int nh, int m2, int n2, int m1, int n1,
                 double *x2, void *stream) {
    return launch_restrict(msk2, x1, nh, m2, n2, m1, n1, x2, STREAM(stream));
}

int f2d_coarsenmatrix(const double *Afine, const int8_t *msk1, const int8_t *msk2, int nh,
                      int m1, int n1, int m2, int n2, double *Acoarse, void *stream) {
    return launch_coarsenmatrix(Afine, msk1, msk2, nh, m1, n1, m2, n2, Acoarse, STREAM(stream));
}

}  // extern "C"
