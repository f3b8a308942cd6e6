// f2d_kernels.cuh -- launchers of the per-routine kernels (internal).
#pragma once
#include "f2d_common.cuh"

namespace f2d {

int launch_advection(int kind, const int8_t *msk, const double *x, double *y, const double *u,
                     const double *v, double *xflx, double *yflx, const double *cst, int nh,
                     int method, int order, int m, int n, cudaStream_t s);
int launch_orthogradient(const int8_t *msk, const double *psi, double dx, double dy, int m, int n,
                         double *u, double *v, cudaStream_t s);
int launch_celltocorner(const double *xr, double *xp, int m, int n, cudaStream_t s);
int launch_cornertocell(const double *xp, double *xr, int m, int n, cudaStream_t s);
int launch_add_diffusion(const int8_t *msk, const double *trac, double dx, double Kdiff,
                         double *dtrac, int m, int n, cudaStream_t s);
int launch_add_torque(const int8_t *msk, const double *b, double dx, int nh, double gravity,
                      double *w, int m, int n, cudaStream_t s);
int launch_reduce(int kind, const int8_t *msk, const double *x, const double *y, int nh, int m,
                  int n, double *out, double *work, cudaStream_t s);
int launch_smoothtwice(const int8_t *msk, const double *A, double *x, const double *b,
                       double coef, int m, int n, double *tmp, cudaStream_t s);
int launch_smoothtridiag(const int8_t *msk, const double *A, double *x, const double *b, int m,
                         int n, double *work, cudaStream_t s);
int launch_residual(const int8_t *msk, const double *A, const double *x, const double *b,
                    double *r, int m, int n, cudaStream_t s);
int launch_fillhalo(double *x, int nh, int m, int n, cudaStream_t s);
int launch_restrict(const int8_t *msk2, const double *x1, int nh, int m2, int n2, int m1, int n1,
                    double *x2, cudaStream_t s);
int launch_interpolate(const int8_t *msk1, const int8_t *msk2, const double *x2, int nh, int m2,
                       int n2, int m1, int n1, double *x1, cudaStream_t s);
int launch_coarsenmatrix(const double *Af, const int8_t *msk1, const int8_t *msk2, int nh, int m1,
                         int n1, int m2, int n2, double *Ac, cudaStream_t s);

// scratch array of at least `bytes` bytes, owned by the library (one per
// device, grown on demand); calls that share it must not overlap on the GPU
void *scratch_buffer(size_t bytes, int *status);

}  // namespace f2d
