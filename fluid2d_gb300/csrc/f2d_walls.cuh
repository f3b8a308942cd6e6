// f2d_walls.cuh -- no-slip source kernels (core/operators.py:245-290).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace f2d {

// computenoslipsourceterm (core/fortran_operators.f90:221-277) on the
// interior cells; the halo is filled by the caller
int noslip_source(const int8_t *msknoslip, const double *psi, double *src, double dx, double dy,
                  int mv, int nv, cudaStream_t s);
// the f2py routine on a caller array: every cell its loop writes, and its
// intent(out) total (to the device double *total, skipped when null)
int launch_noslip_dropin(const int8_t *msk, const double *x, double *y, double dx, double dy,
                         int nh, int m, int n, double *total, cudaStream_t s);
// src -= (sum[0]/bcarea)*mskbc over the whole array
int noslip_mean(double *src, const double *sum, const int8_t *mskbc, double bcarea, size_t n,
                cudaStream_t s);
int plane_sub(double *x, const double *y, size_t n, cudaStream_t s);
int plane_div(double *x, const double *dt, size_t n, cudaStream_t s);
// psi = psi*mskp + psi_island (the islands' streamfunction)
int psi_island(double *psi, const int8_t *mskp, const double *isl, size_t n, cudaStream_t s);
// QG: pvanom += (dt/6)(d0 + d1) with the pv tendencies of stages 0 and 1
// (float64 d0/d1, or float32 f0/f1 in the mixed form)
int pvanom_rk(double *x, const double *d0, const double *d1, const float *f0, const float *f1,
              const double *dt, size_t n, cudaStream_t s);

}  // namespace f2d
