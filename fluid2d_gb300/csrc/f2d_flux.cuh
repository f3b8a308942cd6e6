// f2d_flux.cuh -- element kernels of the flux diagnostic (core/fluxes.py).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace f2d {

// uc = 0.5 (u + roll(u, 1, axis=1)), vc = 0.5 (v + roll(v, 1, axis=0)) over
// the whole array (core/fluxes.py:123-132); the caller fills the halos
int flux_centre(const double *u, const double *v, double *uc, double *vc, int mv, int nv,
                cudaStream_t s);
// x *= msk over the whole array (numpy `y *= self.msk`, int8 -> float64)
int mul_mask(double *x, const int8_t *msk, size_t n, cudaStream_t s);
// X[:ns] = Xe with the planes of `negmask` (bit k = plane k) negated,
// X[ns:next] = 0 (core/fluxes.py:135-152)
int flux_load(double *X, const double *Xe, int ns, int next, size_t pl, unsigned negmask,
              cudaStream_t s);
// RK3_SSP combinations over the extended state (core/timescheme.py:167-180)
// with dtv = sgn * dt:  mode 0: S = X + dtv D0;  mode 1: S = X + (0.25 dtv)(D0 + D1);
// mode 2: X += (dtv / 6)(D0 + D1 + 4 D2)
int flux_rk(int mode, size_t n, double *X, const double *D0, const double *D1,
            const double *D2, double *S, const double *dt, double sgn, cudaStream_t s);
// rev/irr fluxes (core/fluxes.py:154-170) from the forward (Xw) and the
// backward (X) integrations of the flux planes
int flux_final(int nflx, int ns, size_t pl, const double *Xw, const double *X, double *FLX,
               const double *dt, cudaStream_t s);
// cst of the flux advection: [dx, dy, 0.05, cst[3] of the model, aparab]
int flux_cst(double *fcst, const double *cst, double dx, double dy, double aparab,
             cudaStream_t s);

}  // namespace f2d
