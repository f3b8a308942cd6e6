// fluxdiag.cu -- element kernels of the flux diagnostic of core/fluxes.py.
//
// The diagnostic itself (two RK3 integrations of an extended state made of
// the model state, the cell-centred velocities and the edge fluxes of every
// tracer) is sequenced in engine.cu with the per-routine advection, torque,
// halo and multigrid kernels; these kernels are its elementwise parts, with
// numpy's evaluation order.
#include "f2d_common.cuh"
#include "f2d_flux.cuh"
#include "f2d_kernels.cuh"

namespace f2d {

static unsigned grid_for(size_t n) {
    size_t b = (n + 255) / 256;
    return (unsigned)(b > 8192 ? 8192 : (b ? b : 1));
}

__global__ void k_flux_centre(const double *u, const double *v, double *uc, double *vc, int mv,
                              int nv) {
    const size_t n = (size_t)mv * nv;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(q / nv), i = (int)(q - (size_t)j * nv);
        const int iw = i == 0 ? nv - 1 : i - 1;
        const int js = j == 0 ? mv - 1 : j - 1;
        uc[q] = 0.5 * (u[q] + u[(size_t)j * nv + iw]);
        vc[q] = 0.5 * (v[q] + v[(size_t)js * nv + i]);
    }
}

int flux_centre(const double *u, const double *v, double *uc, double *vc, int mv, int nv,
                cudaStream_t s) {
    k_flux_centre<<<grid_for((size_t)mv * nv), 256, 0, s>>>(u, v, uc, vc, mv, nv);
    return launch_status("flux_centre");
}

__global__ void k_mul_mask(double *x, const int8_t *msk, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        x[q] = x[q] * (double)msk[q];
}

int mul_mask(double *x, const int8_t *msk, size_t n, cudaStream_t s) {
    k_mul_mask<<<grid_for(n), 256, 0, s>>>(x, msk, n);
    return launch_status("mul_mask");
}

__global__ void k_flux_load(double *X, const double *Xe, int ns, int next, size_t pl,
                            unsigned negmask) {
    const size_t n = (size_t)next * pl;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(q / pl);
        if (k < ns)
            X[q] = ((negmask >> k) & 1u) ? -Xe[q] : Xe[q];
        else
            X[q] = 0.;
    }
}

int flux_load(double *X, const double *Xe, int ns, int next, size_t pl, unsigned negmask,
              cudaStream_t s) {
    k_flux_load<<<grid_for((size_t)next * pl), 256, 0, s>>>(X, Xe, ns, next, pl, negmask);
    return launch_status("flux_load");
}

__global__ void k_flux_rk(int mode, size_t n, double *X, const double *D0, const double *D1,
                          const double *D2, double *S, const double *dt, double sgn) {
    const double dtv = sgn * *dt;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        if (mode == 0) {
            S[q] = X[q] + dtv * D0[q];
        } else if (mode == 1) {
            S[q] = X[q] + (0.25 * dtv) * (D0[q] + D1[q]);
        } else {
            X[q] = X[q] + (dtv / 6.) * ((D0[q] + D1[q]) + 4. * D2[q]);
        }
    }
}

int flux_rk(int mode, size_t n, double *X, const double *D0, const double *D1,
            const double *D2, double *S, const double *dt, double sgn, cudaStream_t s) {
    k_flux_rk<<<grid_for(n), 256, 0, s>>>(mode, n, X, D0, D1, D2, S, dt, sgn);
    return launch_status("flux_rk");
}

__global__ void k_flux_final(int nflx, int ns, size_t pl, const double *Xw, const double *X,
                             double *FLX, const double *dt) {
    const double cff = 0.5 / *dt;
    const size_t n = (size_t)nflx * pl;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(q / pl);
        const size_t p = q - (size_t)k * pl;
        const size_t l = (size_t)(ns + k) * pl + p;
        // vorticity (k = 0, 1), uc and vc (the last four) change sign when time
        // is reversed; buoyancy does not
        const bool odd = (k < 2) || (k >= nflx - 4);
        const double sx = odd ? -X[l] : X[l];
        FLX[q] = cff * (Xw[l] + sx);
        FLX[(size_t)(nflx + k) * pl + p] = cff * (Xw[l] - sx);
    }
}

int flux_final(int nflx, int ns, size_t pl, const double *Xw, const double *X, double *FLX,
               const double *dt, cudaStream_t s) {
    k_flux_final<<<grid_for((size_t)nflx * pl), 256, 0, s>>>(nflx, ns, pl, Xw, X, FLX, dt);
    return launch_status("flux_final");
}

__global__ void k_flux_cst(double *fcst, const double *cst, double dx, double dy,
                           double aparab) {
    fcst[0] = dx;
    fcst[1] = dy;
    fcst[2] = 0.05;
    fcst[3] = cst[3];
    fcst[4] = aparab;
}

int flux_cst(double *fcst, const double *cst, double dx, double dy, double aparab,
             cudaStream_t s) {
    k_flux_cst<<<1, 1, 0, s>>>(fcst, cst, dx, dy, aparab);
    return launch_status("flux_cst");
}

}  // namespace f2d
