// kernels_walls.cu -- the no-slip vorticity source along the walls.
//
// core/operators.py:245-290 (rhs_noslip) with the source term of
// core/fortran_operators.f90:221-277 (computenoslipsourceterm).  The Fortran
// loop scatters each wall edge's contribution into the fluid cell beside it
// as it sweeps the grid row by row; here every interior cell gathers the
// contributions it receives, in the order the sweep adds them: its own edges
// (west, then south) first, then the one from its east neighbour, then the
// one from its north neighbour.
#include "f2d_common.cuh"
#include "f2d_fused.cuh"
#include "f2d_kernels.cuh"
#include "f2d_walls.cuh"

namespace f2d {

// the tangential velocity at the west edge of (j, i) (core/fortran_operators.f90:240-246)
F2D_DEV double edge_v(const double *x, size_t p, int nv, double cff) {
    return (x[p] + x[p - nv] - x[p - 2] - x[p - nv - 2]) * cff;
}
// the tangential velocity at the south edge of (j, i) (core/fortran_operators.f90:254-260)
F2D_DEV double edge_u(const double *x, size_t p, int nv, double cff) {
    return -(x[p] + x[p - 1] - x[p - 2 * nv] - x[p - 2 * nv - 1]) * cff;
}

__global__ void k_noslip_source(const int8_t *m, const double *psi, double *src, double cff,
                                int mv, int nv) {
    const int i = NH + blockIdx.x * 32 + threadIdx.x;
    const int j = NH + blockIdx.y * 8 + threadIdx.y;
    if (i > nv - NH - 1 || j > mv - NH - 1) return;
    const size_t p = off(j, i, nv);
    double y = 0.;
    const int mc = m[p];
    if (mc != 0) {  // its own west and south wall edges
        if (m[p - 1] + mc == 1) y = y - edge_v(psi, p, nv, cff);
        if (m[p - nv] + mc == 1) y = y + edge_u(psi, p, nv, cff);
    }
    // a solid east neighbour hands its west-edge term to this cell
    if (m[p + 1] == 0 && mc + m[p + 1] == 1) y = y + edge_v(psi, p + 1, nv, cff);
    // a solid north neighbour hands its south-edge term to this cell
    if (m[p + nv] == 0 && mc + m[p + nv] == 1) y = y - edge_u(psi, p + nv, nv, cff);
    src[p] = y;
}

int noslip_source(const int8_t *msknoslip, const double *psi, double *src, double dx, double dy,
                  int mv, int nv, cudaStream_t s) {
    dim3 b(32, 8);
    const double cff = 1. / (2 * dx * dy);
    k_noslip_source<<<grid2d(mv - 2 * NH, nv - 2 * NH, b), b, 0, s>>>(msknoslip, psi, src, cff,
                                                                        mv, nv);
    return launch_status("noslip_source");
}

// source -= (sum/bcarea)*mskbc over the whole array
__global__ void k_noslip_mean(double *src, const double *sum, const int8_t *mskbc, double bcarea,
                              size_t n) {
    const double mean = sum[0] / bcarea;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        src[q] = src[q] - mean * (double)mskbc[q];
}

int noslip_mean(double *src, const double *sum, const int8_t *mskbc, double bcarea, size_t n,
                cudaStream_t s) {
    size_t b = (n + 255) / 256;
    k_noslip_mean<<<(unsigned)(b > 4096 ? 4096 : b), 256, 0, s>>>(src, sum, mskbc, bcarea, n);
    return launch_status("noslip_mean");
}

// x -= y, or x /= *dt (div != null), over the whole array
__global__ void k_plane_update(double *x, const double *y, const double *div, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        x[q] = div ? x[q] / *div : x[q] - y[q];
}

int plane_sub(double *x, const double *y, size_t n, cudaStream_t s) {
    size_t b = (n + 255) / 256;
    k_plane_update<<<(unsigned)(b > 4096 ? 4096 : b), 256, 0, s>>>(x, y, nullptr, n);
    return launch_status("plane_sub");
}

int plane_div(double *x, const double *dt, size_t n, cudaStream_t s) {
    size_t b = (n + 255) / 256;
    k_plane_update<<<(unsigned)(b > 4096 ? 4096 : b), 256, 0, s>>>(x, nullptr, dt, n);
    return launch_status("plane_div");
}

// psi = psi*mskp + psi_island over the whole array (core/operators.py:481-486)
__global__ void k_psi_island(double *psi, const int8_t *mskp, const double *isl, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        psi[q] = psi[q] * (double)mskp[q] + isl[q];
}

int psi_island(double *psi, const int8_t *mskp, const double *isl, size_t n, cudaStream_t s) {
    size_t b = (n + 255) / 256;
    k_psi_island<<<(unsigned)(b > 4096 ? 4096 : b), 256, 0, s>>>(psi, mskp, isl, n);
    return launch_status("psi_island");
}

// QG: the RK update of the pvanom plane that the wall source reads
// (core/timescheme.py:180 over dxdt[pvanom] = dxdt[pv] at stages 0, 1 and 0 at
// the forcing stage, core/quasigeostrophic.py:158-168)
template <typename D>
__global__ void k_pvanom_rk(double *x, const D *d0, const D *d1, const double *dt, size_t n) {
    const double c = *dt / 6.;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        x[q] = x[q] + c * ((double)d0[q] + (double)d1[q]);
}

int pvanom_rk(double *x, const double *d0, const double *d1, const float *f0, const float *f1,
              const double *dt, size_t n, cudaStream_t s) {
    size_t b = (n + 255) / 256;
    const unsigned g = (unsigned)(b > 4096 ? 4096 : b);
    if (f0)
        k_pvanom_rk<float><<<g, 256, 0, s>>>(x, f0, f1, dt, n);
    else
        k_pvanom_rk<double><<<g, 256, 0, s>>>(x, d0, d1, dt, n);
    return launch_status("pvanom_rk");
}

}  // namespace f2d
