// kernels_adv.cu -- masked finite-volume advection on the staggered C-grid.
//
// Drop-in kernels for
//   fortran_advection.adv_upwind   (core/fortran_advection.f90:2-165)
//   fortran_advection.adv_centered (core/fortran_advection.f90:169-284)
//   fortran_fluxes.adv_upwind      (core/fortran_fluxes.f90:2-170)
//   fortran_fluxes.adv_centered    (core/fortran_fluxes.f90:174-279)
//
// The Fortran sweeps rows with rolling mask counts (mx5, mx3, my5(i), my3(i))
// and rolling flux rows (fym).  Here every edge flux is an independent
// function of its 6-cell stencil: the rolling counts equal the direct window
// sums msk(i-2..i+2), msk(i-1..i+1) (right-going) and msk(i-1..i+3),
// msk(i..i+2) (left-going).  A CTA computes the fluxes of its tile's edges
// once into shared memory and then takes their divergence, so each edge is
// evaluated 1 + 1/32 (x) or 1 + 1/8 (y) times instead of twice.
#include "f2d_common.cuh"
#include "f2d_kernels.cuh"
#include "f2d_adv.cuh"

namespace f2d {

constexpr int ADV_TX = 32, ADV_TY = 8;

// One CTA: ADV_TY x ADV_TX interior cells.  Fluxes of the tile's edges go to
// shared memory, then y = -(zdx*(fx(i)-fx(i-1))) - zdy*(fy(j)-fy(j-1))
// (core/fortran_advection.f90:149-161).  Only interior cells are written;
// the halo of y keeps its content, as in the reference.
template <int KIND>
__global__ void __launch_bounds__(ADV_TX * ADV_TY)
k_advection(const int8_t *__restrict__ msk, const double *__restrict__ x,
            double *__restrict__ y, const double *__restrict__ u,
            const double *__restrict__ v, double *__restrict__ xflx,
            double *__restrict__ yflx, const double *__restrict__ cst,
            int nh, int method, int order, int m, int n) {
    __shared__ double sfx[ADV_TY][ADV_TX + 1];
    __shared__ double sfy[ADV_TY + 1][ADV_TX];
    __shared__ SplitConst sc;
    const int tx = threadIdx.x, ty = threadIdx.y;
    // the constants (two divisions, log, cosh) once per CTA
    if (tx == 0 && ty == 0) sc = split_const(cst);
    __syncthreads();
    const SplitConst c = sc;
    const int I = nh + blockIdx.x * ADV_TX + tx;
    const int J = nh + blockIdx.y * ADV_TY + ty;
    const bool in = (I <= n - nh - 1) && (J <= m - nh - 1);
    if (in) {
        size_t p = off(J, I, n);
        sfx[ty][tx + 1] = edge_flux<KIND>(msk, x, u, p, 1, method, order, c);
        sfy[ty + 1][tx] = edge_flux<KIND>(msk, x, v, p, n, method, order, c);
        if (ty == 0) sfy[0][tx] = edge_flux<KIND>(msk, x, v, p - n, n, method, order, c);
    }
    // the tile's west faces: lanes 0..ADV_TY-1 of warp 1, one row each (a warp
    // issues a float64 instruction for all its lanes)
    if (ty == 1 && tx < ADV_TY) {
        const int Jr = nh + blockIdx.y * ADV_TY + tx, I0 = nh + blockIdx.x * ADV_TX;
        if (I0 <= n - nh - 1 && Jr <= m - nh - 1)
            sfx[tx][0] = edge_flux<KIND>(msk, x, u, off(Jr, I0, n) - 1, 1, method, order, c);
    }
    __syncthreads();
    if (!in) return;
    size_t p = off(J, I, n);
    double fx = sfx[ty][tx + 1], fxm = sfx[ty][tx];
    double fy = sfy[ty + 1][tx], fym = sfy[ty][tx];
    y[p] = -(c.zdx * (fx - fxm)) - c.zdy * (fy - fym);
    if (xflx) {  // core/fortran_fluxes.f90:150-163
        xflx[p] = fx;
        yflx[p] = fy;
        if (I == nh) xflx[p - 1] = fxm;
        if (J == nh) yflx[p - n] = fym;
    }
}

int launch_advection(int kind, const int8_t *msk, const double *x, double *y,
                     const double *u, const double *v, double *xflx, double *yflx,
                     const double *cst, int nh, int method, int order, int m, int n,
                     cudaStream_t s) {
    if (nh != 3) {
        set_error("NHALO = 3 is compulsory with UP5 (nh=%d)", nh);
        return ERR_NH;
    }
    if (m < 2 * nh + 1 || n < 2 * nh + 1) {
        set_error("advection: grid (%d, %d) has no interior", m, n);
        return ERR_SHAPE;
    }
    if (!msk || !x || !y || !u || !v || !cst || method < 0 || method > 2) {
        set_error("advection: null pointer or bad method %d", method);
        return ERR_ARG;
    }
    dim3 block(ADV_TX, ADV_TY);
    dim3 grid = grid2d(m - 2 * nh, n - 2 * nh, block);
    if (kind == 0)
        k_advection<0><<<grid, block, 0, s>>>(msk, x, y, u, v, xflx, yflx, cst, nh, method, order, m, n);
    else if (kind == 1)
        k_advection<1><<<grid, block, 0, s>>>(msk, x, y, u, v, xflx, yflx, cst, nh, method, order, m, n);
    else
        k_advection<2><<<grid, block, 0, s>>>(msk, x, y, u, v, xflx, yflx, cst, nh, method, order, m, n);
    return launch_status("advection");
}

}  // namespace f2d
