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

namespace f2d {

// Flux-splitting constants derived from cst = [dx, dy, logcosh, umax, aparab]
// exactly as core/fortran_advection.f90:46-60 derives them.
struct SplitConst {
    double zdx, zdy, a, KK, u1, aa, bb;
};

F2D_DEV SplitConst split_const(const double *cst) {
    SplitConst c;
    double dx = cst[0], dy = cst[1], logcosh = cst[2], umax = cst[3], aparab = cst[4];
    c.zdx = 1. / dx;
    c.zdy = 1. / dy;
    c.a = logcosh / umax;
    c.KK = (umax - log(cosh(umax * c.a)) / c.a) * 0.5;
    c.u1 = aparab * umax;
    c.aa = 1. / (2. * c.u1);
    c.bb = c.u1 * 0.5;
    return c;
}

// |U| of the flux splitting (core/fortran_advection.f90:77-83)
F2D_DEV double split_speed(double uu, int method, const SplitConst &c) {
    double UU = 0.;
    if (method == 0) UU = fabs(uu);
    if (method == 1) {
        UU = fabs(uu);
        if (UU < c.u1) UU = c.aa * (uu * uu) + c.bb;
    }
    if (method == 2) UU = 2 * c.KK + log(cosh(uu * c.a)) / c.a;
    return UU;
}

// Upwind edge flux between cells p0 and p1 along a line with stride s;
// q[k] = x at p0 + (k-2)*s for k = 0..5 (cells p0-2 .. p0+3), mk likewise.
// core/fortran_advection.f90:72-111 (x) and :113-146 (y).
F2D_DEV double upwind_flux(const double *q, const int *mk, double vel, int method,
                           int order, const SplitConst &c) {
    if (mk[2] + mk[3] != 2) return 0.;
    const double d1 = r4(1.f / 30.f), d2 = r4(-13.f / 60.f), d3 = r4(47.f / 60.f),
                 d4 = r4(9.f / 20.f), d5 = r4(-1.f / 20.f);
    const double c1 = r4(-1.f / 6.f), c2 = r4(5.f / 6.f), c3 = r4(2.f / 6.f);
    double UU = split_speed(vel, method, c);
    double up = 0.5 * (vel + UU);
    double um = 0.5 * (vel - UU);
    int m5p = mk[0] + mk[1] + mk[2] + mk[3] + mk[4];
    int m3p = mk[1] + mk[2] + mk[3];
    int m5m = mk[1] + mk[2] + mk[3] + mk[4] + mk[5];
    int m3m = mk[2] + mk[3] + mk[4];
    double qp, qm;
    if (m5p == 5 && order == 5)
        qp = d1 * q[0] + d2 * q[1] + d3 * q[2] + d4 * q[3] + d5 * q[4];
    else if (m3p == 3 && order >= 3)
        qp = c1 * q[1] + c2 * q[2] + c3 * q[3];
    else
        qp = q[2];
    if (m5m == 5 && order == 5)
        qm = d5 * q[1] + d4 * q[2] + d3 * q[3] + d2 * q[4] + d1 * q[5];
    else if (m3m == 3 && order >= 3)
        qm = c3 * q[2] + c2 * q[3] + c1 * q[4];
    else
        qm = q[3];
    return up * qp + um * qm;
}

// Centred edge flux (orders 2/4/6), core/fortran_advection.f90:228-262;
// the fortran_fluxes copy (core/fortran_fluxes.f90:225-258) has no 6th
// order branch (allow6 = false).
F2D_DEV double centered_flux(const double *q, const int *mk, double vel, int order,
                             bool allow6) {
    int m2 = mk[2] + mk[3];
    if (m2 != 2) return 0.;
    const double e1 = r4(1.f / 60.f), e2 = r4(-2.f / 15.f), e3 = r4(37.f / 60.f);
    const double d1 = r4(-1.f / 12.f), d2 = r4(7.f / 12.f);
    const double c1 = r4(1.f / 2.f);
    int m6 = mk[0] + mk[1] + mk[2] + mk[3] + mk[4] + mk[5];
    int m4 = mk[1] + mk[2] + mk[3] + mk[4];
    double qp = 0.;
    if (allow6 && m6 == 6 && order == 6) {
        qp = e1 * (q[0] + q[5]) + e2 * (q[1] + q[4]);
        qp = qp + e3 * (q[2] + q[3]);
    } else if (m4 == 4 && order == 4) {
        qp = d1 * (q[1] + q[4]) + d2 * (q[2] + q[3]);
    } else if (m2 == 2 && order >= 2) {
        qp = c1 * (q[2] + q[3]);
    }
    return vel * qp;
}

template <int KIND>  // 0 upwind, 1 centred (advection), 2 centred (fluxes copy)
F2D_DEV double edge_flux(const int8_t *msk, const double *x, const double *vel,
                         size_t p0, ptrdiff_t s, int method, int order,
                         const SplitConst &c) {
    double q[6];
    int mk[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        ptrdiff_t o = (ptrdiff_t)p0 + (ptrdiff_t)(k - 2) * s;
        mk[k] = msk[o];
    }
    if (mk[2] + mk[3] != 2) return 0.;
#pragma unroll
    for (int k = 0; k < 6; k++) q[k] = __ldg(x + (ptrdiff_t)p0 + (ptrdiff_t)(k - 2) * s);
    double w = __ldg(vel + p0);
    if (KIND == 0) return upwind_flux(q, mk, w, method, order, c);
    return centered_flux(q, mk, w, order, KIND == 1);
}

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
    const SplitConst c = split_const(cst);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int I = nh + blockIdx.x * ADV_TX + tx;
    const int J = nh + blockIdx.y * ADV_TY + ty;
    const bool in = (I <= n - nh - 1) && (J <= m - nh - 1);
    if (in) {
        size_t p = off(J, I, n);
        sfx[ty][tx + 1] = edge_flux<KIND>(msk, x, u, p, 1, method, order, c);
        sfy[ty + 1][tx] = edge_flux<KIND>(msk, x, v, p, n, method, order, c);
        if (tx == 0) sfx[ty][0] = edge_flux<KIND>(msk, x, u, p - 1, 1, method, order, c);
        if (ty == 0) sfy[0][tx] = edge_flux<KIND>(msk, x, v, p - n, n, method, order, c);
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
