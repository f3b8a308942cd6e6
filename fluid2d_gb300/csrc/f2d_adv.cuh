// f2d_adv.cuh -- edge fluxes of the masked upwind/centred advection
// (core/fortran_advection.f90, core/fortran_fluxes.f90), shared by the
// drop-in kernels and the fused stage kernel.
#pragma once
#include "f2d_common.cuh"

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

// Split constants in the compute type T (float for the mixed form)
template <typename T>
struct SplitT {
    T zdx, zdy, a, KK, u1, aa, bb;
};

template <typename T>
F2D_DEV SplitT<T> split_cast(const SplitConst &c) {
    return SplitT<T>{(T)c.zdx, (T)c.zdy, (T)c.a, (T)c.KK, (T)c.u1, (T)c.aa, (T)c.bb};
}

// |U| of the flux splitting (core/fortran_advection.f90:77-83)
template <typename T>
F2D_DEV T split_speed(T uu, int method, const SplitT<T> &c) {
    T UU = 0;
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
// core/fortran_advection.f90:72-111 (x) and :113-146 (y).  The weights are
// the Fortran's REAL*4 literals, exact in float and widened in double.
template <typename T>
F2D_DEV T upwind_flux(const T *q, const int *mk, T vel, int method, int order,
                      const SplitT<T> &c) {
    if (mk[2] + mk[3] != 2) return 0;
    const T d1 = (T)r4(1.f / 30.f), d2 = (T)r4(-13.f / 60.f), d3 = (T)r4(47.f / 60.f),
            d4 = (T)r4(9.f / 20.f), d5 = (T)r4(-1.f / 20.f);
    const T c1 = (T)r4(-1.f / 6.f), c2 = (T)r4(5.f / 6.f), c3 = (T)r4(2.f / 6.f);
    T UU = split_speed(vel, method, c);
    int m5p = mk[0] + mk[1] + mk[2] + mk[3] + mk[4];
    int m3p = mk[1] + mk[2] + mk[3];
    int m5m = mk[1] + mk[2] + mk[3] + mk[4] + mk[5];
    int m3m = mk[2] + mk[3] + mk[4];
#ifndef F2D_EXACT
    if (order == 5 && m5p == 5 && m5m == 5) {
        // product build, both 5th-order reconstructions: the same flux from
        // their symmetric and antisymmetric sums, up qp + um qm =
        // (vel (qp + qm) + UU (qp - qm)) / 2 -- 16 operations instead of 20
        const T s1 = (T)0.5 * d1, s2 = (T)0.5 * (d2 + d5), s3 = (T)0.5 * (d3 + d4);
        const T a2 = (T)0.5 * (d2 - d5), a3 = (T)0.5 * (d3 - d4);
        const T S = fma(s1, q[0] + q[5], fma(s2, q[1] + q[4], s3 * (q[2] + q[3])));
        const T D = fma(s1, q[0] - q[5], fma(a2, q[1] - q[4], a3 * (q[2] - q[3])));
        return fma(UU, D, vel * S);
    }
#endif
    T up = (T)0.5 * (vel + UU);
    T um = (T)0.5 * (vel - UU);
    T qp, qm;
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
template <typename T>
F2D_DEV T centered_flux(const T *q, const int *mk, T vel, int order, bool allow6) {
    int m2 = mk[2] + mk[3];
    if (m2 != 2) return 0;
    const T e1 = (T)r4(1.f / 60.f), e2 = (T)r4(-2.f / 15.f), e3 = (T)r4(37.f / 60.f);
    const T d1 = (T)r4(-1.f / 12.f), d2 = (T)r4(7.f / 12.f);
    const T c1 = (T)r4(1.f / 2.f);
    int m6 = mk[0] + mk[1] + mk[2] + mk[3] + mk[4] + mk[5];
    int m4 = mk[1] + mk[2] + mk[3] + mk[4];
    T qp = 0;
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

// edge flux in compute type T from float64 arrays
template <int KIND, typename T>
F2D_DEV T edge_flux_t(const int8_t *msk, const double *x, const double *vel, size_t p0,
                      ptrdiff_t s, int method, int order, const SplitT<T> &c) {
    T q[6];
    int mk[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        ptrdiff_t o = (ptrdiff_t)p0 + (ptrdiff_t)(k - 2) * s;
        mk[k] = msk[o];
    }
    if (mk[2] + mk[3] != 2) return 0;
#pragma unroll
    for (int k = 0; k < 6; k++) q[k] = (T)__ldg(x + (ptrdiff_t)p0 + (ptrdiff_t)(k - 2) * s);
    T w = (T)__ldg(vel + p0);
    if (KIND == 0) return upwind_flux<T>(q, mk, w, method, order, c);
    return centered_flux<T>(q, mk, w, order, KIND == 1);
}

// float32 edge flux from float32 arrays (mixed form)
F2D_DEV float edge_flux_f32(int kind, const int8_t *msk, const float *x, const float *vel,
                            size_t p0, ptrdiff_t s, int method, int order,
                            const SplitT<float> &c) {
    float q[6];
    int mk[6];
#pragma unroll
    for (int k = 0; k < 6; k++) mk[k] = msk[(ptrdiff_t)p0 + (ptrdiff_t)(k - 2) * s];
    if (mk[2] + mk[3] != 2) return 0.f;
#pragma unroll
    for (int k = 0; k < 6; k++) q[k] = __ldg(x + (ptrdiff_t)p0 + (ptrdiff_t)(k - 2) * s);
    const float w = __ldg(vel + p0);
    if (kind == 0) return upwind_flux<float>(q, mk, w, method, order, c);
    return centered_flux<float>(q, mk, w, order, kind == 1);
}

template <int KIND>
F2D_DEV double edge_flux(const int8_t *msk, const double *x, const double *vel, size_t p0,
                         ptrdiff_t s, int method, int order, const SplitConst &c) {
    return edge_flux_t<KIND, double>(msk, x, vel, p0, s, method, order, split_cast<double>(c));
}

template <typename T>
F2D_DEV T edge_flux_rt_t(int kind, const int8_t *msk, const double *x, const double *vel,
                         size_t p0, ptrdiff_t s, int method, int order, const SplitT<T> &c) {
    if (kind == 0) return edge_flux_t<0, T>(msk, x, vel, p0, s, method, order, c);
    if (kind == 1) return edge_flux_t<1, T>(msk, x, vel, p0, s, method, order, c);
    return edge_flux_t<2, T>(msk, x, vel, p0, s, method, order, c);
}

// runtime-kind dispatch (uniform across the grid)
F2D_DEV double edge_flux_rt(int kind, const int8_t *msk, const double *x, const double *vel,
                            size_t p0, ptrdiff_t s, int method, int order, const SplitConst &c) {
    if (kind == 0) return edge_flux<0>(msk, x, vel, p0, s, method, order, c);
    if (kind == 1) return edge_flux<1>(msk, x, vel, p0, s, method, order, c);
    return edge_flux<2>(msk, x, vel, p0, s, method, order, c);
}

}  // namespace f2d
