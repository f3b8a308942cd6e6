/*
 * f2d_oracle.c -- CPU restatement of Fluid2d's native kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300
 * kernels of fluid2d_gb300.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it, and only as what the
 * GPU results are compared against or as the timed CPU baseline -- never as a
 * product code path.
 *
 * Every routine restates the Fortran routine of the same name in
 *   core/fortran_advection.f90, core/fortran_fluxes.f90,
 *   core/fortran_operators.f90, core/fortran_diag.f90,
 *   core/gmg/fortran_multigrid.f90
 * keeping the Fortran loop ranges (1-based indices through the macros
 * below), the evaluation order of every expression, and the REAL*4 literals
 * of the Fortran source widened to double.  It is meant to be compiled with
 * -ffp-contract=off so that no multiply-add is fused.
 *
 * Array convention (what f2py hands the Fortran): a numpy C-ordered array of
 * shape (m, n) is the Fortran array a(m, n) with a(j, i) == numpy a[j-1, i-1].
 * j runs along y (rows), i along x (columns).  The 5-plane stencil array A
 * is passed as a C-ordered (m, n, 5) array, A(j, i, k) == A[j-1, i-1, k-1];
 * the 9-plane array of coarsenmatrix likewise with 9 planes.
 *
 * Parity status: no Fortran compiler exists where this was written, so the
 * Fortran itself could not be run; the restatement is checked line by line
 * and its Python sequencing is pinned against the reference's own Python
 * layers (see tests/golden/make_golden.py).
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#include <stdlib.h>

/* 1-based (j, i) access into a row-major (m, n) array */
#define AT(a, j, i) (a)[((size_t)(j) - 1) * (size_t)n + (size_t)((i) - 1)]
#define AT1(a, j, i) (a)[((size_t)(j) - 1) * (size_t)n1 + (size_t)((i) - 1)]
#define AT2(a, j, i) (a)[((size_t)(j) - 1) * (size_t)n2 + (size_t)((i) - 1)]
/* 1-based (j, i, k) access into a row-major (m, n, K) array */
#define A5(a, j, i, k) (a)[(((size_t)(j) - 1) * (size_t)n + (size_t)((i) - 1)) * 5 + (size_t)((k) - 1)]

/* REAL*4 literals of the Fortran source, widened to REAL*8 */
#define R4(x) ((double)(float)(x))

/* ------------------------------------------------------------------ */
/* fortran_advection.f90:2-165  adv_upwind                              */
/* fortran_fluxes.f90:2-170     adv_upwind with edge-flux outputs       */
/* ------------------------------------------------------------------ */
static int adv_upwind_impl(const int8_t *msk, const double *x, double *y,
                           const double *u, const double *v,
                           double *xflx, double *yflx, const double *cst,
                           int nh, int method, int order, int m, int n,
                           double *fx, double *fy, double *fym,
                           int *my5, int *my3)
{
    if (nh != 3) return 1; /* the Fortran stops the process here */
    const double d1 = (double)(1.f / 30.f);
    const double d2 = (double)(-13.f / 60.f);
    const double d3 = (double)(47.f / 60.f);
    const double d4 = (double)(9.f / 20.f);
    const double d5 = (double)(-1.f / 20.f);
    const double c1 = (double)(-1.f / 6.f);
    const double c2 = (double)(5.f / 6.f);
    const double c3 = (double)(2.f / 6.f);

    double dx = cst[0], dy = cst[1], logcosh = cst[2], umax = cst[3],
           aparab = cst[4];
    double zdx = 1. / dx;
    double zdy = 1. / dy;
    double a = logcosh / umax;
    double KK = (umax - log(cosh(umax * a)) / a) * 0.5;
    double u1 = aparab * umax;
    double aa = 1. / (2. * u1);
    double bb = u1 * 0.5;
    double UU = 0., up, um, qp, qm;
    int mx5, mx3, mx2, my2;

    for (int i = nh; i <= n - nh; i++) {
        my5[i] = AT(msk, 1, i) + AT(msk, 2, i) + AT(msk, 3, i) + AT(msk, 4, i) + AT(msk, 5, i);
        my3[i] = AT(msk, 2, i) + AT(msk, 3, i) + AT(msk, 4, i);
    }
    for (int j = nh; j <= m - nh; j++) {
        mx5 = AT(msk, j, 1) + AT(msk, j, 2) + AT(msk, j, 3) + AT(msk, j, 4) + AT(msk, j, 5);
        mx3 = AT(msk, j, 2) + AT(msk, j, 3) + AT(msk, j, 4);
        for (int i = nh; i <= n - nh; i++) {
            mx2 = AT(msk, j, i) + AT(msk, j, i + 1);
            if (mx2 == 2) {
                double uu = AT(u, j, i);
                if (method == 0) UU = fabs(uu);
                if (method == 1) {
                    UU = fabs(uu);
                    if (UU < u1) UU = aa * (uu * uu) + bb;
                }
                if (method == 2) UU = 2 * KK + log(cosh(uu * a)) / a;
                up = 0.5 * (uu + UU);
                um = 0.5 * (uu - UU);
                if (mx5 == 5 && order == 5) {
                    qp = d1 * AT(x, j, i - 2) + d2 * AT(x, j, i - 1) + d3 * AT(x, j, i)
                         + d4 * AT(x, j, i + 1) + d5 * AT(x, j, i + 2);
                } else if (mx3 == 3 && order >= 3) {
                    qp = c1 * AT(x, j, i - 1) + c2 * AT(x, j, i) + c3 * AT(x, j, i + 1);
                } else {
                    qp = AT(x, j, i);
                }
                mx5 = mx5 - AT(msk, j, i - 2) + AT(msk, j, i + 3);
                mx3 = mx3 - AT(msk, j, i - 1) + AT(msk, j, i + 2);
                if (mx5 == 5 && order == 5) {
                    qm = d5 * AT(x, j, i - 1) + d4 * AT(x, j, i) + d3 * AT(x, j, i + 1)
                         + d2 * AT(x, j, i + 2) + d1 * AT(x, j, i + 3);
                } else if (mx3 == 3 && order >= 3) {
                    qm = c3 * AT(x, j, i) + c2 * AT(x, j, i + 1) + c1 * AT(x, j, i + 2);
                } else {
                    qm = AT(x, j, i + 1);
                }
                fx[i] = up * qp + um * qm;
            } else {
                mx5 = mx5 - AT(msk, j, i - 2) + AT(msk, j, i + 3);
                mx3 = mx3 - AT(msk, j, i - 1) + AT(msk, j, i + 2);
                fx[i] = 0.;
            }
            my2 = AT(msk, j, i) + AT(msk, j + 1, i);
            if (my2 == 2) {
                double vv = AT(v, j, i);
                if (method == 0) UU = fabs(vv);
                if (method == 1) {
                    UU = fabs(vv);
                    if (UU < u1) UU = aa * (vv * vv) + bb;
                }
                if (method == 2) UU = 2 * KK + log(cosh(vv * a)) / a;
                up = 0.5 * (vv + UU);
                um = 0.5 * (vv - UU);
                if (my5[i] == 5 && order == 5) {
                    qp = d1 * AT(x, j - 2, i) + d2 * AT(x, j - 1, i) + d3 * AT(x, j, i)
                         + d4 * AT(x, j + 1, i) + d5 * AT(x, j + 2, i);
                } else if (my3[i] == 3 && order >= 3) {
                    qp = c1 * AT(x, j - 1, i) + c2 * AT(x, j, i) + c3 * AT(x, j + 1, i);
                } else {
                    qp = AT(x, j, i);
                }
                my5[i] = my5[i] - AT(msk, j - 2, i) + AT(msk, j + 3, i);
                my3[i] = my3[i] - AT(msk, j - 1, i) + AT(msk, j + 2, i);
                if (my5[i] == 5 && order == 5) {
                    qm = d5 * AT(x, j - 1, i) + d4 * AT(x, j, i) + d3 * AT(x, j + 1, i)
                         + d2 * AT(x, j + 2, i) + d1 * AT(x, j + 3, i);
                } else if (my3[i] == 3 && order >= 3) {
                    qm = c3 * AT(x, j, i) + c2 * AT(x, j + 1, i) + c1 * AT(x, j + 2, i);
                } else {
                    qm = AT(x, j + 1, i);
                }
                fy[i] = up * qp + um * qm;
            } else {
                my5[i] = my5[i] - AT(msk, j - 2, i) + AT(msk, j + 3, i);
                my3[i] = my3[i] - AT(msk, j - 1, i) + AT(msk, j + 2, i);
                fy[i] = 0.;
            }
        }
        if (j > nh) {
            if (xflx) AT(xflx, j, nh) = fx[nh];
            for (int i = nh + 1; i <= n - nh; i++) {
                AT(y, j, i) = -(zdx * (fx[i] - fx[i - 1])) - zdy * (fy[i] - fym[i]);
                if (xflx) AT(xflx, j, i) = fx[i];
                if (yflx) AT(yflx, j, i) = fy[i];
                fym[i] = fy[i];
            }
        } else {
            for (int i = nh + 1; i <= n - nh; i++) {
                if (yflx) AT(yflx, j, i) = fy[i];
                fym[i] = fy[i];
            }
        }
    }
    return 0;
}

/* scratch for the Fortran automatic arrays fx, fy, fym, my5, my3 (1-based) */
#define MAXN 8200
static double s_fx[MAXN + 2], s_fy[MAXN + 2], s_fym[MAXN + 2];
static int s_my5[MAXN + 2], s_my3[MAXN + 2], s_my2[MAXN + 2];

int adv_upwind(const int8_t *msk, const double *x, double *y, const double *u,
               const double *v, const double *cst, int nh, int method,
               int order, int m, int n)
{
    if (n > MAXN) return 2;
    return adv_upwind_impl(msk, x, y, u, v, NULL, NULL, cst, nh, method, order,
                           m, n, s_fx, s_fy, s_fym, s_my5, s_my3);
}

int adv_upwind_flux(const int8_t *msk, const double *x, double *y,
                    const double *u, const double *v, double *xflx,
                    double *yflx, const double *cst, int nh, int method,
                    int order, int m, int n)
{
    if (n > MAXN) return 2;
    return adv_upwind_impl(msk, x, y, u, v, xflx, yflx, cst, nh, method, order,
                           m, n, s_fx, s_fy, s_fym, s_my5, s_my3);
}

/* ------------------------------------------------------------------ */
/* fortran_advection.f90:169-284  adv_centered (orders 2/4/6)           */
/* ------------------------------------------------------------------ */
int adv_centered(const int8_t *msk, const double *x, double *y, const double *u,
                 const double *v, const double *cst, int nh, int method,
                 int order, int m, int n)
{
    (void)method;
    if (nh != 3) return 1;
    if (n > MAXN) return 2;
    const double e1 = (double)(1.f / 60.f);
    const double e2 = (double)(-2.f / 15.f);
    const double e3 = (double)(37.f / 60.f);
    const double d1 = (double)(-1.f / 12.f);
    const double d2 = (double)(7.f / 12.f);
    const double c1 = (double)(1.f / 2.f);
    double dx = cst[0], dy = cst[1];
    double zdx = 1. / dx, zdy = 1. / dy;
    double qp = 0.;
    int *my6 = s_my5, *my4 = s_my3, *my2 = s_my2;
    double *fx = s_fx, *fy = s_fy, *fym = s_fym;

    for (int i = nh; i <= n - nh; i++) {
        my6[i] = AT(msk, 1, i) + AT(msk, 2, i) + AT(msk, 3, i) + AT(msk, 4, i) + AT(msk, 5, i) + AT(msk, 6, i);
        my4[i] = AT(msk, 2, i) + AT(msk, 3, i) + AT(msk, 4, i) + AT(msk, 5, i);
        my2[i] = AT(msk, 3, i) + AT(msk, 4, i);
    }
    for (int j = nh; j <= m - nh; j++) {
        for (int i = nh; i <= n - nh; i++) {
            int mx6 = AT(msk, j, i - 2) + AT(msk, j, i - 1) + AT(msk, j, i) + AT(msk, j, i + 1) + AT(msk, j, i + 2);
            mx6 = mx6 + AT(msk, j, i + 3);
            int mx4 = AT(msk, j, i - 1) + AT(msk, j, i) + AT(msk, j, i + 1) + AT(msk, j, i + 2);
            int mx2 = AT(msk, j, i) + AT(msk, j, i + 1);
            if (mx2 == 2) {
                if (mx6 == 6 && order == 6) {
                    qp = e1 * (AT(x, j, i - 2) + AT(x, j, i + 3)) + e2 * (AT(x, j, i - 1) + AT(x, j, i + 2));
                    qp = qp + e3 * (AT(x, j, i) + AT(x, j, i + 1));
                } else if (mx4 == 4 && order == 4) {
                    qp = d1 * (AT(x, j, i - 1) + AT(x, j, i + 2)) + d2 * (AT(x, j, i) + AT(x, j, i + 1));
                } else if (mx2 == 2 && order >= 2) {
                    qp = c1 * (AT(x, j, i) + AT(x, j, i + 1));
                }
                fx[i] = AT(u, j, i) * qp;
            } else {
                fx[i] = 0.;
            }
            if (my2[i] == 2) {
                if (my6[i] == 6 && order == 6) {
                    qp = e1 * (AT(x, j - 2, i) + AT(x, j + 3, i));
                    qp = qp + e2 * (AT(x, j - 1, i) + AT(x, j + 2, i)) + e3 * (AT(x, j, i) + AT(x, j + 1, i));
                } else if (my4[i] == 4 && order == 4) {
                    qp = d1 * (AT(x, j - 1, i) + AT(x, j + 2, i)) + d2 * (AT(x, j, i) + AT(x, j + 1, i));
                } else if (my2[i] == 2 && order >= 2) {
                    qp = c1 * (AT(x, j, i) + AT(x, j + 1, i));
                }
                fy[i] = AT(v, j, i) * qp;
            } else {
                fy[i] = 0.;
            }
            my6[i] = my6[i] - AT(msk, j - 2, i) + AT(msk, j + 4, i);
            my4[i] = my4[i] - AT(msk, j - 1, i) + AT(msk, j + 3, i);
            my2[i] = my2[i] - AT(msk, j, i) + AT(msk, j + 2, i);
        }
        if (j > nh) {
            for (int i = nh + 1; i <= n - nh; i++) {
                AT(y, j, i) = -(zdx * (fx[i] - fx[i - 1])) - zdy * (fy[i] - fym[i]);
                fym[i] = fy[i];
            }
        } else {
            for (int i = nh + 1; i <= n - nh; i++) fym[i] = fy[i];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* fortran_fluxes.f90:174-279  adv_centered with edge fluxes (orders 2/4)*/
/* ------------------------------------------------------------------ */
int adv_centered_flux(const int8_t *msk, const double *x, double *y,
                      const double *u, const double *v, double *xflx,
                      double *yflx, const double *cst, int nh, int method,
                      int order, int m, int n)
{
    (void)method;
    if (nh != 3) return 1;
    if (n > MAXN) return 2;
    const double d1 = (double)(-1.f / 12.f);
    const double d2 = (double)(7.f / 12.f);
    const double c1 = (double)(1.f / 2.f);
    double dx = cst[0], dy = cst[1];
    double zdx = 1. / dx, zdy = 1. / dy;
    double qp = 0.;
    int *my4 = s_my3, *my2 = s_my2;
    double *fx = s_fx, *fy = s_fy, *fym = s_fym;

    for (int i = nh; i <= n - nh; i++) {
        my4[i] = AT(msk, 2, i) + AT(msk, 3, i) + AT(msk, 4, i) + AT(msk, 5, i);
        my2[i] = AT(msk, 3, i) + AT(msk, 4, i);
    }
    for (int j = nh; j <= m - nh; j++) {
        for (int i = nh; i <= n - nh; i++) {
            int mx4 = AT(msk, j, i - 1) + AT(msk, j, i) + AT(msk, j, i + 1) + AT(msk, j, i + 2);
            int mx2 = AT(msk, j, i) + AT(msk, j, i + 1);
            if (mx2 == 2) {
                if (mx4 == 4 && order == 4) {
                    qp = d1 * (AT(x, j, i - 1) + AT(x, j, i + 2)) + d2 * (AT(x, j, i) + AT(x, j, i + 1));
                } else if (mx2 == 2 && order >= 2) {
                    qp = c1 * (AT(x, j, i) + AT(x, j, i + 1));
                }
                fx[i] = AT(u, j, i) * qp;
            } else {
                fx[i] = 0.;
            }
            if (my2[i] == 2) {
                if (my4[i] == 4 && order == 4) {
                    qp = d1 * (AT(x, j - 1, i) + AT(x, j + 2, i)) + d2 * (AT(x, j, i) + AT(x, j + 1, i));
                } else if (my2[i] == 2 && order >= 2) {
                    qp = c1 * (AT(x, j, i) + AT(x, j + 1, i));
                }
                fy[i] = AT(v, j, i) * qp;
            } else {
                fy[i] = 0.;
            }
            my4[i] = my4[i] - AT(msk, j - 1, i) + AT(msk, j + 3, i);
            my2[i] = my2[i] - AT(msk, j, i) + AT(msk, j + 2, i);
        }
        if (j > nh) {
            AT(xflx, j, nh) = fx[nh];
            for (int i = nh + 1; i <= n - nh; i++) {
                AT(y, j, i) = -(zdx * (fx[i] - fx[i - 1])) - zdy * (fy[i] - fym[i]);
                AT(xflx, j, i) = fx[i];
                AT(yflx, j, i) = fy[i];
                fym[i] = fy[i];
            }
        } else {
            for (int i = nh + 1; i <= n - nh; i++) {
                AT(yflx, j, i) = fy[i];
                fym[i] = fy[i];
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* fortran_operators.f90                                               */
/* ------------------------------------------------------------------ */
/* :2-39 */
void computeorthogradient(const int8_t *msk, const double *psi, double dx,
                          double dy, int nh, int m, int n, double *u, double *v)
{
    (void)nh;
    double zdx = 1. / dx, zdy = 1. / dy;
    for (int j = 2; j <= m - 1; j++)
        for (int i = 2; i <= n - 1; i++) {
            int mm = AT(msk, j, i) + AT(msk, j, i + 1);
            if (mm == 2) AT(u, j, i) = zdy * (AT(psi, j - 1, i) - AT(psi, j, i));
            else AT(u, j, i) = 0.;
            mm = AT(msk, j, i) + AT(msk, j + 1, i);
            if (mm == 2) AT(v, j, i) = zdx * (AT(psi, j, i) - AT(psi, j, i - 1));
            else AT(v, j, i) = 0.;
        }
}

/* :44-64 */
void celltocorner(const double *xr, double *xp, int m, int n)
{
    for (int j = 1; j <= m - 1; j++)
        for (int i = 1; i <= n - 1; i++)
            AT(xp, j, i) = 0.25 * (AT(xr, j, i) + AT(xr, j, i + 1) + AT(xr, j + 1, i) + AT(xr, j + 1, i + 1));
}

/* :102-122 */
void cornertocell(const double *xp, double *xr, int m, int n)
{
    for (int j = 2; j <= m; j++)
        for (int i = 2; i <= n; i++)
            AT(xr, j, i) = 0.25 * (AT(xp, j, i) + AT(xp, j, i - 1) + AT(xp, j - 1, i) + AT(xp, j - 1, i - 1));
}

/* :125-156 */
void add_diffusion(const int8_t *msk, const double *trac, double dx, int nh,
                   double Kdiff, double *dtrac, int m, int n)
{
    (void)nh;
    double coef = Kdiff / (dx * dx);
    for (int j = 2; j <= m - 1; j++)
        for (int i = 2; i <= n - 1; i++)
            if (AT(msk, j, i) == 1) {
                double t = AT(trac, j, i);
                AT(dtrac, j, i) = AT(dtrac, j, i) + coef * (
                    +(double)AT(msk, j, i - 1) * (AT(trac, j, i - 1) - t)
                    + (double)AT(msk, j, i + 1) * (AT(trac, j, i + 1) - t)
                    + (double)AT(msk, j - 1, i) * (AT(trac, j - 1, i) - t)
                    + (double)AT(msk, j + 1, i) * (AT(trac, j + 1, i) - t));
            }
}

/* :221-277 ; returns 'total' (the f2py intent(out) value) */
double computenoslipsourceterm(const int8_t *msk, const double *x, double *y,
                               double dx, double dy, int nh, int m, int n)
{
    double cff = 1. / (2 * dx * dy);
    double total = 0., u, v;
    for (int j = 1; j <= nh; j++)
        for (int i = 1; i <= n; i++) AT(y, j, i) = 0.;
    for (int j = nh + 1; j <= m - nh + 1; j++) {
        for (int i = 1; i <= nh; i++) AT(y, j, i) = 0.;
        for (int i = nh + 1; i <= n - nh + 1; i++) {
            AT(y, j, i) = 0.;
            int msku = AT(msk, j, i - 1) + AT(msk, j, i);
            if (msku == 1) {
                v = (AT(x, j, i) + AT(x, j - 1, i) - AT(x, j, i - 2) - AT(x, j - 1, i - 2)) * cff;
                if (AT(msk, j, i) != 0) {
                    AT(y, j, i) = AT(y, j, i) - v;
                    total = total - v;
                } else {
                    AT(y, j, i - 1) = AT(y, j, i - 1) + v;
                    total = total + v;
                }
            }
            int mskv = AT(msk, j - 1, i) + AT(msk, j, i);
            if (mskv == 1) {
                u = -(AT(x, j, i) + AT(x, j, i - 1) - AT(x, j - 2, i) - AT(x, j - 2, i - 1)) * cff;
                if (AT(msk, j, i) != 0) {
                    AT(y, j, i) = AT(y, j, i) + u;
                    total = total + u;
                } else {
                    AT(y, j - 1, i) = AT(y, j - 1, i) - u;
                    total = total - u;
                }
            }
        }
    }
    return total;
}

/* :330-381 */
void add_torque(const int8_t *msk, const double *buoy, double dx, int nh,
                double gravity, double *domega, int m, int n)
{
    double coef = 0.5 * gravity / dx;
    for (int j = 1 + nh; j <= m - nh; j++) {
        int i = 1 + nh;
        int s = AT(msk, j, i) + AT(msk, j, i - 1);
        int ml = s > 1 ? s : 1;
        for (i = 1 + nh; i <= n - nh; i++) {
            s = AT(msk, j, i + 1) + AT(msk, j, i);
            int mr = s > 1 ? s : 1;
            int mm = ml + mr;
            if (mm == 4)
                AT(domega, j, i) = AT(domega, j, i)
                    + (AT(buoy, j, i + 1) - AT(buoy, j, i - 1)) * coef * (double)AT(msk, j, i);
            ml = mr;
        }
    }
}

/* ------------------------------------------------------------------ */
/* fortran_diag.f90 (sequential sums in the Fortran loop order)        */
/* ------------------------------------------------------------------ */
/* :3-30 */
double computedotprod(const int8_t *msk, const double *x, const double *y, int nh, int m, int n)
{
    double z = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) != 0) z = z + AT(x, j, i) * AT(y, j, i);
    return z;
}

/* :33-60 */
double computemax(const int8_t *msk, const double *x, int nh, int m, int n)
{
    double y = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) != 0) {
                double a = fabs(AT(x, j, i));
                y = (y > a) ? y : a; /* Fortran max() */
            }
    return y;
}

/* :63-90 */
double computesum(const int8_t *msk, const double *x, int nh, int m, int n)
{
    double y = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) != 0) y = y + AT(x, j, i);
    return y;
}

/* :93-120 */
void computesumandnorm(const int8_t *msk, const double *x, int nh, int m, int n,
                       double *y, double *y2)
{
    double s = 0., s2 = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) == 1) {
                double a = AT(x, j, i);
                s = s + a;
                s2 = s2 + a * a;
            }
    *y = s;
    *y2 = s2;
}

/* :123-152 */
void computenormmaxu(const int8_t *msk, const double *x, int nh, int m, int n,
                     double *y, double *ymax)
{
    double s = 0., mx = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) + AT(msk, j, i + 1) == 2) {
                double a = AT(x, j, i);
                s = s + a * a;
                double b = fabs(a);
                mx = (mx > b) ? mx : b;
            }
    *y = s;
    *ymax = mx;
}

/* :155-195 */
void computekemaxu(const int8_t *msk, const double *u, const double *v, int nh,
                   int m, int n, double *ke, double *maxu)
{
    double k = 0., mu = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) == 1) {
                double a = AT(u, j, i), b = AT(u, j, i - 1);
                double c = AT(v, j, i), d = AT(v, j - 1, i);
                double zu = a * a + b * b;
                double zv = c * c + d * d;
                double um = fabs(a + b);
                double vm = fabs(c + d);
                k = k + zu + zv;
                double s = um + vm;
                mu = (mu > s) ? mu : s;
            }
    *ke = k * 0.25;
    *maxu = mu * 0.5;
}

/* :198-236 */
void computekemaxuv(const int8_t *msk, const double *u, const double *v, int nh,
                    int m, int n, double *ke, double *maxu, double *maxv)
{
    double k = 0., mu = 0., mv = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) == 1) {
                double a = AT(u, j, i), b = AT(u, j, i - 1);
                double c = AT(v, j, i), d = AT(v, j - 1, i);
                double zu = a * a + b * b;
                double zv = c * c + d * d;
                k = k + zu + zv;
                mu = (mu > zu) ? mu : zu;
                mv = (mv > zv) ? mv : zv;
            }
    *ke = k * 0.25;
    *maxu = sqrt(mu / 2.);
    *maxv = sqrt(mv / 2.);
}

/* :239-267 */
double computekewithpsi(const int8_t *msk, const double *omega, const double *psi,
                        int nh, int m, int n)
{
    double ke = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) == 1)
                ke = ke - 0.125 * (AT(psi, j, i) + AT(psi, j - 1, i) + AT(psi, j - 1, i - 1) + AT(psi, j, i - 1))
                     * AT(omega, j, i);
    return ke;
}

/* ------------------------------------------------------------------ */
/* gmg/fortran_multigrid.f90                                            */
/* ------------------------------------------------------------------ */
/* :2-127  two fused damped-Jacobi sweeps through a 3-row buffer yo(3,n) */
void smoothtwicewitha(const int8_t *msk, const double *A, double *x,
                      const double *b, double coef, int m, int n, double *yo)
{
#define YO(l, i) yo[((size_t)(l) - 1) * (size_t)n + (size_t)((i) - 1)]
    int lm = 1, lo = 2, lp = 3;
    double c1 = coef;
    double c2 = 1. - c1;
    double c3;
    for (int i = 1; i <= n; i++) YO(lo, i) = AT(x, 1, i);
    for (int j = 2; j <= m - 1; j++) {
        int jm = j - 1, jp = j + 1;
        YO(lo, 1) = AT(x, j - 1, 1);
        YO(lp, 1) = AT(x, j, 1);
        for (int i = 2; i <= n - 1; i++) {
            int ip = i + 1, im = i - 1;
            if (AT(msk, j, i) != 0) {
                c3 = c1 / fabs(A5(A, j, i, 5));
                YO(lp, i) = AT(x, j, i) * c2 + c3 * (
                    +A5(A, j, i, 1) * AT(x, j - 1, i - 1)
                    + A5(A, j, i, 2) * AT(x, j - 1, i)
                    + A5(A, j, i, 3) * AT(x, j - 1, i + 1)
                    + A5(A, j, i, 4) * AT(x, j, i - 1)
                    + A5(A, j, ip, 4) * AT(x, j, ip)
                    + A5(A, jp, im, 3) * AT(x, jp, im)
                    + A5(A, jp, i, 2) * AT(x, jp, i)
                    + A5(A, jp, ip, 1) * AT(x, jp, ip)
                    - AT(b, j, i));
            } else {
                YO(lp, i) = 0.;
            }
        }
        int jmm = jm - 1;
        if (jm >= 3) {
            AT(x, jmm, 2) = YO(lm, 2);
            AT(x, jmm, n - 1) = YO(lm, n - 1);
            AT(x, jm, 2) = YO(lo, 2);
            for (int i = 3; i <= n - 2; i++) {
                int ip = i + 1, im = i - 1;
                if (AT(msk, jm, i) != 0) {
                    c3 = c1 / fabs(A5(A, jm, i, 5));
                    AT(x, jm, i) = YO(lo, i) * c2 + c3 * (
                        +A5(A, jm, i, 1) * YO(lm, i - 1)
                        + A5(A, jm, i, 2) * YO(lm, i)
                        + A5(A, jm, i, 3) * YO(lm, i + 1)
                        + A5(A, jm, i, 4) * YO(lo, i - 1)
                        + A5(A, jm, ip, 4) * YO(lo, ip)
                        + A5(A, j, im, 3) * YO(lp, im)
                        + A5(A, j, i, 2) * YO(lp, i)
                        + A5(A, j, ip, 1) * YO(lp, ip)
                        - AT(b, jm, i));
                } else {
                    AT(x, jm, i) = 0.;
                }
            }
        }
        lm = lm % 3 + 1;
        lo = lo % 3 + 1;
        lp = lp % 3 + 1;
    }
#undef YO
}

/* :130-212  single in-place sweep (unused by the reference's drivers) */
void smoothoncewitha(const int8_t *msk, const double *A, double *x,
                     const double *b, double coef, int m, int n)
{
    double c1 = coef, c2 = 1. - c1, c3;
    for (int j = 2; j <= m - 1; j++) {
        int jm = j - 1, jp = j + 1;
        for (int i = 2; i <= n - 1; i++) {
            int ip = i + 1, im = i - 1;
            if (AT(msk, j, i) != 0) {
                c3 = c1 / fabs(A5(A, j, i, 5));
                AT(x, j, i) = AT(x, j, i) * c2 + c3 * (
                    +A5(A, j, i, 1) * AT(x, jm, im)
                    + A5(A, j, i, 2) * AT(x, jm, i)
                    + A5(A, j, i, 3) * AT(x, jm, ip)
                    + A5(A, j, i, 4) * AT(x, j, im)
                    + A5(A, j, ip, 4) * AT(x, j, ip)
                    + A5(A, jp, im, 3) * AT(x, jp, im)
                    + A5(A, jp, i, 2) * AT(x, jp, i)
                    + A5(A, jp, ip, 1) * AT(x, jp, ip)
                    - AT(b, j, i));
            } else {
                AT(x, j, i) = 0.;
            }
        }
    }
}

/* :290-317 */
static void tridiag(const double *d, const double *dd, const double *b,
                    double *xc, int l, double *gam)
{
    /* 1-based vectors */
    int k0 = 4;
    double bet = 1. / d[k0];
    xc[k0] = b[k0] * bet;
    for (int k = k0 + 1; k <= l - 4; k++) {
        gam[k] = dd[k - 1] * bet;
        bet = 1. / (d[k] - dd[k - 1] * gam[k]);
        xc[k] = (b[k] - dd[k - 1] * xc[k - 1]) * bet;
    }
    for (int k = l - 5; k >= k0; k--) xc[k] = xc[k] - gam[k + 1] * xc[k + 1];
}

/* :215-288  vertical line relaxation */
#define MAXM 8200
static double s_y[MAXM + 2], s_d[MAXM + 2], s_ud[MAXM + 2], s_rhs[MAXM + 2], s_gam[MAXM + 2];
int smoothtridiag(const int8_t *msk, const double *A, double *x, const double *b,
                  int m, int n)
{
    if (m > MAXM) return 2;
    for (int i = 2; i <= n - 1; i++) {
        int ip = i + 1, im = i - 1;
        if (AT(msk, 4, i) != 0) {
            for (int j = 1; j <= m; j++) s_y[j] = 0.;
            for (int j = 4; j <= m - 4; j++) {
                int jm = j - 1, jp = j + 1;
                s_rhs[j] = AT(b, j, i)
                    - A5(A, j, i, 1) * AT(x, jm, im)
                    - A5(A, j, i, 3) * AT(x, jm, ip)
                    - A5(A, j, i, 4) * AT(x, j, im)
                    - A5(A, j, ip, 4) * AT(x, j, ip)
                    - A5(A, jp, im, 3) * AT(x, jp, im)
                    - A5(A, jp, ip, 1) * AT(x, jp, ip);
                s_d[j] = A5(A, j, i, 5);
                s_ud[j] = A5(A, jp, i, 2);
            }
            tridiag(s_d, s_ud, s_rhs, s_y, m, s_gam);
            for (int j = 4; j <= m - 4; j++) AT(x, j, i) = s_y[j];
        }
    }
    return 0;
}

/* :320-362 */
void computeresidualwitha(const int8_t *msk, const double *A, const double *x,
                          const double *b, double *y, int m, int n)
{
    for (int j = 2; j <= m - 1; j++)
        for (int i = 2; i <= n - 1; i++) {
            if (AT(msk, j, i) != 0) {
                AT(y, j, i) = AT(b, j, i)
                    - A5(A, j, i, 1) * AT(x, j - 1, i - 1)
                    - A5(A, j, i, 2) * AT(x, j - 1, i)
                    - A5(A, j, i, 3) * AT(x, j - 1, i + 1)
                    - A5(A, j, i, 4) * AT(x, j, i - 1)
                    - A5(A, j, i, 5) * AT(x, j, i)
                    - A5(A, j, i + 1, 4) * AT(x, j, i + 1)
                    - A5(A, j + 1, i - 1, 3) * AT(x, j + 1, i - 1)
                    - A5(A, j + 1, i, 2) * AT(x, j + 1, i)
                    - A5(A, j + 1, i + 1, 1) * AT(x, j + 1, i + 1);
            } else {
                AT(y, j, i) = 0.;
            }
        }
}

/* :365-412  periodic wrap of the eight halo blocks */
void fillhalo(double *x, int nh, int m, int n)
{
    int n2 = n - 2 * nh, m2 = m - 2 * nh;
    for (int j = 1; j <= nh; j++) {
        for (int i = 1; i <= nh; i++) AT(x, j, i) = AT(x, m2 + j, n2 + i);
        for (int i = 1; i <= n2; i++) AT(x, j, i + nh) = AT(x, m2 + j, i + nh);
        for (int i = 1; i <= nh; i++) AT(x, j, i + n - nh) = AT(x, m2 + j, nh + i);
    }
    for (int j = 1; j <= m2; j++) {
        int jj = j + nh;
        for (int i = 1; i <= nh; i++) {
            AT(x, jj, i) = AT(x, jj, n2 + i);
            AT(x, jj, i + n - nh) = AT(x, jj, i + nh);
        }
    }
    for (int j = 1; j <= nh; j++) {
        int jj = j + m2 + nh;
        for (int i = 1; i <= nh; i++) AT(x, jj, i) = AT(x, j + nh, n2 + i);
        for (int i = 1; i <= n - 2 * nh; i++) AT(x, jj, i + nh) = AT(x, j + nh, i + nh);
        for (int i = 1; i <= nh; i++) AT(x, jj, i + n - nh) = AT(x, j + nh, i + nh);
    }
}

/* :415-498  mask-aware bilinear prolongation, coarse x2 -> fine x1 */
int interpolate(const int8_t *msk1, const int8_t *msk2, const double *x2, int nh,
                int m2, int n2, int m1, int n1, double *x1)
{
    static const double c2[3] = {0., 1., 0.5};
    const double c3[5] = {0., 1., 0.5, R4(0.3333333333333333333333333333), 0.25};
    int j1 = 0, i1;
    if (nh == 2) j1 = 2;
    else if (nh == 3) j1 = 1;
    else return 1;
    (void)m1;
    for (int j2 = 2; j2 <= m2 - 2; j2++) {
        i1 = (nh == 2) ? 2 : 1;
        for (int i2 = 2; i2 <= n2 - 2; i2++) {
            int s;
            if (AT1(msk1, j1, i1) > 0) AT1(x1, j1, i1) = AT2(x2, j2, i2);
            else AT1(x1, j1, i1) = 0.;

            if (AT1(msk1, j1, i1 + 1) > 0) {
                s = AT2(msk2, j2, i2) + AT2(msk2, j2, i2 + 1);
                AT1(x1, j1, i1 + 1) = (AT2(x2, j2, i2) + AT2(x2, j2, i2 + 1)) * c2[s];
            } else AT1(x1, j1, i1 + 1) = 0.;

            if (AT1(msk1, j1 + 1, i1) > 0) {
                s = AT2(msk2, j2, i2) + AT2(msk2, j2 + 1, i2);
                AT1(x1, j1 + 1, i1) = (AT2(x2, j2, i2) + AT2(x2, j2 + 1, i2)) * c2[s];
            } else AT1(x1, j1 + 1, i1) = 0.;

            if (AT1(msk1, j1 + 1, i1 + 1) > 0) {
                s = AT2(msk2, j2, i2) + AT2(msk2, j2, i2 + 1) + AT2(msk2, j2 + 1, i2) + AT2(msk2, j2 + 1, i2 + 1);
                AT1(x1, j1 + 1, i1 + 1) = c3[s] * (AT2(x2, j2, i2) + AT2(x2, j2, i2 + 1)
                                                   + AT2(x2, j2 + 1, i2) + AT2(x2, j2 + 1, i2 + 1));
            } else AT1(x1, j1 + 1, i1 + 1) = 0.;
            i1 = i1 + 2;
        }
        j1 = j1 + 2;
    }
    return 0;
}

/* :501-546  full-weighting restriction, fine x1 -> coarse x2 */
void restrict_(const int8_t *msk2, const double *x1, int nh, int m2, int n2,
               int m1, int n1, double *x2)
{
    (void)m1;
    int j1 = nh;
    for (int j2 = nh; j2 <= m2 - nh; j2++) {
        int i1 = nh;
        for (int i2 = nh; i2 <= n2 - nh; i2++) {
            if (AT2(msk2, j2, i2) != 0) {
                AT2(x2, j2, i2) = 0.25 * AT1(x1, j1, i1)
                    + 0.125 * (AT1(x1, j1, i1 - 1) + AT1(x1, j1, i1 + 1) + AT1(x1, j1 - 1, i1) + AT1(x1, j1 + 1, i1))
                    + 0.0625 * (AT1(x1, j1 - 1, i1 - 1) + AT1(x1, j1 - 1, i1 + 1) + AT1(x1, j1 + 1, i1 - 1) + AT1(x1, j1 + 1, i1 + 1));
            } else {
                AT2(x2, j2, i2) = 0.;
            }
            i1 = i1 + 2;
        }
        j1 = j1 + 2;
    }
}

/* :706-811  Galerkin coarse operator on the 9-point stencil */
void coarsenmatrix(const double *Afine, double *Acoarse, const int8_t *msk1,
                   const int8_t *msk2, int nh, int m1, int n1, int m2, int n2)
{
    (void)m1;
#define AF(j, i, k) Afine[(((size_t)(j) - 1) * (size_t)n1 + (size_t)((i) - 1)) * 9 + (size_t)((k) - 1)]
#define AC(j, i, k) Acoarse[(((size_t)(j) - 1) * (size_t)n2 + (size_t)((i) - 1)) * 9 + (size_t)((k) - 1)]
    /* coef(ki,kj), ki,kj in -1..1 ; DATA order is column-major */
    static const double cdata[9] = {0.125, 0.25, 0.125, 0.25, 0.5, 0.25, 0.125, 0.25, 0.125};
#define COEF(ki, kj) cdata[((ki) + 1) + ((kj) + 1) * 3]
    double z5[5][5]; /* z5(i,j) -> z5[i+2][j+2] */
    double z3[3][3]; /* z3(ii,jj) -> z3[ii+1][jj+1] */
    for (int j2 = nh; j2 <= m2 - nh; j2++)
        for (int i2 = nh; i2 <= n2 - nh; i2++) {
            if (AT2(msk2, j2, i2) == 1) {
                for (int l = 1; l <= 9; l++) {
                    int i1 = 2 * (i2 - nh) + nh;
                    int j1 = 2 * (j2 - nh) + nh;
                    int di2 = (l - 1) % 3 - 1;
                    int dj2 = (l - 1) / 3 - 1;
                    memset(z5, 0, sizeof(z5));
                    for (int kj = -1; kj <= 1; kj++)
                        for (int ki = -1; ki <= 1; ki++) {
                            int i = 2 * di2 + ki;
                            int j = 2 * dj2 + kj;
                            if (abs(i) <= 2 && abs(j) <= 2) {
                                if (AT1(msk1, j1 + j, i1 + i) == 1)
                                    z5[i + 2][j + 2] = 2. * COEF(ki, kj);
                            }
                        }
                    memset(z3, 0, sizeof(z3));
                    for (int jj = -1; jj <= 1; jj++)
                        for (int ii = -1; ii <= 1; ii++)
                            for (int kj = -1; kj <= 1; kj++)
                                for (int ki = -1; ki <= 1; ki++) {
                                    int k = 1 + (ki + 1) + (kj + 1) * 3;
                                    if (AT1(msk1, j1 + jj, i1 + ii) == 1)
                                        z3[ii + 1][jj + 1] = z3[ii + 1][jj + 1]
                                            + AF(j1 + jj, i1 + ii, k) * z5[ii + ki + 2][jj + kj + 2];
                                }
                    double w = 0.;
                    if (AT2(msk2, j2, i2) != 0)
                        for (int jj = -1; jj <= 1; jj++)
                            for (int ii = -1; ii <= 1; ii++)
                                w = w + 0.5 * COEF(ii, jj) * z3[ii + 1][jj + 1];
                    AC(j2, i2, l) = w;
                }
            } else {
                for (int l = 1; l <= 9; l++) AC(j2, i2, l) = 0.;
            }
        }
#undef AF
#undef AC
#undef COEF
}

/* :813-839 */
double computenorm(const int8_t *msk, const double *x, int nh, int m, int n)
{
    double y = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) != 0) y = y + AT(x, j, i) * AT(x, j, i);
    return y;
}

/* :841-867 */
double computeinner(const int8_t *msk, const double *x, const double *y, int nh, int m, int n)
{
    double z = 0.;
    for (int j = nh + 1; j <= m - nh; j++)
        for (int i = nh + 1; i <= n - nh; i++)
            if (AT(msk, j, i) != 0) z = z + AT(x, j, i) * AT(y, j, i);
    return z;
}
