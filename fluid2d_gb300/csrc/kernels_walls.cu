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

// ---- the f2py routine itself (core/fortran_operators.f90:221-277), for
// callers of fortran_operators.computenoslipsourceterm (core/operators.py:256).
// Its loop visits 1-based rows nh+1..m-nh+1 and columns nh+1..n-nh+1, so it
// also writes the first halo row and column after the interior, and its
// scatters reach row and column nh.  Written here, 0-based:
//  * rows [0, nh): 0, except row nh-1 at columns [nh, n-nh], which takes the
//    south-edge term of the visited cell above it when that cell is solid;
//  * rows [nh, m-nh]: columns [0, nh-1) are 0; column nh-1 takes the
//    west-edge term of its solid east neighbour; columns [nh, n-nh] gather
//    their terms in the loop's order (own west, own south, east neighbour's
//    west, north neighbour's south), the last visited column and row
//    receiving nothing from beyond;
//  * every other cell keeps its value (f2py intent(inplace)).
__global__ void k_noslip_dropin(const int8_t *m, const double *x, double *y, double cff, int nh,
                                int mm, int nn) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= nn || j > mm - nh) return;
    const size_t p = off(j, i, nn);
    const int ilast = nn - nh, jlast = mm - nh;  // last visited column and row
    double r = 0.;
    if (j < nh) {
        if (j == nh - 1 && i >= nh && i <= ilast && m[p + nn] == 0 && m[p] + m[p + nn] == 1)
            r = r - edge_u(x, p + nn, nn, cff);
    } else if (i < nh - 1) {
        // zeroed by y(j,1:nh)=0
    } else if (i == nh - 1) {
        if (m[p + 1] == 0 && m[p] + m[p + 1] == 1) r = r + edge_v(x, p + 1, nn, cff);
    } else if (i <= ilast) {
        const int mc = m[p];
        if (mc != 0) {
            if (m[p - 1] + mc == 1) r = r - edge_v(x, p, nn, cff);
            if (m[p - nn] + mc == 1) r = r + edge_u(x, p, nn, cff);
        }
        if (i < ilast && m[p + 1] == 0 && mc + m[p + 1] == 1) r = r + edge_v(x, p + 1, nn, cff);
        if (j < jlast && m[p + nn] == 0 && mc + m[p + nn] == 1)
            r = r - edge_u(x, p + nn, nn, cff);
    } else {
        return;  // beyond the last visited column: untouched
    }
    y[p] = r;
}

// The routine's intent(out) 'total': the terms added in the loop's order,
// one after the other as the Fortran adds them (one CTA walks the rows; each
// chunk of a row compacts its terms in column order, then one thread adds
// them), so the value is the reference's to the last bit.
constexpr int NS_THREADS = 1024;

__global__ void __launch_bounds__(NS_THREADS)
    k_noslip_total(const int8_t *m, const double *x, double cff, int nh, int mm, int nn,
                   double *total) {
    __shared__ double terms[2 * NS_THREADS];
    __shared__ int wbase[NS_THREADS / 32];
    __shared__ int nterms;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int ilast = nn - nh;
    double acc = 0.;  // thread 0's running sum
    for (int j = nh; j <= mm - nh; j++) {
        for (int c0 = nh; c0 <= ilast; c0 += NS_THREADS) {
            const int i = c0 + t;
            double a = 0., b = 0.;
            int na = 0, nb = 0;
            if (i <= ilast) {
                const size_t p = off(j, i, nn);
                const int mc = m[p];
                if (m[p - 1] + mc == 1) {
                    const double v = edge_v(x, p, nn, cff);
                    a = mc != 0 ? -v : v;
                    na = 1;
                }
                if (m[p - nn] + mc == 1) {
                    const double u = edge_u(x, p, nn, cff);
                    b = mc != 0 ? u : -u;
                    nb = 1;
                }
            }
            const int cnt = na + nb;
            int s = cnt;  // inclusive scan over the warp
            for (int o = 1; o < 32; o <<= 1) {
                const int up = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += up;
            }
            if (lane == 31) wbase[w] = s;
            __syncthreads();
            if (w == 0) {
                const int own = wbase[lane];
                int e = own;
                for (int o = 1; o < 32; o <<= 1) {
                    const int up = __shfl_up_sync(0xffffffffu, e, o);
                    if (lane >= o) e += up;
                }
                wbase[lane] = e - own;
                if (lane == 31) nterms = e;
            }
            __syncthreads();
            int pos = wbase[w] + s - cnt;
            if (na) terms[pos++] = a;
            if (nb) terms[pos] = b;
            __syncthreads();
            if (t == 0)
                for (int q = 0; q < nterms; q++) acc = acc + terms[q];
            __syncthreads();
        }
    }
    if (t == 0) *total = acc;
}

int launch_noslip_dropin(const int8_t *msk, const double *x, double *y, double dx, double dy,
                         int nh, int m, int n, double *total, cudaStream_t s) {
    if (!msk || !x || !y) {
        set_error("computenoslipsourceterm: null array");
        return ERR_ARG;
    }
    if (nh < 2 || m < 2 * nh + 1 || n < 2 * nh + 1) {
        set_error("computenoslipsourceterm: nh=%d with (m, n) = (%d, %d)", nh, m, n);
        return nh < 2 ? ERR_NH : ERR_SHAPE;
    }
    const double cff = 1. / (2 * dx * dy);
    dim3 b(32, 8);
    k_noslip_dropin<<<grid2d(m - nh + 1, n, b), b, 0, s>>>(msk, x, y, cff, nh, m, n);
    int st = launch_status("computenoslipsourceterm");
    if (st || !total) return st;
    k_noslip_total<<<1, NS_THREADS, 0, s>>>(msk, x, cff, nh, m, n, total);
    return launch_status("computenoslipsourceterm total");
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
