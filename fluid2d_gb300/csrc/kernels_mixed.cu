// kernels_mixed.cu -- stage kernels of the mixed-precision form.
//
// The mixed form keeps the state, the psi tendencies (the multigrid warm
// starts), the RK accumulation of the state and the diagnostics in float64,
// and everything else in float32: the stage states read by the advection,
// the tracer and velocity tendencies, the fluxes.  On GB300 a conversion
// between float64 and float32 runs on the same narrow pipe as float64
// arithmetic, so these kernels read and write float32 wherever the value is
// consumed in float32 and convert once per value, not once per use.
//
// Same update formulas as core/timescheme.py:167-180 (RK3_SSP),
// core/operators.py:214-236, 303-314, 421-498; only the precision differs.
#include "f2d_adv.cuh"
#include "f2d_common.cuh"
#include "f2d_fused.cuh"
#include "f2d_kernels.cuh"
#include "f2d_mixed.cuh"
#include "f2d_batch.cuh"

namespace f2d {

// float copies of the planes the advection reads (tracers, u, v)
struct ToF32Args {
    const double *x;
    float *y;
    size_t n;
};

F2D_DEV void to_f32_body(const ToF32Args &a, const VB vb) {
    for (size_t q = vb.x * (size_t)blockDim.x + threadIdx.x; q < a.n;
         q += (size_t)vb.gx * blockDim.x)
        a.y[q] = (float)a.x[q];
}

__global__ void k_to_f32(ToF32Args a) { pdl_prologue();
    to_f32_body(a, F2D_VB_NATIVE); }

struct BToF32 {
    using Args = ToF32Args;
    static constexpr int THREADS = 256, KIND = BK_ToF32;
    F2D_DEV static void run(const Args &a, VB vb) { to_f32_body(a, vb); }
};
F2D_BATCH_ENTRY(ToF32, BToF32)

int vec_to_f32(const double *x, float *y, size_t n, cudaStream_t s) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    return launch_body<BToF32>(k_to_f32, ToF32Args{x, y, n}, dim3(blocks), dim3(256), 0, s,
                               "to_f32");
}

// celltocorner of a float tendency into the float64 right-hand side
// (core/fortran_operators.f90:58-62, rows/cols 0..m-2)
struct C2CF32Args {
    const float *xr;
    double *xp;
    int m, n;
};

F2D_DEV void c2c_f32_body(const C2CF32Args &a, const VB vb) {
    const int m = a.m, n = a.n;
    int i = vb.x * 32 + threadIdx.x;
    int j = vb.y * 8 + threadIdx.y;
    if (i > n - 2 || j > m - 2) return;
    size_t p = off(j, i, n);
    const float *xr = a.xr;
    a.xp[p] = (double)(0.25f * (xr[p] + xr[p + 1] + xr[p + n] + xr[p + n + 1]));
}

__global__ void k_c2c_f32(C2CF32Args a) { pdl_prologue();
    c2c_f32_body(a, F2D_VB_NATIVE); }

struct BC2CF32 {
    using Args = C2CF32Args;
    static constexpr int THREADS = 256, KIND = BK_C2CF32;
    F2D_DEV static void run(const Args &a, VB vb) { c2c_f32_body(a, vb); }
};
F2D_BATCH_ENTRY(C2CF32, BC2CF32)

int c2c_f32(const float *xr, double *xp, int m, int n, cudaStream_t s) {
    dim3 b(32, 8);
    return launch_body<BC2CF32>(k_c2c_f32, C2CF32Args{xr, xp, m, n}, grid2d(m - 1, n - 1, b), b,
                                0, s, "c2c_f32");
}

// float RK combinations of the stage states (core/timescheme.py:172-176)
F2D_DEV float rk_stage_f32(int rk, float base, float d0, float dq, float dt) {
    if (rk == 1) return base + dt * dq;
    return base + (0.25f * dt) * (d0 + dq);
}

// Advection of one tracer, float32 fluxes from float32 stage states.
// rk 1, 2: next stage state (float); rk 3: final float64 accumulation
// x += (dt/6)*(dx0 + dx1 + 4*dx2) of the state.
F2D_DEV void stage_adv_mixed_body(const AdvMixed &a, const VB vb) {
    __shared__ float sfx[8][33];
    __shared__ float sfy[9][32];
    __shared__ float sdt6;  // dt/6 of the final combination, divided once a CTA
    const int tx = threadIdx.x, ty = threadIdx.y;
    if (tx == 0 && ty == 0 && a.rk == 3) sdt6 = a.dtf[0] / 6.f;
    const int nv = a.nv, mv = a.mv;
    const int I = NH + vb.x * 32 + tx;
    const int J = NH + vb.y * 8 + ty;
    const bool in = (I <= nv - NH - 1) && (J <= mv - NH - 1);
    const SplitT<float> c = *a.advf;
    if (in) {
        const size_t p = off(J, I, nv);
        sfx[ty][tx + 1] = edge_flux_f32(a.kind, a.msk, a.q, a.u, p, 1, a.method, a.order, c);
        sfy[ty + 1][tx] = edge_flux_f32(a.kind, a.msk, a.q, a.v, p, nv, a.method, a.order, c);
        if (ty == 0)
            sfy[0][tx] = edge_flux_f32(a.kind, a.msk, a.q, a.v, p - nv, nv, a.method, a.order, c);
    }
    // the tile's west faces: lanes 0-7 of warp 1, one row each
    if (ty == 1 && tx < 8) {
        const int Jr = NH + vb.y * 8 + tx, I0 = NH + vb.x * 32;
        if (I0 <= nv - NH - 1 && Jr <= mv - NH - 1)
            sfx[tx][0] = edge_flux_f32(a.kind, a.msk, a.q, a.u, off(Jr, I0, nv) - 1, 1, a.method,
                                       a.order, c);
    }
    __syncthreads();
    if (!in) return;
    const size_t p = off(J, I, nv);
    float y = -(c.zdx * (sfx[ty][tx + 1] - sfx[ty][tx])) - c.zdy * (sfy[ty + 1][tx] - sfy[ty][tx]);
    if (a.buoy) {  // rhs_torque (core/operators.py:311-312)
        const int mc = a.msk[p];
        y = mc ? y : 0.f;
        const int sl = mc + a.msk[p - 1], sr = a.msk[p + 1] + mc;
        const int ml = sl > 1 ? sl : 1, mr = sr > 1 ? sr : 1;
        if (ml + mr == 4) y = y + (a.buoy[p + 1] - a.buoy[p - 1]) * a.torque_coef;
    }
    if (a.diff_coef != 0.f && a.msk[p] == 1) {  // add_diffusion
        const float t = a.q[p];
        const float lap = (float)a.msk[p - 1] * (a.q[p - 1] - t) +
                          (float)a.msk[p + 1] * (a.q[p + 1] - t) +
                          (float)a.msk[p - nv] * (a.q[p - nv] - t) +
                          (float)a.msk[p + nv] * (a.q[p + nv] - t);
        y = y + a.diff_coef * lap;
    }
    const float dt = a.dtf[0], dt6 = a.rk == 3 ? sdt6 : 0.f;
    // the point and its periodic halo images
    for_images(J, I, mv, nv, [&](size_t q) {
        a.dq[q] = y;
        if (a.rk < 3) {
            a.sout[q] = rk_stage_f32(a.rk, a.sbase[q], a.d0 ? a.d0[q] : 0.f, y, dt);
        } else {
            const float inc = dt6 * (a.d0[q] + a.d1[q] + 4.f * y);
            a.xout[q] = a.xout[q] + (double)inc;
        }
    });
}

__global__ void __launch_bounds__(256) k_stage_adv_mixed(AdvMixed a) {
    pdl_prologue();
    stage_adv_mixed_body(a, F2D_VB_NATIVE);
}

struct BAdvMixed {
    using Args = AdvMixed;
    static constexpr int THREADS = 256, KIND = BK_AdvMixed, MIN_BLOCKS = 5;
    F2D_DEV static void run(const Args &a, VB vb) { stage_adv_mixed_body(a, vb); }
};
F2D_BATCH_ENTRY(AdvMixed, BAdvMixed)

int stage_advection_mixed(const AdvMixed &a, cudaStream_t s) {
    dim3 b(32, 8);
    return launch_body<BAdvMixed>(k_stage_adv_mixed, a, grid2d(a.mv - 2 * NH, a.nv - 2 * NH, b),
                                  b, 0, s, "stage_advection_mixed");
}

// psi <- psi*mskp (float64, whole array), u, v = orthogradient(psi) in float64
// (the differences of psi need it) stored as float tendencies, and the
// stage-state / final combinations.
F2D_DEV void stage_ortho_mixed_body(const OrthoMixed &a, const VB vb) {
    // dt/6 in float64 (psi) and float (u, v), divided once a CTA
    __shared__ double sdt6;
    __shared__ float sdt6f;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        if (a.psi_rk) sdt6 = *a.dt / 6.;
        if (a.rk == 3) sdt6f = a.dtf[0] / 6.f;
    }
    __syncthreads();
    const int i = vb.x * 32 + threadIdx.x;
    const int j = vb.y * 8 + threadIdx.y;
    const int nv = a.nv, mv = a.mv;
    if (i >= nv || j >= mv) return;
    const size_t p = off(j, i, nv);
    const double pc = a.mskp[p] ? a.psi[p] : 0.;
    a.psi[p] = pc;
    if (a.psi_rk) {
        const double d1 = a.psi1 ? a.psi1[p] : pc;
        const double d2 = a.psi1 ? pc : 0.;
        a.psiout[p] = a.psibase[p] + sdt6 * (a.psi0[p] + d1 + 4 * d2);
    }
    if (i < 1 || j < 1 || i > nv - 2 || j > mv - 2) return;
    const double ps = a.mskp[p - nv] ? a.psi[p - nv] : 0.;
    const double pw = a.mskp[p - 1] ? a.psi[p - 1] : 0.;
    const int mc = a.msk[p];
    const float u = (mc + a.msk[p + 1] == 2) ? (float)(a.zdy * (ps - pc)) : 0.f;
    const float v = (mc + a.msk[p + nv] == 2) ? (float)(a.zdx * (pc - pw)) : 0.f;
    a.du[p] = u;
    a.dv[p] = v;
    const float dt = a.dtf[0];
    if (a.rk == 1 || a.rk == 2) {
        a.su[p] = rk_stage_f32(a.rk, a.ubase[p], a.u0 ? a.u0[p] : 0.f, u, dt);
        a.sv[p] = rk_stage_f32(a.rk, a.vbase[p], a.v0 ? a.v0[p] : 0.f, v, dt);
    } else if (a.rk == 3) {
        a.xu[p] = a.xu[p] + (double)(sdt6f * (a.u0[p] + a.u1[p] + 4.f * u));
        a.xv[p] = a.xv[p] + (double)(sdt6f * (a.v0[p] + a.v1[p] + 4.f * v));
    }
}

__global__ void __launch_bounds__(256) k_stage_ortho_mixed(OrthoMixed a) {
    pdl_prologue();
    stage_ortho_mixed_body(a, F2D_VB_NATIVE);
}

struct BOrthoMixed {
    using Args = OrthoMixed;
    static constexpr int THREADS = 256, KIND = BK_OrthoMixed;
    F2D_DEV static void run(const Args &a, VB vb) { stage_ortho_mixed_body(a, vb); }
};
F2D_BATCH_ENTRY(OrthoMixed, BOrthoMixed)

int stage_ortho_mixed(const OrthoMixed &a, cudaStream_t s) {
    dim3 b(32, 8);
    return launch_body<BOrthoMixed>(k_stage_ortho_mixed, a, grid2d(a.mv, a.nv, b), b, 0, s,
                                    "stage_ortho_mixed");
}

// float32 split constants and dt (set once per step, after set_dt)
struct SplitF32Args {
    const SplitConst *c;
    const double *dt;
    SplitT<float> *cf;
    float *dtf;
};

F2D_DEV void split_f32_body(const SplitF32Args &a, const VB) {
    *a.cf = split_cast<float>(*a.c);
    *a.dtf = (float)*a.dt;
}

__global__ void k_split_f32(SplitF32Args a) { pdl_prologue();
    split_f32_body(a, F2D_VB_NATIVE); }

struct BSplitF32 {
    using Args = SplitF32Args;
    static constexpr int THREADS = 1, KIND = BK_SplitF32;
    F2D_DEV static void run(const Args &a, VB vb) { split_f32_body(a, vb); }
};
F2D_BATCH_ENTRY(SplitF32, BSplitF32)

int split_f32(const double *advc, const double *dt, void *advf, float *dtf, cudaStream_t s) {
    SplitF32Args a{(const SplitConst *)advc, dt, (SplitT<float> *)advf, dtf};
    return launch_body<BSplitF32>(k_split_f32, a, dim3(1), dim3(1), 0, s, "split_f32");
}

}  // namespace f2d
