// timeloop.cu -- clock kernels of the device-resident time loop.
//
// core/fluid2d.py:235-314 (loop), :376-397 (set_dt) and core/output.py:62-94
// (Output.do) restated as one-thread kernels that read and write a clock in
// device memory.  The arithmetic is the reference's, operation by operation,
// with explicit round-to-nearest intrinsics where a compiler could otherwise
// fuse a multiply and an add, so the times and the time steps are the
// reference's bits in every build.
#include <cmath>

#include "f2d_adv.cuh"
#include "f2d_common.cuh"
#include "f2d_fused.cuh"
#include "f2d_kernels.cuh"
#include "f2d_loop.cuh"

namespace f2d {

F2D_DEV bool loop_can_step(const LoopClock &c, const LoopConst &k) {
    return c.status == LOOP_RUNNING && c.t < c.tend && c.steps_left > 0 && c.nhis < k.his_cap &&
           c.ndiag < k.diag_cap;
}

// the while-condition for the first iteration of a launch
__global__ void k_loop_gate(LoopClock *c, LoopConst k, cudaGraphConditionalHandle h) {
    LoopClock &C = *c;
    if (C.status == LOOP_RUNNING && !(C.t < C.tend)) C.status = LOOP_TEND;
    cudaGraphSetConditional(h, loop_can_step(C, k) ? 1u : 0u);
}

// set_dt (core/fluid2d.py:376-397) and the exact-history-time adjustment
// (core/fluid2d.py:245-254)
__global__ void k_loop_pre(LoopClock *c, LoopConst k, double *dt, double *cst, SplitConst *advc,
                           const double *diag) {
    LoopClock &C = *c;
    const double maxspeed = diag[0];
    double d = k.dt0;
    if (k.adaptable && maxspeed != 0) {
        d = k.cfl * k.hmin / maxspeed;
        if (d > k.dtmax) d = k.dtmax;
    }
    cst[3] = maxspeed;
    *advc = split_const(cst);
    if (k.exacthistime && k.adaptable) {
        if (__dadd_rn(C.t, __dmul_rn(8., d)) > C.tnexthis && C.reduce == 0) C.reduce = 8;
        if (C.reduce > 0) {
            d = (C.tnexthis - C.t) / ((double)C.reduce * 0.95);
            C.reduce -= 1;
        }
        if (C.t + d > C.tnexthis) {
            C.reduce = 0;
            d = C.tnexthis - C.t;
        }
    }
    *dt = d;
    C.dt = d;
    C.ke_old = diag[k.ike];
    C.ens_old = diag[k.iens];
    C.his_slot = -1;
}

// Output.do (core/output.py:85-94) at the clock's time: a diagnostic row when
// t >= tnextdiag, a history slot when t >= tnexthis
F2D_DEV void loop_output(LoopClock &C, const LoopConst &k, const double *diag, const LoopRings &r,
                         double dkedt, double dvdt) {
    if (C.t >= C.tnextdiag) {
        C.tnextdiag += C.freq_diag;
        double *row = r.diag + (size_t)C.ndiag * (k.ndiag + 4);
        row[0] = C.t;
        row[1] = (double)C.kt;
        for (int q = 0; q < k.ndiag; q++) row[2 + q] = diag[q];
        row[2 + k.ndiag] = dkedt;
        row[3 + k.ndiag] = dvdt;
        C.ndiag += 1;
    }
    if (C.t >= C.tnexthis) {
        C.tnexthis += C.freq_his;
        C.his_slot = C.nhis;
        r.his_t[C.nhis] = C.t;
        r.his_kt[C.nhis] = C.kt;
        C.nhis += 1;
    }
}

// after the step and the diagnostics: clock advance, dkedt/dvdt, output,
// blow-up check, and the while-condition of the next iteration
// (core/fluid2d.py:256-311)
__global__ void k_loop_post(LoopClock *c, LoopConst k, const double *diag, LoopRings r,
                            cudaGraphConditionalHandle h, cudaGraphConditionalHandle hflux) {
    LoopClock &C = *c;
    const double d = C.dt;
    if (k.rescale)  // rescaledtime == 'enstrophy': the enstrophy before the step
        C.t = __dadd_rn(C.t, __dmul_rn(d, sqrt(C.ens_old)));
    else
        C.t = C.t + d;
    C.kt += 1;
    const double dkedt = (diag[k.ike] - C.ke_old) / d;
    const double dvdt = (diag[k.iens] - C.ens_old) / d;
    loop_output(C, k, diag, r, dkedt, dvdt);
    // a time step that does not advance the clock stops the loop
    if (!(d > 0.) || !isfinite(d)) C.status = LOOP_BAD_DT;
    if (C.status == LOOP_RUNNING && diag[0] > 1e3) C.status = LOOP_BLOWUP;
    if (C.status == LOOP_RUNNING && !(C.t < C.tend)) C.status = LOOP_TEND;
    C.steps_left -= 1;
    cudaGraphSetConditional(h, loop_can_step(C, k) ? 1u : 0u);
    // the flux diagnostic runs before a history record is written
    // (core/fluid2d.py:291-293)
    if (k.fluxes) cudaGraphSetConditional(hflux, C.his_slot >= 0 ? 1u : 0u);
}

// Output.do at the start of the loop (core/fluid2d.py:199-214): dkedt and dvdt
// are 0 there
__global__ void k_loop_record(LoopClock *c, LoopConst k, const double *diag, LoopRings r) {
    c->his_slot = -1;
    loop_output(*c, k, diag, r, 0., 0.);
}

// history record of this step: the interior of the saved planes, float32
__global__ void k_loop_snapshot(const LoopClock *c, LoopRings r) {
    const int slot = c->his_slot;
    if (slot < 0) return;
    const int ny = r.mv - 2 * NH, nx = r.nv - 2 * NH;
    const size_t per = (size_t)ny * nx;
    const size_t total = per * r.nsave;
    float *dst = r.his + (size_t)slot * total;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total;
         q += (size_t)gridDim.x * blockDim.x) {
        const int v = (int)(q / per);
        const size_t rem = q - (size_t)v * per;
        const int j = (int)(rem / nx), i = (int)(rem - (size_t)j * nx);
        dst[q] = (float)r.X[(size_t)r.planes[v] * r.pl + off(j + NH, i + NH, r.nv)];
    }
}

// flux record of this step: the interior of the flux planes, float32
__global__ void k_loop_flux_snapshot(const LoopClock *c, LoopRings r) {
    const int slot = c->his_slot;
    if (slot < 0) return;
    const int ny = r.mv - 2 * NH, nx = r.nv - 2 * NH;
    const size_t per = (size_t)ny * nx;
    const size_t total = per * r.nfull;
    float *dst = r.flx + (size_t)slot * total;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total;
         q += (size_t)gridDim.x * blockDim.x) {
        const int v = (int)(q / per);
        const size_t rem = q - (size_t)v * per;
        const int j = (int)(rem / nx), i = (int)(rem - (size_t)j * nx);
        dst[q] = (float)r.FLX[(size_t)v * r.pl + off(j + NH, i + NH, r.nv)];
    }
}

int loop_gate(LoopClock *c, LoopConst k, cudaGraphConditionalHandle h, cudaStream_t s) {
    k_loop_gate<<<1, 1, 0, s>>>(c, k, h);
    return launch_status("loop_gate");
}

int loop_pre(LoopClock *c, LoopConst k, double *dt, double *cst, void *advc, const double *diag,
             cudaStream_t s) {
    k_loop_pre<<<1, 1, 0, s>>>(c, k, dt, cst, (SplitConst *)advc, diag);
    return launch_status("loop_pre");
}

int loop_post(LoopClock *c, LoopConst k, const double *diag, LoopRings r,
              cudaGraphConditionalHandle h, cudaGraphConditionalHandle hflux, cudaStream_t s) {
    k_loop_post<<<1, 1, 0, s>>>(c, k, diag, r, h, hflux);
    return launch_status("loop_post");
}

int loop_record(LoopClock *c, LoopConst k, const double *diag, LoopRings r, cudaStream_t s) {
    k_loop_record<<<1, 1, 0, s>>>(c, k, diag, r);
    return launch_status("loop_record");
}

int loop_snapshot(const LoopClock *c, LoopRings r, cudaStream_t s) {
    const size_t total = (size_t)(r.mv - 2 * NH) * (r.nv - 2 * NH) * r.nsave;
    if (total == 0) return OK;
    size_t blocks = (total + 255) / 256;
    if (blocks > 2048) blocks = 2048;
    k_loop_snapshot<<<(unsigned)blocks, 256, 0, s>>>(c, r);
    return launch_status("loop_snapshot");
}

}  // namespace f2d

namespace f2d {

int loop_flux_snapshot(const LoopClock *c, LoopRings r, cudaStream_t s) {
    const size_t total = (size_t)(r.mv - 2 * NH) * (r.nv - 2 * NH) * r.nfull;
    if (total == 0 || !r.flx) return OK;
    size_t blocks = (total + 255) / 256;
    if (blocks > 2048) blocks = 2048;
    k_loop_flux_snapshot<<<(unsigned)blocks, 256, 0, s>>>(c, r);
    return launch_status("loop_flux_snapshot");
}

}  // namespace f2d
