// f2d_loop.cuh -- the time loop of core/fluid2d.py:235-314 kept on the device.
//
// The clock (t, dt, kt, the next history and diagnostic times, the
// exact-history-time countdown) lives in device memory and is advanced by
// one-thread kernels inside the step graph, so a whole run to `tend` is one
// graph launch: a conditional WHILE node whose body is one step.  History
// snapshots and diagnostic rows go to device rings that the host drains when
// they fill or the run ends.
#pragma once
#include <cuda_runtime.h>

namespace f2d {

enum LoopStatus {
    LOOP_RUNNING = 0,  // t < tend, no blow-up
    LOOP_TEND = 1,     // t >= tend (core/fluid2d.py:235)
    LOOP_BLOWUP = 2,   // maxspeed > 1e3 (core/fluid2d.py:306-311)
    LOOP_BAD_DT = 3,   // dt not a positive finite number: stopped, not stepped
};

#define LOOP_MAX_SAVE 8
#define LOOP_MAX_DIAG 8

// Device-resident clock; the host reads it after a launch and writes it at
// setup (a restart sets t, kt, tnexthis, tnextdiag).
struct LoopClock {
    double t, dt, tend;
    double tnexthis, tnextdiag, freq_his, freq_diag;
    double ke_old, ens_old;
    int kt, reduce;
    int steps_left;   // iteration limit of one launch
    int status;       // LoopStatus
    int nhis, ndiag;  // records waiting in the rings
    int his_slot;     // ring slot of this step's history record, -1 if none
    int pad;
};

// Settings fixed for a captured loop (passed by value to the kernels).
struct LoopConst {
    int adaptable, exacthistime, rescale;
    int ike, iens, ndiag;  // diag indices of ke and enstrophy, diag count
    int his_cap, diag_cap;
    int fluxes;  // flux diagnostic before each history record
    double dt0, cfl, hmin, dtmax;
};

// Ring buffers: history [his_cap][nsave][ny][nx] float32 (the interior,
// as core/output.py:234-243 stores it), their (t, kt), and diagnostic rows
// [diag_cap][2 + ndiag + 2] = t, kt, the model's diagnostics, dkedt, dvdt.
struct LoopRings {
    float *his;
    double *his_t;
    int *his_kt;
    double *diag;
    const double *X;  // model state (nvar, mv, nv)
    size_t pl;
    int mv, nv, nsave;
    int planes[LOOP_MAX_SAVE];
    float *flx;        // [his_cap][nfull][ny][nx] flux records, or null
    const double *FLX; // the flux diagnostic's planes (nfull, mv, nv)
    int nfull;
};

int loop_gate(LoopClock *c, LoopConst k, cudaGraphConditionalHandle h, cudaStream_t s);
int loop_pre(LoopClock *c, LoopConst k, double *dt, double *cst, void *advc, const double *diag,
             cudaStream_t s);
int loop_post(LoopClock *c, LoopConst k, const double *diag, LoopRings r,
              cudaGraphConditionalHandle h, cudaGraphConditionalHandle hflux, cudaStream_t s);
int loop_record(LoopClock *c, LoopConst k, const double *diag, LoopRings r, cudaStream_t s);
int loop_snapshot(const LoopClock *c, LoopRings r, cudaStream_t s);
int loop_flux_snapshot(const LoopClock *c, LoopRings r, cudaStream_t s);

}  // namespace f2d
