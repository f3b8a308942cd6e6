// f2d_mixed.cuh -- stage kernels of the mixed-precision form (internal).
#pragma once
#include "f2d_adv.cuh"
#include "f2d_common.cuh"

namespace f2d {

struct AdvMixed {
    const int8_t *msk;
    const float *q, *u, *v;     // stage state (float)
    const SplitT<float> *advf;  // float split constants
    const float *dtf;
    float *dq;                  // tendency (float, interior + periodic halo)
    const float *buoy;          // Boussinesq torque: stage buoyancy (null: none)
    float torque_coef;          // 0.5*gravity/dx
    float diff_coef;            // add_diffusion coefficient Kdiff/(dx*dx), 0: none
    int rk;                     // 1, 2: sout = stage combination; 3: xout += (dt/6)(...)
    const float *sbase, *d0, *d1;
    float *sout;
    double *xout;
    int kind, method, order, mv, nv;
};

struct OrthoMixed {
    const int8_t *msk, *mskp;
    double *psi;                // float64 psi tendency, masked in place
    float *du, *dv;             // float velocity tendencies (rows/cols 1..m-2)
    double zdx, zdy;
    int rk;                     // 1, 2: stage states su, sv; 3: xu, xv += (dt/6)(...)
    const float *ubase, *vbase, *u0, *v0, *u1, *v1;
    float *su, *sv;
    double *xu, *xv;
    int psi_rk;                 // as OrthoStage::psi_rk, in float64
    const double *psibase, *psi0, *psi1;
    double *psiout;
    const double *dt;
    const float *dtf;
    int mv, nv;
};

int vec_to_f32(const double *x, float *y, size_t n, cudaStream_t s);
int c2c_f32(const float *xr, double *xp, int m, int n, cudaStream_t s);
int stage_advection_mixed(const AdvMixed &a, cudaStream_t s);
int stage_ortho_mixed(const OrthoMixed &a, cudaStream_t s);
int split_f32(const double *advc, const double *dt, void *advf, float *dtf, cudaStream_t s);

}  // namespace f2d
