// eqwp.h -- internal interface of the elastic-wave stage kernels (eqwp.cu).
#pragma once
#include "b2r_common.cuh"

namespace b2r {

struct FieldPtrs {
    float* p[10];   // vx, vy, vz, sxx, sxy, sxz, syy, syz, szz, disp
};
struct AccPtrs {
    float* p[3];    // unscaled velocity-stage stencil sums ax, ay, az
};
struct MatPtrs {
    const float* p[3];   // lambda, mu, buoyancy
};

struct EqwpRefParams {
    float ca, cb;                    // FD4 weights / dx
    float l2m_dt, l_dt, mu_dt;       // dt * (lambda+2mu), dt*lambda, dt*mu
    float dt_rho, dt2_rho;           // dt/rho, dt^2/rho
    float fval;                      // body force (y)
    int fsteps;                      // force active while ts < fsteps
    int fy, fx0, fx1, fz0, fz1;      // force plane / patch (block coordinates)
};

struct EqwpStagParams {
    float dt, inv_h;
    int src[3];                      // source cell, global interior coordinates
    const float* src_host;           // per-step source increment (host array)
    int src_len;
};

EqwpRefParams eqwp_ref_params(const BlockLayout& L);
cudaError_t launch_eqwp_ref_substep(float* const* fld, const BlockLayout& L, int step_i, int ts,
                                    const EqwpRefParams& p, cudaStream_t st);
cudaError_t launch_eqwp_stag_substep(float* const* fld, float* const* mat, const BlockLayout& L,
                                     int step_i, int ts, const EqwpStagParams& p, cudaStream_t st);
// One staggered time step for the adjoint's forward replay: velocities read
// from v_in and written to v_out (with the stencil sums into acc), stresses s
// (order sxx, sxy, sxz, syy, syz, szz) updated in place.  One block, R = 1.
cudaError_t launch_eqwp_stag_step_replay(const float* const* v_in, float* const* s, float* const* v_out,
                                         float* const* acc, float* const* mat, const BlockLayout& L,
                                         int ts, const EqwpStagParams& p, cudaStream_t st);

// eqwp_tma.cu: the staggered stress stage with its inputs streamed through
// TMA rings, on the plain stage launch's tiles: eqwp_stress_tma_shape gives
// the CTA shape tx x ty of sub-step step_i; maps.v: vx, vy, vz with boxes of
// (4 tx + 8) x (ty + 4) cells; maps.o: sxx, syy, szz, sxy, sxz, syz, lambda,
// mu with boxes of 4 tx x ty cells.  In place on fld (the stresses);
// bit-identical to the plain-load stress stage.
struct EqwpStressMaps {
    CUtensorMap v[3];
    CUtensorMap o[8];
};
void eqwp_stress_tma_shape(const BlockLayout& L, int step_i, int* tx, int* ty);
cudaError_t launch_eqwp_stress_tma(const EqwpStressMaps& maps, int tx, float* const* fld, const BlockLayout& L,
                                   int step_i, float src_amp, const EqwpStagParams& p, int* status,
                                   cudaStream_t st);
// The stress stage alone (plain loads; in place): split 0 = every tile,
// 1 = only the tiles holding an owned cell within H of a face with a
// neighbour block (every cell the halo exchange reads), 2 = only the other
// tiles, which read no halo cell.
cudaError_t launch_eqwp_stag_stress(float* const* fld, float* const* mat, const BlockLayout& L, int step_i, int ts,
                                    const EqwpStagParams& p, int split, cudaStream_t st);
// The velocity stage alone (plain loads), for a step whose stress stage is
// launched separately.
cudaError_t launch_eqwp_stag_velocity(float* const* fld, float* const* mat, const BlockLayout& L, int step_i,
                                      const EqwpStagParams& p, cudaStream_t st);

// eqwp_fused.cu: one staggered time step in one pass, v^n, s^n -> v^{n+1},
// s^{n+1} (out of place).  maps: tensor maps of the six s^n fields (xx, xy,
// xz, yy, yz, zz) with boxes of eqwp_fused_box()^2 cells; sout in the same
// order.  status receives DEV_TIMEOUT if a bounded wait gave up.
struct StressMaps {
    CUtensorMap m[6];
};
size_t eqwp_fused_smem();
int eqwp_fused_box();
cudaError_t launch_eqwp_stag_fused(const StressMaps& maps, const float* const* vin, float* const* vout,
                                   float* const* sout, float* const* mat, const BlockLayout& L, int step_i,
                                   int ts, const EqwpStagParams& p, int* status, cudaStream_t st);

// adjoint.cu: receiver sampling / injection and one reverse step of the
// staggered scheme (tmp = vb[3], sb[6], q[6], w[3]; stress order xx, xy, xz,
// yy, yz, zz; v_n = forward v^n, acc_n = forward stencil sums of step n;
// last = step 0, whose stress-side half has no earlier step to feed).
cudaError_t adjoint_sample(const float* vy, const long long* d_idx, int nrec, float* out, cudaStream_t st);
cudaError_t adjoint_inject(float* vby, const long long* d_idx, int nrec, const float* res, cudaStream_t st);
cudaError_t adjoint_step(float* const* tmp, const float* const* v_n, const float* const* acc_n,
                         const float* const* mat, float* const* g, const BlockLayout& L, float dt_h,
                         bool last, bool fused, cudaStream_t st);
// g holds FP32 partial sums of the lambda, mu and b gradients; every
// adjoint_fold_steps() reverse steps (at step numbers that are multiples of
// it, and at step 0) adjoint_fold adds them into the FP64 gradients g64 and
// clears them.
int adjoint_fold_steps();
cudaError_t adjoint_fold(float* const* g, double* const* g64, const BlockLayout& L, cudaStream_t st);
cudaError_t adjoint_grad_out(const double* g, const float* buoy, int rho, const BlockLayout& L,
                             double* out, cudaStream_t st);

}  // namespace b2r
