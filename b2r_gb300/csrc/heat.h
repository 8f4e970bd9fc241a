// heat.h -- internal interface of the heat sweep kernels (heat.cu).
#pragma once
#include "b2r_common.cuh"

namespace b2r {

// Folded stencil weights: u' = a0*u + sum_k ax[k-1]*(u[x-k]+u[x+k]) + ... .
struct HeatCoef {
    float a0;
    float ax[4], ay[4], az[4];
};

HeatCoef heat_coef(int D, double alpha_dt, double dx, double dy, double dz);

// heat_adjoint.cu: the Laplacian of order 2D times alpha*dt/dx^2 per axis,
// L u = w0*u + sum_k wx[k-1]*(u[x-k]+u[x+k]) + ...; the conductivity-scaled
// step u' = u + kappa * L u on the interior window of one block, and one
// reverse step of its adjoint (lam: adjoint of u^{n+1}, updated to that of
// u^n; yb: scratch, zero outside the window; g += lam * L u^n in FP64).
struct HeatLap {
    float w0;
    float wx[4], wy[4], wz[4];
};
HeatLap heat_lap(int D, double alpha_dt, double dx, double dy, double dz);
cudaError_t launch_heat_kappa_step(const float* in, float* out, const float* kappa, const BlockLayout& L, int D,
                                   const HeatLap& c, cudaStream_t st);
cudaError_t launch_heat_adjoint_step(float* lam, float* yb, const float* u, const float* kappa, double* g,
                                     const BlockLayout& L, int D, const HeatLap& c, cudaStream_t st);
cudaError_t launch_fill(float* p, size_t n, float v, cudaStream_t st);
// TMA box of one ring slot (cells): width and height for radius D.
int heat_box_w();
int heat_box_h(int D);
// One sub-step (shrink D*(step_i+1)) of every block: reads the blocks
// through `tin` (a tensor map over the input buffer), writes `out`.
// Launch schedule knobs (the autotuner's search space).
struct HeatTune {
    int zchunk = 0;        // output planes per work unit; 0 = 16 (fewer for small grids)
    int ctas_per_sm = 0;   // 0 = one CTA per unit; k > 0 = persistent, k CTAs per SM
    int pdl = 1;           // programmatic dependent launch on the stream
    int tblock = 2;        // time steps per HBM pass: radius 1 (2 = heat2.cu, 3-4 = heat_tb.cu), radius 2 (2 = heat_tb2.cu, with r2)
    int zchunk2 = 0;       // output planes per unit of the several-step kernels (0 = 16 / 64)
    int tb16 = 0;          // two steps per pass: 0 = heat2.cu (8-warp CTAs), 1 = heat_tb.cu (16 warps)
    int tbn = 0;           // heat_tb.cu tiles: 0 = 128 x 32 cells, 1 = 64 x 64 cells
    int r2 = 0;            // radius 2: 1 = two steps per pass (heat_tb2.cu) when tblock >= 2
};

// One sub-step of every block: units (block, z-chunk, tile row, tile column)
// dealt round-robin to the CTAs.
cudaError_t launch_heat_substep(const CUtensorMap* tin, float* out, const BlockLayout& L, int D,
                                int step_i, const HeatCoef& c, int* status, cudaStream_t st,
                                const HeatTune& tune = HeatTune());

// Two sub-steps (step_i, step_i+1) of radius 1 per launch (heat2.cu).  The
// tensor map must have the box heat2_box_w() x heat2_box_h().
int heat2_box_w();
int heat2_box_h();
cudaError_t launch_heat_substep2(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                                 const HeatCoef& c, int* status, cudaStream_t st, int zchunk);

// Two sub-steps (step_i, step_i+1) of radius 2 per launch (heat_tb2.cu),
// on tiles of 64 x 64 cells.  The tensor map must have the box
// heat_tb2_box_w() x heat_tb2_box_h().
int heat_tb2_box_w();
int heat_tb2_box_h();
cudaError_t launch_heat_substep_tb2(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                                    const HeatCoef& c, int* status, cudaStream_t st, int zchunk);

// T = 2, 3 or 4 sub-steps (step_i .. step_i+T-1) of radius 1 per launch
// (heat_tb.cu), on tiles of 128 x 32 cells (narrow = 0) or 64 x 64 cells
// (narrow = 1).  The tensor map must have the box heat_tb_box_w(narrow) x
// heat_tb_box_h(narrow).
int heat_tb_box_w(int narrow);
int heat_tb_box_h(int narrow);
cudaError_t launch_heat_substep_tb(int T, int narrow, const CUtensorMap* tin, float* out, const BlockLayout& L,
                                   int step_i, const HeatCoef& c, int* status, cudaStream_t st, int zchunk);

}  // namespace b2r
