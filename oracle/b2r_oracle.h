/*
 * b2r_oracle.h -- CPU restatement of the B2R stencil hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests compare the CUDA implementation in
 * b2r_gb300/csrc against this library; only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it.  The product path never calls it.
 *
 * Storage convention (identical to the reference, heat-3D.cpp:42-45):
 * a block of nx*ny*nz cells, x fastest, index z*nx*ny + y*nx + x.
 *
 * Update regions.  A sub-step (or a stage of one) with shrink s updates the
 * cells whose distance to every block face is >= s, the B2R shrinking
 * region of heat-3D.cu:191,268 / eqwp.cu:83 ([D(i+1), N-1-D(i+1)]).
 * "edge" is a bit mask: bit 0 = low-x face of the block is the domain
 * boundary, bit 1 = high-x, bits 2/3 = y, bits 4/5 = z.  On a boundary face
 * the H-deep halo is the fixed (Dirichlet) shell and is never updated: the
 * mask of fdm_heat_diffuse_delta1_verify (heat-3D.cu:81-114) generalised to
 * any stencil radius and halo depth.
 */
#ifndef B2R_ORACLE_H
#define B2R_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* region of a stage with shrink s along one axis (both ends inclusive) */
void orc_region(int n, int s, int H, int lo_edge, int hi_edge, int* lo, int* hi);

/* ---- heat ---------------------------------------------------------------- */
/* One explicit heat sub-step (shrink D*(i+1)) with the reference's mixed
 * precision: float storage, float stencil sums, double weighting
 * (heat-3D.cu:228-231, 315-318, 410-413, 514-517; heat-3D.cpp:57-60).
 * Cells outside the region are not written. */
void orc_heat_substep_f32(const float* in, float* out, int nx, int ny, int nz,
                          int D, double alpha_dt, double dx, double dy, double dz,
                          int i, int H, int edge);
/* The same scheme entirely in FP64 with exact rational coefficients. */
void orc_heat_substep_f64(const double* in, double* out, int nx, int ny, int nz,
                          int D, double alpha_dt, double dx, double dy, double dz,
                          int i, int H, int edge);
/* nsteps steps over one domain stored with an H-deep fixed shell (i=0, all
 * faces on the boundary), ping-pong in an internal buffer. */
void orc_heat_run_f32(float* field, int nx, int ny, int nz, int D,
                      double alpha_dt, double dx, double dy, double dz,
                      int H, int nsteps, int nthreads);
void orc_heat_run_f64(double* field, int nx, int ny, int nz, int D,
                      double alpha_dt, double dx, double dy, double dz,
                      int H, int nsteps, int nthreads);
/* Mirror of heat_3D_cpu_main (heat-3D.cpp:136-184): R sub-steps on one
 * block with the reference's OpenMP loop nest (x outer, z descending inner),
 * ping-pong, odd-R copy-back of planes [R*D, nz-R*D).  Delta 2-4 use the GPU
 * formulas over in-bounds regions.  Returns wall seconds of the sub-steps. */
double orc_heat_cpu_main(float* h_in, int R, int D, int nx, int ny, int nz,
                         double alpha_dt, double dx, double dy, double dz,
                         int nthreads);

/* ---- 3-D Game of Life ---------------------------------------------------- */
/* One generation (shrink i+1) on a block (gol-3D.cu:83-99): 26-neighbour
 * sum; a live cell with <=1 or >=8 live neighbours dies, a dead cell with
 * exactly 5 is born, every other cell keeps its state. */
void orc_gol_substep(const uint8_t* in, uint8_t* out, int nx, int ny, int nz,
                     int i, int H, int edge);
/* nsteps generations on an nx*ny*nz torus (no shell). */
void orc_gol_run_periodic(uint8_t* grid, int nx, int ny, int nz, int nsteps,
                          int nthreads);

/* ---- elastic wave, reference (collocated FD4) physics --------------------- */
/* f[0..9] = vx, vy, vz, sxx, sxy, sxz, syy, syz, szz, disp.  One sub-step:
 * stress stage (shrink 4i+2) then vx, vy (+disp), vz (shrink 4i+4), in the
 * order of eqwp.cu:679-684 and the mixed precision of eqwp.cu:131-138,
 * 225-235, 320-327, 450-473.  Body force fval is added to the vy/disp update
 * on plane y == fy for x in [fx0,fx1), z in [fz0,fz1) while ts < fsteps
 * (eqwp.cu:135,229-231,561-566). */
void orc_eqwp_ref_substep_f32(float* const* f, int nx, int ny, int nz,
                              int i, int H, int edge, int ts,
                              int fy, int fx0, int fx1, int fz0, int fz1,
                              double fval, int fsteps);
void orc_eqwp_ref_substep_f64(double* const* f, int nx, int ny, int nz,
                              int i, int H, int edge, int ts,
                              int fy, int fx0, int fx1, int fz0, int fz1,
                              double fval, int fsteps);

/* ---- elastic wave, staggered-grid FD4 with heterogeneous material --------- */
/* f[0..8] = vx, vy, vz, sxx, sxy, sxz, syy, syz, szz; m[0..2] = lambda, mu,
 * buoyancy (1/rho) per cell.  One step: velocity stage (shrink 4i+2), stress
 * stage (shrink 4i+4), then sxx, syy, szz += src at cell
 * (src_x,src_y,src_z) when that cell is in the stress region. */
void orc_eqwp_stag_step_f32(float* const* f, const float* const* m,
                            int nx, int ny, int nz, double dt, double dx,
                            int i, int H, int edge, int src_x, int src_y, int src_z,
                            double src);
void orc_eqwp_stag_step_f64(double* const* f, const double* const* m,
                            int nx, int ny, int nz, double dt, double dx,
                            int i, int H, int edge, int src_x, int src_y, int src_z,
                            double src);

/* One reverse step of the discrete adjoint of orc_eqwp_stag_step_f64 on the
 * window [lo, hi] (inclusive, per axis): tmp = vb[3] (vx, vy, vz), sb[6]
 * (xx, xy, xz, yy, yz, zz); fv = forward v after the step (3); fs = forward
 * stress before the step (6, same order); m = lambda, mu, buoyancy; g =
 * gradients wrt lambda, mu, buoyancy (accumulated).  k = dt/dx. */
void orc_eqwp_stag_adjoint_step_f64(double* const* tmp, const double* const* fv,
                                    const double* const* fs, const double* const* m,
                                    double* const* g, int nx, int ny, int nz, double k,
                                    const int* lo, const int* hi);

#ifdef __cplusplus
}
#endif
#endif
