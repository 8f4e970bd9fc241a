/*
 * b2r.h -- C ABI of libb2r: the B2R stencil hot path on one GB300 (sm_103a).
 *
 * Plain C: pointers, sizes and ints only.  A cudaStream_t is passed as
 * void*.  Every entry point returns a b2r_status; nothing calls exit().
 *
 * Model: the global domain of env[0] x env[1] x env[2] interior cells is
 * tiled by blocks[0] x blocks[1] x blocks[2] subdomains (the reference's
 * BLOCK_DIM_X/Y/Z, b2r.cpp:139-146), each stored on the device as a padded
 * block of (B + 2H) cells per axis with B = env/blocks and halo depth
 * H = R * (cells consumed by one time step) -- the reference's
 * B2R_BLOCK_SIZE_* = B + 2*B2R_D*B2R_R (b2r.cpp:61-64).  One period = one
 * halo exchange between the resident subdomains (device-side
 * boundary_updating, b2r_halo_sync.cu:442) followed by R time steps during
 * which the valid region of every block shrinks (heat-3D.cu:191).
 *
 * Host data layout (identical to the reference, heat-3D.cpp:42-45): x
 * fastest, index z*nx*ny + y*nx + x.  A "domain array" is the global field:
 * for B2R_BC_SHELL it carries a fixed shell of `shell` = D cells around the
 * interior ((env+2D) cells per axis, e.g. 130^3 for a 128^3 heat interior);
 * for B2R_BC_PERIODIC it is the bare torus (env cells per axis).
 *
 * Threads: distinct handles (and batches) may be driven from distinct host
 * threads at once, each on its own stream; the library's process-wide state
 * (kernel setup, autotuner caches, the launch counter) is locked or atomic.
 * One handle is not to be used by two threads at a time.
 */
#ifndef B2R_H
#define B2R_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    B2R_OK = 0,
    B2R_ERR_ARG = 1,      /* invalid argument or configuration */
    B2R_ERR_CUDA = 2,     /* a CUDA runtime call failed */
    B2R_ERR_OOM = 3,      /* device allocation failed */
    B2R_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up */
    B2R_ERR_STATE = 5     /* call not valid in the handle's current state */
} b2r_status;

typedef enum {
    B2R_MODEL_HEAT = 1,       /* fdm_heat_diffuse_delta1..4 (heat-3D.cu:173-521) */
    B2R_MODEL_GOL = 2,        /* gol_3d_kernel (gol-3D.cu:30-102) */
    B2R_MODEL_EQWP_REF = 3,   /* eqwp_fd4_stress + eqwp_fd4_v{x,y,z} (eqwp.cu:60-477) */
    B2R_MODEL_EQWP_STAG = 4   /* staggered-grid FD4 elastic wave, layered material */
} b2r_model;

typedef enum { B2R_BC_SHELL = 0, B2R_BC_PERIODIC = 1 } b2r_boundary;

/* Field ids.  Heat and GoL have one field (0).  Elastic wave: */
enum {
    B2R_F_VX = 0, B2R_F_VY, B2R_F_VZ, B2R_F_SXX, B2R_F_SXY, B2R_F_SXZ,
    B2R_F_SYY, B2R_F_SYZ, B2R_F_SZZ, B2R_F_DISP,      /* 9: displacement (REF) */
    B2R_F_LAMBDA = 16, B2R_F_MU = 17, B2R_F_BUOY = 18, /* material (STAG) */
    B2R_F_KAPPA = 19                                   /* heat: conductivity of the
                                                          differentiable form (default 1) */
};

typedef struct {
    int model;          /* b2r_model */
    int env[3];         /* ENV_DIM_X/Y/Z (b2r_config.h:6-8) */
    int blocks[3];      /* BLOCK_DIM_X/Y/Z; env[a] % blocks[a] == 0 (b2r.cpp:154) */
    int R;              /* B2R_R >= 1; R*D <= min(B)/2 (b2r.cpp:54) */
    int D;              /* stencil radius: heat 1..4 (B2R_D), GoL 1, eqwp 2 */
    int boundary;       /* b2r_boundary */
    /* heat: u += alpha_dt*(Lx/dx^2 + Ly/dy^2 + Lz/dz^2) (heat-3D.cu:228-231) */
    double alpha_dt, dx, dy, dz;
    /* eqwp STAG: time step and grid spacing; source cell (global interior
       coordinates) for the explosive source */
    double dt, h;
    int src[3];
} b2r_config;

typedef struct b2r_handle b2r_handle;

/* ---- life cycle ------------------------------------------------------- */
/* Validates cfg as simu_env_init does (b2r.cpp:47-67, 154-159) and allocates
 * every device field.  Replaces b2r_sync_init (b2r_halo_sync.cu:74) and
 * eqwp_cuda_init (eqwp.cu:515). */
b2r_status b2r_create(const b2r_config* cfg, b2r_handle** out);
/* Replaces b2r_sync_finalize (b2r_halo_sync.cu:121) / eqwp_cuda_finalize
 * (eqwp.cu:592). */
b2r_status b2r_destroy(b2r_handle* h);
const char* b2r_last_error(const b2r_handle* h);
/* All work of the handle is enqueued on this stream (default: legacy 0). */
b2r_status b2r_set_stream(b2r_handle* h, void* cuda_stream);
b2r_status b2r_synchronize(b2r_handle* h);

/* Geometry: padded block size per axis, halo depth H, host domain size per
 * axis, bytes per cell. */
b2r_status b2r_geometry(const b2r_handle* h, int block_n[3], int* halo,
                        int domain_n[3], int* cell_bytes);
/* Cells advanced per time step over the whole domain (env product). */
int64_t b2r_cells(const b2r_handle* h);

/* ---- data movement ------------------------------------------------------ */
/* A domain array is domain_n[0]*domain_n[1]*domain_n[2] cells (x fastest) of
 * cell_bytes each (b2r_geometry); the material and conductivity fields are
 * float32 whatever the model's cells.  The library reads or writes exactly
 * that many bytes through the pointer: a smaller buffer is the caller's bug,
 * it cannot be detected here. */
/* Load a domain array into every block (interiors, halos and shell).
 * src_is_device: 0 = host memory (pinned recommended), 1 = device memory.
 * Resets the time-step counter to 0.  The next b2r_step starts without a
 * halo exchange when every field's halos are current: they were before the
 * upload, or every field (not the material) has been uploaded since the
 * last step. */
b2r_status b2r_upload(b2r_handle* h, int field, const void* src, int src_is_device);
/* Gather the block interiors (and the shell) into a domain array. */
b2r_status b2r_download(b2r_handle* h, int field, void* dst, int dst_is_device);

/* Copy every padded block of a field, halos included, into a dense array of
 * blocks*Ngz*Ngy*Ngx cells (block index slowest, x fastest) -- the per-rank
 * blocks of the reference (B2R_BLOCK_SIZE_*, b2r.h:81-85) side by side. */
b2r_status b2r_download_blocks(b2r_handle* h, int field, void* dst, int dst_is_device);

/* ---- time stepping ------------------------------------------------------ */
/* Advance nsteps time steps: periods of one halo exchange of every field
 * (b2r.cpp:197-206) and R steps (b2r.cpp:215); a trailing partial period
 * runs fewer steps.  Asynchronous on the handle's stream. */
b2r_status b2r_step(b2r_handle* h, int nsteps);
/* Replay whole periods (halo exchange + R sub-steps, >= 32 time steps) from
 * CUDA graphs captured on first use (heat and Game of Life, when the handle
 * has a non-default stream).  Default on; results are identical either way. */
b2r_status b2r_set_graphs(b2r_handle* h, int enable);
/* Launch-schedule knobs of the heat sweep (the autotuner's search space). */
enum {
    B2R_TUNE_ZCHUNK = 1,       /* planes per work unit of the one-step sweep (0 = 16) */
    B2R_TUNE_CTAS_PER_SM = 2,  /* 0 = one CTA per unit, k = persistent k CTAs per SM */
    B2R_TUNE_PDL = 3,          /* programmatic dependent launch on / off */
    B2R_TUNE_TBLOCK = 4,       /* time steps per pass: heat of radius 1 takes up to tblock (2, 3
                                  or 4; default 2) steps per HBM pass and Game of Life
                                  (bit-sliced cells, tblock >= 2) up to four generations per L2
                                  pass, never across a halo exchange; byte cells need >= 4;
                                  1 = one step per pass */
    B2R_TUNE_ZCHUNK2 = 5,      /* planes per work unit of the several-step heat sweeps (0 = 16
                                  for two steps, 64 for three or four) */
    B2R_TUNE_EQWP_FUSED = 6,   /* staggered elastic wave: 1 = one-pass step, 0 = the velocity
                                  and stress stages as two passes (default); bit-identical */
    B2R_TUNE_GOL_BYTES = 7,    /* Game of Life one-generation kernel: 0 = bit-sliced cells
                                  (default), 1 = four byte cells per word; identical results */
    B2R_TUNE_ADJ_FUSED = 8,    /* elastic-wave adjoint: 1 = the stress adjoint and the lambda /
                                  mu gradients in one sweep (default), 0 = two kernels;
                                  bit-identical */
    B2R_TUNE_GOL_PUSH = 9,     /* Game of Life: 1 = a several-generation pass that ends a period
                                  also fills the next period's halos, so no gather runs between
                                  periods (block rows of a multiple of 32 cells; otherwise the
                                  gather runs); 0 = the gather (default, faster on this GPU so
                                  far); identical results */
    B2R_TUNE_TB16 = 10,        /* heat, two steps per pass: 0 = two 8-warp CTAs per SM (default),
                                  1 = the 16-warp kernel of three and four steps; bit-identical */
    B2R_TUNE_TB_NARROW = 11,   /* heat, the 16-warp several-step kernel: 0 = tiles of 128 x 32
                                  cells (default), 1 = 64 x 64 cells; bit-identical */
    B2R_TUNE_TB_R2 = 12,       /* heat radius 2: 1 = two steps per HBM pass (with TBLOCK >= 2) on
                                  64 x 64-cell tiles, 0 = one step per pass (default: the one-step
                                  sweep is faster on this GPU so far); bit-identical */
    B2R_TUNE_EQWP_TMA = 13,    /* staggered elastic wave, two-pass step: 1 = the stress stage with
                                  its inputs streamed through TMA rings, 0 = plain loads (default);
                                  bit-identical */
    B2R_TUNE_EQWP_OVERLAP = 14,/* staggered elastic wave, two-pass step on several blocks: 1 = the
                                  last stress stage of a period computes the tiles that the next
                                  halo exchange reads first, then that exchange runs on a second
                                  stream while the other tiles finish; 0 = the exchange at the
                                  period start (default: faster on one GPU so far); bit-identical */
    B2R_TUNE_GOL_ROWS = 15     /* Game of Life, the several-generation bit-sliced pass: output rows
                                  per band of a CTA at most (0 = 32, the default; a value at least
                                  the block height gives one band per block); identical results */
};
b2r_status b2r_set_tuning(b2r_handle* h, int key, int value);
/* Current value of a knob (after b2r_autotune: the schedule it picked). */
b2r_status b2r_get_tuning(const b2r_handle* h, int key, int* value);
/* Time every schedule candidate for trial_steps time steps on the live
 * fields, keep the fastest, restore the fields and the time step.  Heat:
 * time steps per pass x z-chunk length x persistent CTAs per SM x
 * programmatic dependent launch, best[3] = {zchunk, ctas_per_sm, pdl}.
 * Game of Life: generations per pass x bit-sliced / byte cells x period-end
 * halo fill x band height of the several-generation pass, best = {tblock,
 * gol_bytes, gol_push} (the band height: b2r_get_tuning).  Staggered elastic wave:
 * one-pass or two-pass step, the latter with the plain or TMA-streamed
 * stress stage and, on several blocks, with the halo exchange at the period
 * start or overlapped with the last stress stage, best = {tblock,
 * eqwp_fused, 0} (the other choices: b2r_get_tuning).  Results are
 * cached per (model, D, block size, block count) for the process and
 * applied to later handles of the same shape.  best may be NULL; *best_ms
 * gets the time per step (-1 if cached). */
b2r_status b2r_autotune(b2r_handle* h, int trial_steps, int best[3], double* best_ms);
/* Upload, b2r_step, download: the whole job through host buffers. */
b2r_status b2r_run_host(b2r_handle* h, int field, const void* host_in, int nsteps,
                        void* host_out);
/* b2r_run_host over count independent inputs of the same shape (field must
 * be 0): problem i is uploaded from host_in[i], stepped nsteps times and
 * downloaded to host_out[i], with the copy of the next input and of the
 * previous result overlapping the stepping (two copy streams, two device
 * buffers per direction).  A problem is every field of the model back to
 * back in field-id order: one domain array for heat and Game of Life; the
 * nine wavefield components (B2R_F_VX .. B2R_F_SZZ) of the staggered elastic
 * wave, and those and the displacement (ten) of the reference model, whose
 * material stays resident.  Pinned host buffers make the copies
 * asynchronous.  Returns when every result is on the host. */
b2r_status b2r_run_host_batch(b2r_handle* h, int field, const void* const* host_in, void* const* host_out,
                              int count, int nsteps);
/* Time steps done since the last upload. */
int64_t b2r_time_step(const b2r_handle* h);

/* Explosive source of the staggered model: amps[t] is added to sxx, syy and
 * szz of the source cell (cfg.src) after the stress update of time step t
 * (t < n).  Copied; n = 0 clears it. */
b2r_status b2r_set_source(b2r_handle* h, const float* amps, int n);

/* ---- B2R boundary update (b2r_halo_sync.cu) ------------------------------ */
/* Device-side X->Y->Z halo exchange of one field between the resident
 * subdomains.  _direct copies neighbour slabs straight into the halos
 * (boundary_updating_direct, b2r_halo_sync.cu:389-431); the staged form packs
 * every face slab into a device bounce buffer and unpacks it
 * (sub_matrix_pack/unpack_{x,y,z} + boundary_updating,
 * b2r_halo_sync.cu:195-379, 442-508).  Both give identical halos.
 * time_step is the reference's message-tag argument; it is recorded only. */
b2r_status b2r_boundary_updating_direct(b2r_handle* h, int time_step, int field);
b2r_status b2r_boundary_updating(b2r_handle* h, int time_step, int field);

/* Number of CUDA kernels this library has launched in this process. */
int64_t b2r_kernel_launches(void);

/* ---- reference-shaped per-block entries ---------------------------------- */
/* heat_3D_gpu_main (heat-3D.cu:583): R sub-steps of the order-D heat
 * stencil on one padded host block of Ngx*Ngy*Ngz cells with shrinking
 * region [D(i+1), N-1-D(i+1)], then the planes [R*D, Ngz-R*D) are copied
 * back into h_in.  edge_flag[3] in {-1,0,1} per axis as the reference
 * documents (-1 low face on the domain boundary, 1 high face, 0 inside);
 * NULL means 0,0,0.  On a boundary face the H = R*D deep halo is not updated
 * (fdm_heat_diffuse_delta1_verify, heat-3D.cu:81-114).  *gpu_seconds (may be
 * NULL) receives the device time of the sub-steps (cudaEvent, as
 * heat-3D.cu:595-641).  Coefficients as in b2r_config. */
b2r_status b2r_heat_3D_gpu_main(float* h_in, int R, int D, const char* edge_flag,
                                int Ngx, int Ngy, int Ngz, double alpha_dt,
                                double dx, double dy, double dz, void* cuda_stream,
                                double* gpu_seconds);
/* heat_3D_cpu_main (heat-3D.hpp:12, heat-3D.cpp:136-184) on the host cores:
 * the contract of b2r_heat_3D_gpu_main (same arguments, edge flags and
 * copy-back of planes [R*D, Ngz-R*D)), computed with the GPU sweep's float
 * operations in its order, so the result is bit-identical to
 * b2r_heat_3D_gpu_main's.  nthreads <= 0: every hardware thread.
 * *cpu_seconds (may be NULL) gets the wall time (heat-3D.cpp:141,181).
 * Touches no GPU; no GPU entry falls back to it. */
b2r_status b2r_heat_3D_cpu_main(float* h_in, int R, int D, const char* edge_flag, int Ngx, int Ngy, int Ngz,
                                double alpha_dt, double dx, double dy, double dz, int nthreads,
                                double* cpu_seconds);
/* The hybrid CPU+GPU form of one block (heat-3D.cpp:47,170): the block is
 * cut along z, the host cores compute the last cpu_planes result planes and
 * the GPU the others, at the same time; each side holds R*D planes of the
 * other's beyond the cut, so the R sub-steps need no exchange between them.
 * The result is bit-identical to b2r_heat_3D_gpu_main's.  cpu_planes = 0 is
 * the GPU alone, cpu_planes >= Ngz - 2*R*D the host alone.  A part's deep
 * halo never crosses a fixed z face: with edge_flag[2] = 1 a positive
 * cpu_planes below R*D is raised to R*D, and with edge_flag[2] = -1 a split
 * that would leave the GPU fewer than R*D result planes gives the host the
 * whole block.  *seconds (may be NULL) gets the wall time of the call. */
b2r_status b2r_heat_3D_hybrid_main(float* h_in, int R, int D, const char* edge_flag, int Ngx, int Ngy, int Ngz,
                                   double alpha_dt, double dx, double dy, double dz, int cpu_planes,
                                   int nthreads, void* cuda_stream, double* seconds);
/* gol_3D_gpu_main (gol-3D.cu:119): R generations on one padded host block,
 * region [i+1, N-2-i]; the whole block is copied back (gol-3D.cu:149). */
b2r_status b2r_gol_3D_gpu_main(uint8_t* h_in, int R, const char* edge_flag, int Ngx,
                               int Ngy, int Ngz, void* cuda_stream, double* gpu_seconds);
/* No counterpart in the reference.  The computation of b2r_heat_3D_gpu_main
 * for callers that cannot allocate device memory -- e.g. code running inside
 * a framework that owns all device memory through its own pool and forbids
 * raw cudaMalloc/cudaFree (whose implicit device-wide synchronisation would
 * stall its other streams).  d_in and d_out are device blocks of
 * Ngx*Ngy*Ngz floats (may be the same block); on return d_out holds d_in
 * with planes [R*D, Ngz-R*D) replaced by the result of R sub-steps.  The
 * ping-pong blocks live in a fixed 32 MiB device array inside the library
 * (held by every GPU that loads it until exit): a block is accepted when
 * P * Ngy * Ngz <= 4,194,304 cells, P being its row pitch padded as
 * b2r_heat_3D_gpu_main pads it (Ngx plus at least 12 cells, rounded up to a
 * multiple of 32) -- cubes up to 147^3 at R*D = 1; larger blocks are
 * rejected with B2R_ERR_ARG and a message on stderr.  All calls share that
 * array, so calls that overlap on the GPU race.  Every call looks up the
 * array's address on the current device; the first call on a device also
 * loads the library's device code there and should come before any stream
 * capture.  Synchronous on cuda_stream; allocates nothing. */
b2r_status b2r_heat_3D_gpu_main_noalloc(const float* d_in, float* d_out, int R, int D,
                                        const char* edge_flag, int Ngx, int Ngy, int Ngz,
                                        double alpha_dt, double dx, double dy, double dz,
                                        void* cuda_stream);
/* eqwp_gpu_main (eqwp.cu:661): R steps of the reference elastic-wave model on
 * the handle's fields (model B2R_MODEL_EQWP_REF), ts = the outer time step
 * (selects the body force, eqwp.cu:135).  Does not exchange halos. */
b2r_status b2r_eqwp_gpu_main(b2r_handle* h, int ts, int R, double* gpu_seconds);
/* write_block_data_bin / write_block_data (eqwp.cu:616-651): one padded
 * block of a float field (halos included, Ngx*Ngy*Ngz cells, x fastest) to
 * <dir>/<name>-<time_step>.bin as an int32[3] {Ngx, Ngy, Ngz} header and the
 * cells, or with text != 0 to <dir>/<name>-<time_step>.txt as "v," per cell
 * and one line per row.  name is "displacement" for B2R_F_DISP (the
 * reference's file) and otherwise the field's own name (u, kappa, vx .. szz,
 * lambda, mu, buoyancy); a block other than 0 appends "-b<block>".  dir NULL
 * is the working directory.  The path written is copied to path_out (may be
 * NULL) of path_cap bytes.  Game-of-Life cells are bytes: B2R_ERR_ARG. */
b2r_status b2r_write_block_data(b2r_handle* h, int field, int block, int time_step, const char* dir,
                                int text, char* path_out, int path_cap);

/* ---- adjoint of the staggered elastic wave (no reference counterpart) ---- */
/* Forward nsteps from the current fields and record vy at nrec receivers
 * (rec_xyz: 3*nrec global interior coordinates) after every step into
 * d_out[nsteps*nrec] (host).  One block, R = 1, model B2R_MODEL_EQWP_STAG. */
b2r_status b2r_eqwp_record(b2r_handle* h, int nsteps, int nrec, const int* rec_xyz, float* d_out);
/* Misfit J = 1/2 sum (d_syn - d_obs)^2 of the same recording and its
 * gradient with respect to lambda, mu and rho per interior cell (host
 * arrays of env cells, x fastest, FP64; any may be NULL), by the discrete
 * adjoint run backward in time.  The forward state is checkpointed every
 * ckpt_every steps (<= 0: once) and each segment is recomputed before its
 * reverse sweep.  Gradients accumulate in FP64.  d_syn (may be NULL) gets
 * the synthetic recording.  The fields end in an unspecified state. */
b2r_status b2r_eqwp_misfit_gradient(b2r_handle* h, int nsteps, int nrec, const int* rec_xyz,
                                    const float* d_obs, int ckpt_every, double* misfit,
                                    double* grad_lambda, double* grad_mu, double* grad_rho,
                                    float* d_syn);

/* ---- heat adjoint (no reference counterpart) ------------------------------ *
 * The differentiable heat step scales the stencil of fdm_heat_diffuse_deltaD
 * (heat-3D.cu:173-521) by a per-cell conductivity kappa (field
 * B2R_F_KAPPA, 1 everywhere unless uploaded): u' = u + kappa * (L u) on the
 * interior, with L the order-2D Laplacian times alpha*dt/dx^2 per axis.
 * b2r_step keeps the plain scheme; these two calls use kappa.  One block,
 * fixed shell (B2R_BC_SHELL), model B2R_MODEL_HEAT. */
/* Forward nsteps from the current field, recording u at nrec receivers after
 * every step into d_out[nsteps*nrec] (host). */
b2r_status b2r_heat_record(b2r_handle* h, int nsteps, int nrec, const int* rec_xyz, float* d_out);
/* Misfit J = 1/2 sum (d_syn - d_obs)^2 of that recording and dJ/dkappa per
 * interior cell (host, env cells, x fastest, FP64), by the discrete adjoint
 * backward in time with checkpoints every ckpt_every steps (<= 0: once) and
 * recomputation in between; FP64 accumulation.  d_syn may be NULL.  The
 * field ends in an unspecified state. */
b2r_status b2r_heat_misfit_gradient(b2r_handle* h, int nsteps, int nrec, const int* rec_xyz,
                                    const float* d_obs, int ckpt_every, double* misfit,
                                    double* grad_kappa, float* d_syn);

/* ---- batched instances (no reference counterpart) ------------------------ */
/* Many independent single-block heat domains of uneven sizes and stencil
 * orders advanced in one persistent launch driven by a device work queue of
 * (time step, instance, tile chunk) items, replayable from a CUDA graph.
 * Each instance is a domain array with a fixed shell of D cells
 * ((env+2D) cells per axis, reference layout) stepped nsteps times with the
 * heat scheme; results are identical to a plain b2r_step run of the same
 * instance. */
typedef struct {
    int env[3];                      /* interior cells per axis */
    int D;                           /* stencil radius 1..4 */
    int nsteps;                      /* time steps of this instance */
    double alpha_dt, dx, dy, dz;     /* heat coefficients as in b2r_config */
} b2r_batch_item;
typedef struct b2r_batch b2r_batch;

b2r_status b2r_batch_create(const b2r_batch_item* items, int n, b2r_batch** out);
b2r_status b2r_batch_destroy(b2r_batch* b);
const char* b2r_batch_last_error(void);
/* Domain array of instance i (caller order) into both of its buffers. */
b2r_status b2r_batch_upload(b2r_batch* b, int i, const float* src, int src_is_device,
                            void* cuda_stream);
/* Result of instance i after its nsteps (synchronous for host dst). */
b2r_status b2r_batch_download(b2r_batch* b, int i, float* dst, int dst_is_device,
                              void* cuda_stream);
/* Run every instance to its nsteps: one persistent launch (plus two counter
 * resets), captured once into a CUDA graph and replayed when use_graph != 0
 * and the stream is not the legacy default stream.  Asynchronous. */
b2r_status b2r_batch_run(b2r_batch* b, void* cuda_stream, int use_graph);
/* Wait for the stream and report a device-side timeout of the work queue. */
b2r_status b2r_batch_synchronize(b2r_batch* b, void* cuda_stream);
/* Total lattice-site updates of one run (sum of cells x steps). */
int64_t b2r_batch_lups(const b2r_batch* b);
/* Planes per work unit along z (0 = whole column). */
b2r_status b2r_batch_set_zchunk(b2r_batch* b, int zchunk);
/* Tile shape of the instances: 128 x 16, 64 x 32 or 32 x 64 cells (x by
 * y, for D <= 2; half the rows for D >= 3), by width 128, 64 or 32, for
 * every instance; 0 gives each instance the shape that computes the fewest
 * cells of its planes (the default at creation).  Instances of different
 * shapes share the one launch.  b2r_batch_tile returns the width shared by
 * every instance (0 if they differ), b2r_batch_instance_tile the width of
 * instance i (caller order). */
b2r_status b2r_batch_set_tile(b2r_batch* b, int width);
int b2r_batch_tile(const b2r_batch* b);
int b2r_batch_instance_tile(const b2r_batch* b, int i);
/* Time steps per HBM pass of the radius-1 instances: 2 puts every one of
 * them on two-step units (tiles of 128 x 16 cells read once per two steps,
 * the last unit of an odd step count taking one step; bit-identical to one
 * step per pass), 1 back on one-step units of their fewest-cells shape.
 * Instances of other radii keep their shapes.  b2r_batch_instance_pass_steps
 * returns 1 or 2 for instance i (caller order). */
b2r_status b2r_batch_set_pass_steps(b2r_batch* b, int steps);
int b2r_batch_instance_pass_steps(const b2r_batch* b, int i);
/* Autotune on the uploaded inputs (restored afterwards), timing whole runs:
 * the z-chunk cap (8, 16, 32, 64, whole column), then the tile shape and
 * steps per pass per (stencil order, size class) -- the instances of one
 * class (order D, interior width <= 64, <= 128 or wider) try each tile shape
 * and, at radius 1, the two-step units, while the others keep theirs --
 * then the z-chunk cap again. */
b2r_status b2r_batch_autotune(b2r_batch* b, void* cuda_stream, int* best_zchunk, double* best_ms);

/* ---- batched elastic-wave instances (no reference counterpart) ----------- */
/* Many staggered elastic-wave handles (B2R_MODEL_EQWP_STAG, one block each,
 * fixed shell) of uneven sizes advanced in one persistent launch driven by a
 * device work queue of (stage round, instance, tile chunk) items: a time step
 * of an instance is its velocity stage then its stress stage, each waiting
 * for the instance's previous stage to finish everywhere.  Each run advances
 * handle i by nsteps[i] steps from its current time step, in place, with its
 * own material and source; results are identical to b2r_step on each handle
 * with the two-pass step.  The batch keeps pointers to the handles: they must
 * outlive it.  A run is ordered after the work already queued on the
 * handles' streams, and the work queued on them afterwards after the run
 * (events, no host wait), so the handles are used as usual around runs
 * (b2r_upload, b2r_download, b2r_step, b2r_time_step). */
typedef struct b2r_eqwp_batch b2r_eqwp_batch;
b2r_status b2r_eqwp_batch_create(b2r_handle* const* handles, const int* nsteps, int n, b2r_eqwp_batch** out);
b2r_status b2r_eqwp_batch_destroy(b2r_eqwp_batch* b);
const char* b2r_eqwp_batch_last_error(void);
/* One run on the stream (asynchronous): the per-step source increments are
 * copied first, then the persistent launch (captured once into a CUDA graph
 * and replayed when use_graph != 0 and the stream is not the legacy default
 * stream); every handle's time step advances by its nsteps. */
b2r_status b2r_eqwp_batch_run(b2r_eqwp_batch* b, void* cuda_stream, int use_graph);
/* Wait for the stream and report a device-side timeout of the work queue. */
b2r_status b2r_eqwp_batch_synchronize(b2r_eqwp_batch* b, void* cuda_stream);
/* Lattice-site updates of one run (sum of interior cells x steps). */
int64_t b2r_eqwp_batch_lups(const b2r_eqwp_batch* b);
/* Planes per work unit along z (0 = whole column).  Default: 8 when units
 * of 32 planes would give fewer than 8 per resident CTA in a round (small
 * instances), else 32. */
b2r_status b2r_eqwp_batch_set_zchunk(b2r_eqwp_batch* b, int zchunk);

/* ---- diagnostics (no reference counterpart) ------------------------------- *
 * Run the device-side failure path once: a one-CTA kernel waits with the
 * library's bounded wait for an mbarrier phase that nothing completes, gives
 * up after limit_ms (0 < limit_ms <= 10000), reports through a status word
 * and exits.  Returns B2R_ERR_TIMEOUT when the path works; the context stays
 * usable. */
b2r_status b2r_selfcheck_bounded_wait(double limit_ms, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
