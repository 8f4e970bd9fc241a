/*
 * b2r_oracle.c -- CPU restatement of the B2R stencil hot path.
 *
 * TEST INFRASTRUCTURE ONLY: what the tests compare the CUDA path against,
 * never part of it.
 * Built with -ffp-contract=off so that float and double expressions are
 * evaluated exactly as written on x86-64 and on aarch64 alike (the
 * reference's CPU build has no FMA contraction on x86-64 either).
 *
 * Every function cites the reference lines whose arithmetic it restates.
 */
#include "b2r_oracle.h"
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(x, y, z) ((size_t)(z) * (size_t)nx * (size_t)ny + (size_t)(y) * (size_t)nx + (size_t)(x))

static double now_sec(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

void orc_region(int n, int s, int H, int lo_edge, int hi_edge, int* lo, int* hi)
{
    int l = s, h = n - 1 - s;
    /* the fixed shell never goes stale: on a boundary face the window is the
     * whole interior side, whatever the shrink */
    if (lo_edge) l = H;
    if (hi_edge) h = n - 1 - H;
    *lo = l;
    *hi = h;
}

static void region3(int nx, int ny, int nz, int s, int H, int edge, int lo[3], int hi[3])
{
    orc_region(nx, s, H, edge & 1, (edge >> 1) & 1, &lo[0], &hi[0]);
    orc_region(ny, s, H, (edge >> 2) & 1, (edge >> 3) & 1, &lo[1], &hi[1]);
    orc_region(nz, s, H, (edge >> 4) & 1, (edge >> 5) & 1, &lo[2], &hi[2]);
}

/* ------------------------------------------------------------------------ */
/* heat                                                                      */
/* ------------------------------------------------------------------------ */

/* float stencil coefficients exactly as the reference spells them
 * (heat-3D.cu:15-28): float literals, float divisions. */
static const float K2A = -1.f / 12.f, K2B = 4.f / 3.f, K2C = -2.5f;
static const float K3A = 1.f / 90.f, K3B = -3.f / 20.f, K3C = 1.5f, K3D = -49.f / 18.f;
static const float K4A = -1.f / 560.f, K4B = 8.f / 315.f, K4C = -0.2f, K4D = 1.6f,
                   K4E = -205.f / 72.f;

/* float sum of one axis: p points at the centre, s is the stride of the axis */
static inline float axis_f32(const float* p, ptrdiff_t s, int D)
{
    float c = p[0];
    switch (D) {
    case 1: /* heat-3D.cu:229 : (m - 2*c + p) */
        return p[-s] - 2 * c + p[s];
    case 2: /* heat-3D.cu:316 */
        return K2A * (p[-2 * s] + p[2 * s]) + K2B * (p[-s] + p[s]) + K2C * c;
    case 3: /* heat-3D.cu:411 */
        return K3A * (p[-3 * s] + p[3 * s]) + K3B * (p[-2 * s] + p[2 * s]) +
               K3C * (p[-s] + p[s]) + K3D * c;
    default: /* heat-3D.cu:515 */
        return K4A * (p[-4 * s] + p[4 * s]) + K4B * (p[-3 * s] + p[3 * s]) +
               K4C * (p[-2 * s] + p[2 * s]) + K4D * (p[-s] + p[s]) + K4E * c;
    }
}

static inline double axis_f64(const double* p, ptrdiff_t s, int D)
{
    double c = p[0];
    switch (D) {
    case 1:
        return p[-s] - 2.0 * c + p[s];
    case 2:
        return (-1.0 / 12.0) * (p[-2 * s] + p[2 * s]) + (4.0 / 3.0) * (p[-s] + p[s]) +
               (-5.0 / 2.0) * c;
    case 3:
        return (1.0 / 90.0) * (p[-3 * s] + p[3 * s]) + (-3.0 / 20.0) * (p[-2 * s] + p[2 * s]) +
               (3.0 / 2.0) * (p[-s] + p[s]) + (-49.0 / 18.0) * c;
    default:
        return (-1.0 / 560.0) * (p[-4 * s] + p[4 * s]) + (8.0 / 315.0) * (p[-3 * s] + p[3 * s]) +
               (-1.0 / 5.0) * (p[-2 * s] + p[2 * s]) + (8.0 / 5.0) * (p[-s] + p[s]) +
               (-205.0 / 72.0) * c;
    }
}

/* heat-3D.cpp:57-60 / heat-3D.cu:228-231: c + (Alpha*Dt)*(Lx/(Dx*Dx) + ...)
 * with the float axis sums promoted to double. */
static inline float heat_cell_f32(const float* p, ptrdiff_t sy, ptrdiff_t sz, int D,
                                  double adt, double dx2, double dy2, double dz2)
{
    float lx = axis_f32(p, 1, D);
    float ly = axis_f32(p, sy, D);
    float lz = axis_f32(p, sz, D);
    return (float)(p[0] + adt * (lx / dx2 + ly / dy2 + lz / dz2));
}

static inline double heat_cell_f64(const double* p, ptrdiff_t sy, ptrdiff_t sz, int D,
                                   double adt, double dx2, double dy2, double dz2)
{
    double lx = axis_f64(p, 1, D);
    double ly = axis_f64(p, sy, D);
    double lz = axis_f64(p, sz, D);
    return p[0] + adt * (lx / dx2 + ly / dy2 + lz / dz2);
}

void orc_heat_substep_f32(const float* in, float* out, int nx, int ny, int nz,
                          int D, double alpha_dt, double dx, double dy, double dz,
                          int i, int H, int edge)
{
    int lo[3], hi[3];
    region3(nx, ny, nz, D * (i + 1), H, edge, lo, hi);
    const ptrdiff_t sy = nx, sz = (ptrdiff_t)nx * ny;
    const double dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
#pragma omp parallel for schedule(static)
    for (int z = lo[2]; z <= hi[2]; z++)
        for (int y = lo[1]; y <= hi[1]; y++)
            for (int x = lo[0]; x <= hi[0]; x++) {
                size_t id = IDX(x, y, z);
                out[id] = heat_cell_f32(in + id, sy, sz, D, alpha_dt, dx2, dy2, dz2);
            }
}

void orc_heat_substep_f64(const double* in, double* out, int nx, int ny, int nz,
                          int D, double alpha_dt, double dx, double dy, double dz,
                          int i, int H, int edge)
{
    int lo[3], hi[3];
    region3(nx, ny, nz, D * (i + 1), H, edge, lo, hi);
    const ptrdiff_t sy = nx, sz = (ptrdiff_t)nx * ny;
    const double dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
#pragma omp parallel for schedule(static)
    for (int z = lo[2]; z <= hi[2]; z++)
        for (int y = lo[1]; y <= hi[1]; y++)
            for (int x = lo[0]; x <= hi[0]; x++) {
                size_t id = IDX(x, y, z);
                out[id] = heat_cell_f64(in + id, sy, sz, D, alpha_dt, dx2, dy2, dz2);
            }
}

static void set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

void orc_heat_run_f32(float* field, int nx, int ny, int nz, int D,
                      double alpha_dt, double dx, double dy, double dz,
                      int H, int nsteps, int nthreads)
{
    set_threads(nthreads);
    size_t n = (size_t)nx * ny * nz;
    float* tmp = (float*)malloc(n * sizeof(float));
    memcpy(tmp, field, n * sizeof(float));
    float *a = field, *b = tmp;
    for (int s = 0; s < nsteps; s++) {
        orc_heat_substep_f32(a, b, nx, ny, nz, D, alpha_dt, dx, dy, dz, 0, H, 63);
        float* t = a; a = b; b = t;
    }
    if (a != field) memcpy(field, a, n * sizeof(float));
    free(tmp);
}

void orc_heat_run_f64(double* field, int nx, int ny, int nz, int D,
                      double alpha_dt, double dx, double dy, double dz,
                      int H, int nsteps, int nthreads)
{
    set_threads(nthreads);
    size_t n = (size_t)nx * ny * nz;
    double* tmp = (double*)malloc(n * sizeof(double));
    memcpy(tmp, field, n * sizeof(double));
    double *a = field, *b = tmp;
    for (int s = 0; s < nsteps; s++) {
        orc_heat_substep_f64(a, b, nx, ny, nz, D, alpha_dt, dx, dy, dz, 0, H, 63);
        double* t = a; a = b; b = t;
    }
    if (a != field) memcpy(field, a, n * sizeof(double));
    free(tmp);
}

/* heat-3D.cpp:48-62 loop nest: parallel over x, then y, z descending. */
static void cpu_ref_nest_substep(const float* in, float* out, int nx, int ny, int nz,
                                 int D, double adt, double dx2, double dy2, double dz2, int i)
{
    const int s = D * (i + 1);
    const ptrdiff_t sy = nx, sz = (ptrdiff_t)nx * ny;
#pragma omp parallel for
    for (int ix = s; ix <= nx - 1 - s; ix++)
        for (int iy = s; iy <= ny - 1 - s; iy++)
            for (int iz = nz - 1 - s; iz >= s; iz--) {
                size_t id = IDX(ix, iy, iz);
                out[id] = heat_cell_f32(in + id, sy, sz, D, adt, dx2, dy2, dz2);
            }
}

double orc_heat_cpu_main(float* h_in, int R, int D, int nx, int ny, int nz,
                         double alpha_dt, double dx, double dy, double dz, int nthreads)
{
    set_threads(nthreads);
    size_t n = (size_t)nx * ny * nz;
    float* p_in = h_in;
    float* p_out = (float*)malloc(n * sizeof(float));
    memcpy(p_out, h_in, n * sizeof(float));
    double t0 = now_sec();
    for (int i = 0; i < R; i++) {
        cpu_ref_nest_substep(p_in, p_out, nx, ny, nz, D, alpha_dt, dx * dx, dy * dy, dz * dz, i);
        float* t = p_in; p_in = p_out; p_out = t;
    }
    double t1 = now_sec();
    /* heat-3D.cpp:172-179 */
    if (R % 2) {
        size_t off = (size_t)R * D * nx * ny;
        memcpy(h_in + off, p_in + off, sizeof(float) * (size_t)nx * ny * (nz - 2 * R * D));
        free(p_in);
    } else {
        free(p_out);
    }
    return t1 - t0;
}

/* ------------------------------------------------------------------------ */
/* Game of Life                                                              */
/* ------------------------------------------------------------------------ */

/* gol-3D.cu:93-99 rule, with "no rule fires" meaning "keep current". */
static inline uint8_t gol_rule(uint8_t cur, int cnt)
{
    if (cur && cnt <= 1) return 0;
    if (!cur && cnt == 5) return 1;
    if (cur && cnt >= 8) return 0;
    return cur;
}

void orc_gol_substep(const uint8_t* in, uint8_t* out, int nx, int ny, int nz,
                     int i, int H, int edge)
{
    int lo[3], hi[3];
    region3(nx, ny, nz, i + 1, H, edge, lo, hi);
#pragma omp parallel for schedule(static)
    for (int z = lo[2]; z <= hi[2]; z++)
        for (int y = lo[1]; y <= hi[1]; y++)
            for (int x = lo[0]; x <= hi[0]; x++) {
                int cnt = 0; /* gol-3D.cu:83-91: 26 neighbours */
                for (int dz = -1; dz <= 1; dz++)
                    for (int dy = -1; dy <= 1; dy++)
                        for (int dx = -1; dx <= 1; dx++)
                            if (dx | dy | dz) cnt += in[IDX(x + dx, y + dy, z + dz)];
                out[IDX(x, y, z)] = gol_rule(in[IDX(x, y, z)], cnt);
            }
}

void orc_gol_run_periodic(uint8_t* grid, int nx, int ny, int nz, int nsteps, int nthreads)
{
    set_threads(nthreads);
    size_t n = (size_t)nx * ny * nz;
    uint8_t* tmp = (uint8_t*)malloc(n);
    uint8_t *a = grid, *b = tmp;
    for (int s = 0; s < nsteps; s++) {
#pragma omp parallel for schedule(static)
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) {
                    int cnt = 0;
                    for (int dz = -1; dz <= 1; dz++) {
                        int zz = (z + dz + nz) % nz;
                        for (int dy = -1; dy <= 1; dy++) {
                            int yy = (y + dy + ny) % ny;
                            for (int dx = -1; dx <= 1; dx++) {
                                int xx = (x + dx + nx) % nx;
                                if (dx | dy | dz) cnt += a[IDX(xx, yy, zz)];
                            }
                        }
                    }
                    b[IDX(x, y, z)] = gol_rule(a[IDX(x, y, z)], cnt);
                }
        uint8_t* t = a; a = b; b = t;
    }
    if (a != grid) memcpy(grid, a, n);
    free(tmp);
}

/* ------------------------------------------------------------------------ */
/* elastic wave, reference collocated physics (eqwp.cu)                      */
/* ------------------------------------------------------------------------ */

/* eqwp.cu:9-23 */
#define EQ_DT 0.5
#define EQ_DX 10.
#define EQ_INV_RHO 0.0005555555555555556
#define EQ_LAME1 32.00
#define EQ_LAME2 174.87
static const float EA = -1.f / 12.f, EB = 2.f / 3.f;

/* eqwp.cu:131: (a*(f[+2]-f[-2]) + b*(f[+1]-f[-1])) / Dx, stored to float */
static inline float d4_f32(const float* p, ptrdiff_t s)
{
    return (float)((EA * (p[2 * s] - p[-2 * s]) + EB * (p[s] - p[-s])) / EQ_DX);
}
static inline double d4_f64(const double* p, ptrdiff_t s)
{
    return ((-1.0 / 12.0) * (p[2 * s] - p[-2 * s]) + (2.0 / 3.0) * (p[s] - p[-s])) / EQ_DX;
}

enum { VX, VY, VZ, SXX, SXY, SXZ, SYY, SYZ, SZZ, DISP };

#define EQWP_REF_BODY(T, D4, CAST)                                                           \
    int lo[3], hi[3];                                                                        \
    const ptrdiff_t sy = nx, sz = (ptrdiff_t)nx * ny;                                        \
    /* stress stage, eqwp.cu:450-473 */                                                     \
    region3(nx, ny, nz, 4 * i + 2, H, edge, lo, hi);                                         \
    _Pragma("omp parallel for schedule(static)")                                             \
    for (int z = lo[2]; z <= hi[2]; z++)                                                     \
        for (int y = lo[1]; y <= hi[1]; y++)                                                 \
            for (int x = lo[0]; x <= hi[0]; x++) {                                           \
                size_t id = IDX(x, y, z);                                                    \
                T dvxx = D4(f[VX] + id, 1), dvyy = D4(f[VY] + id, sy), dvzz = D4(f[VZ] + id, sz); \
                T dvxy = D4(f[VX] + id, sy), dvyx = D4(f[VY] + id, 1);                       \
                T dvxz = D4(f[VX] + id, sz), dvzx = D4(f[VZ] + id, 1);                       \
                T dvyz = D4(f[VY] + id, sz), dvzy = D4(f[VZ] + id, sy);                      \
                T dsxx = CAST((EQ_LAME1 + 2 * EQ_LAME2) * dvxx + EQ_LAME1 * (dvyy + dvzz));  \
                T dsyy = CAST((EQ_LAME1 + 2 * EQ_LAME2) * dvyy + EQ_LAME1 * (dvxx + dvzz));  \
                T dszz = CAST((EQ_LAME1 + 2 * EQ_LAME2) * dvzz + EQ_LAME1 * (dvxx + dvyy));  \
                T dsxy = CAST(EQ_LAME2 * (dvxy + dvyx));                                     \
                T dsxz = CAST(EQ_LAME2 * (dvxz + dvzx));                                     \
                T dsyz = CAST(EQ_LAME2 * (dvyz + dvzy));                                     \
                f[SXX][id] = CAST(f[SXX][id] + EQ_DT * dsxx);                                \
                f[SXY][id] = CAST(f[SXY][id] + EQ_DT * dsxy);                                \
                f[SXZ][id] = CAST(f[SXZ][id] + EQ_DT * dsxz);                                \
                f[SYY][id] = CAST(f[SYY][id] + EQ_DT * dsyy);                                \
                f[SYZ][id] = CAST(f[SYZ][id] + EQ_DT * dsyz);                                \
                f[SZZ][id] = CAST(f[SZZ][id] + EQ_DT * dszz);                                \
            }                                                                                \
    /* velocity stage, eqwp.cu:131-138, 225-235, 320-327 */                                 \
    region3(nx, ny, nz, 4 * i + 4, H, edge, lo, hi);                                         \
    const T fv = CAST(fval);                                                                 \
    _Pragma("omp parallel for schedule(static)")                                             \
    for (int z = lo[2]; z <= hi[2]; z++)                                                     \
        for (int y = lo[1]; y <= hi[1]; y++)                                                 \
            for (int x = lo[0]; x <= hi[0]; x++) {                                           \
                size_t id = IDX(x, y, z);                                                    \
                T sx = D4(f[SXX] + id, 1), sxy_y = D4(f[SXY] + id, sy), sxz_z = D4(f[SXZ] + id, sz); \
                f[VX][id] = CAST(f[VX][id] + EQ_DT * EQ_INV_RHO * (sx + sxy_y + sxz_z));     \
                T sxy_x = D4(f[SXY] + id, 1), syy_y = D4(f[SYY] + id, sy), syz_z = D4(f[SYZ] + id, sz); \
                T sumy = sxy_x + syy_y + syz_z;                                              \
                if (y == fy && ts < fsteps && x >= fx0 && x < fx1 && z >= fz0 && z < fz1)    \
                    sumy = sumy + fv;                                                        \
                f[VY][id] = CAST(f[VY][id] + EQ_DT * EQ_INV_RHO * sumy);                     \
                f[DISP][id] = CAST(f[DISP][id] + EQ_DT * EQ_DT * EQ_INV_RHO * sumy);         \
                T sxz_x = D4(f[SXZ] + id, 1), syz_y = D4(f[SYZ] + id, sy), szz_z = D4(f[SZZ] + id, sz); \
                f[VZ][id] = CAST(f[VZ][id] + EQ_DT * EQ_INV_RHO * (sxz_x + syz_y + szz_z));  \
            }

#define CAST_F(v) ((float)(v))
#define CAST_D(v) ((double)(v))

void orc_eqwp_ref_substep_f32(float* const* f, int nx, int ny, int nz,
                              int i, int H, int edge, int ts,
                              int fy, int fx0, int fx1, int fz0, int fz1,
                              double fval, int fsteps)
{
    EQWP_REF_BODY(float, d4_f32, CAST_F)
}

void orc_eqwp_ref_substep_f64(double* const* f, int nx, int ny, int nz,
                              int i, int H, int edge, int ts,
                              int fy, int fx0, int fx1, int fz0, int fz1,
                              double fval, int fsteps)
{
    EQWP_REF_BODY(double, d4_f64, CAST_D)
}

/* ------------------------------------------------------------------------ */
/* elastic wave, staggered grid FD4 (no reference counterpart: new physics)  */
/* ------------------------------------------------------------------------ */
/* Grid: vx at (i+1/2,j,k), vy at (i,j+1/2,k), vz at (i,j,k+1/2), normal
 * stresses at (i,j,k), sxy at (i+1/2,j+1/2,k), sxz at (i+1/2,j,k+1/2), syz at
 * (i,j+1/2,k+1/2).  Forward difference Dp f(i) approximates df/dx at i+1/2,
 * backward Dm f(i) at i-1/2, 4th order: c1 = 9/8, c2 = -1/24. */
#define STAG_BODY(T, C1, C2)                                                                 \
    int lo[3], hi[3];                                                                        \
    const ptrdiff_t sy = nx, sz = (ptrdiff_t)nx * ny;                                        \
    const T idx_ = (T)(1.0 / dx), dt_ = (T)dt;                                               \
    region3(nx, ny, nz, 4 * i + 2, H, edge, lo, hi);                                         \
    _Pragma("omp parallel for schedule(static)")                                             \
    for (int z = lo[2]; z <= hi[2]; z++)                                                     \
        for (int y = lo[1]; y <= hi[1]; y++)                                                 \
            for (int x = lo[0]; x <= hi[0]; x++) {                                           \
                size_t id = IDX(x, y, z);                                                    \
                T b = m[2][id];                                                              \
                T ax = DP(f[SXX], id, 1) + DM(f[SXY], id, sy) + DM(f[SXZ], id, sz);          \
                T ay = DM(f[SXY], id, 1) + DP(f[SYY], id, sy) + DM(f[SYZ], id, sz);          \
                T az = DM(f[SXZ], id, 1) + DM(f[SYZ], id, sy) + DP(f[SZZ], id, sz);          \
                f[VX][id] += dt_ * b * (ax * idx_);                                          \
                f[VY][id] += dt_ * b * (ay * idx_);                                          \
                f[VZ][id] += dt_ * b * (az * idx_);                                          \
            }                                                                                \
    region3(nx, ny, nz, 4 * i + 4, H, edge, lo, hi);                                         \
    _Pragma("omp parallel for schedule(static)")                                             \
    for (int z = lo[2]; z <= hi[2]; z++)                                                     \
        for (int y = lo[1]; y <= hi[1]; y++)                                                 \
            for (int x = lo[0]; x <= hi[0]; x++) {                                           \
                size_t id = IDX(x, y, z);                                                    \
                T lam = m[0][id], mu = m[1][id];                                             \
                T exx = DM(f[VX], id, 1) * idx_;                                             \
                T eyy = DM(f[VY], id, sy) * idx_;                                            \
                T ezz = DM(f[VZ], id, sz) * idx_;                                            \
                T l2m = lam + 2 * mu;                                                        \
                f[SXX][id] += dt_ * (l2m * exx + lam * (eyy + ezz));                         \
                f[SYY][id] += dt_ * (l2m * eyy + lam * (exx + ezz));                         \
                f[SZZ][id] += dt_ * (l2m * ezz + lam * (exx + eyy));                         \
                f[SXY][id] += dt_ * mu * ((DP(f[VX], id, sy) + DP(f[VY], id, 1)) * idx_);    \
                f[SXZ][id] += dt_ * mu * ((DP(f[VX], id, sz) + DP(f[VZ], id, 1)) * idx_);    \
                f[SYZ][id] += dt_ * mu * ((DP(f[VY], id, sz) + DP(f[VZ], id, sy)) * idx_);   \
            }                                                                                \
    if (sx >= lo[0] && sx <= hi[0] && sy_ >= lo[1] && sy_ <= hi[1] && sz_ >= lo[2] &&         \
        sz_ <= hi[2]) {                                                                      \
        size_t id = IDX(sx, sy_, sz_);                                                       \
        T add = (T)(src);                                                                    \
        f[SXX][id] += add;                                                                   \
        f[SYY][id] += add;                                                                   \
        f[SZZ][id] += add;                                                                   \
    }

#define DP(F, id, s) (C1 * ((F)[(id) + (s)] - (F)[(id)]) + C2 * ((F)[(id) + 2 * (s)] - (F)[(id) - (s)]))
#define DM(F, id, s) (C1 * ((F)[(id)] - (F)[(id) - (s)]) + C2 * ((F)[(id) + (s)] - (F)[(id) - 2 * (s)]))

void orc_eqwp_stag_step_f32(float* const* f, const float* const* m,
                            int nx, int ny, int nz, double dt, double dx,
                            int i, int H, int edge, int sx, int sy_, int sz_,
                            double src)
{
    const float C1 = 9.f / 8.f, C2 = -1.f / 24.f;
    STAG_BODY(float, C1, C2)
}

void orc_eqwp_stag_step_f64(double* const* f, const double* const* m,
                            int nx, int ny, int nz, double dt, double dx,
                            int i, int H, int edge, int sx, int sy_, int sz_,
                            double src)
{
    const double C1 = 9.0 / 8.0, C2 = -1.0 / 24.0;
    STAG_BODY(double, C1, C2)
}

/* ------------------------------------------------------------------------ */
/* discrete adjoint of the staggered step (no reference counterpart)         */
/* ------------------------------------------------------------------------ */
/* Dp^T = -Dm and Dm^T = -Dp; fields outside the window are zero in q and w. */
static inline double dpd(const double* f, ptrdiff_t s)
{
    return 1.125 * (f[s] - f[0]) + (-1.0 / 24.0) * (f[2 * s] - f[-s]);
}
static inline double dmd(const double* f, ptrdiff_t s)
{
    return 1.125 * (f[0] - f[-s]) + (-1.0 / 24.0) * (f[s] - f[-2 * s]);
}

void orc_eqwp_stag_adjoint_step_f64(double* const* tmp, const double* const* fv,
                                    const double* const* fs, const double* const* m,
                                    double* const* g, int nx, int ny, int nz, double k,
                                    const int* lo, const int* hi)
{
    const size_t n = (size_t)nx * ny * nz;
    const ptrdiff_t sy = nx, sz = (ptrdiff_t)nx * ny;
    double* q[6];
    double* w[3];
    for (int i = 0; i < 6; ++i) q[i] = (double*)calloc(n, sizeof(double));
    for (int i = 0; i < 3; ++i) w[i] = (double*)calloc(n, sizeof(double));
    double** vb = (double**)tmp;
    double** sb = (double**)tmp + 3;
#define INW(x, y, z) ((x) >= lo[0] && (x) <= hi[0] && (y) >= lo[1] && (y) <= hi[1] && (z) >= lo[2] && (z) <= hi[2])
    /* stress stage: q = C sb on W, gradients of lambda and mu */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                if (!INW(x, y, z)) continue;
                size_t id = IDX(x, y, z);
                double l = m[0][id], mu = m[1][id];
                double tr = sb[0][id] + sb[3][id] + sb[5][id];
                q[0][id] = 2 * mu * sb[0][id] + l * tr;
                q[3][id] = 2 * mu * sb[3][id] + l * tr;
                q[5][id] = 2 * mu * sb[5][id] + l * tr;
                q[1][id] = mu * sb[1][id];
                q[2][id] = mu * sb[2][id];
                q[4][id] = mu * sb[4][id];
                double exx = dmd(fv[0] + id, 1), eyy = dmd(fv[1] + id, sy), ezz = dmd(fv[2] + id, sz);
                double gxy = dpd(fv[0] + id, sy) + dpd(fv[1] + id, 1);
                double gxz = dpd(fv[0] + id, sz) + dpd(fv[2] + id, 1);
                double gyz = dpd(fv[1] + id, sz) + dpd(fv[2] + id, sy);
                g[0][id] += k * (exx + eyy + ezz) * tr;
                g[1][id] += k * (2 * (exx * sb[0][id] + eyy * sb[3][id] + ezz * sb[5][id]) +
                                 gxy * sb[1][id] + gxz * sb[2][id] + gyz * sb[4][id]);
            }
#pragma omp parallel for schedule(static)
    for (int z = 2; z < nz - 2; z++)
        for (int y = 2; y < ny - 2; y++)
            for (int x = 2; x < nx - 2; x++) {
                size_t id = IDX(x, y, z);
                vb[0][id] -= k * (dpd(q[0] + id, 1) + dmd(q[1] + id, sy) + dmd(q[2] + id, sz));
                vb[1][id] -= k * (dpd(q[3] + id, sy) + dmd(q[1] + id, 1) + dmd(q[4] + id, sz));
                vb[2][id] -= k * (dpd(q[5] + id, sz) + dmd(q[2] + id, 1) + dmd(q[4] + id, sy));
            }
    /* velocity stage: w = b vb on W, gradient of buoyancy */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                if (!INW(x, y, z)) continue;
                size_t id = IDX(x, y, z);
                double b = m[2][id];
                w[0][id] = b * vb[0][id];
                w[1][id] = b * vb[1][id];
                w[2][id] = b * vb[2][id];
                double ax = dpd(fs[0] + id, 1) + dmd(fs[1] + id, sy) + dmd(fs[2] + id, sz);
                double ay = dmd(fs[1] + id, 1) + dpd(fs[3] + id, sy) + dmd(fs[4] + id, sz);
                double az = dmd(fs[2] + id, 1) + dmd(fs[4] + id, sy) + dpd(fs[5] + id, sz);
                g[2][id] += k * (ax * vb[0][id] + ay * vb[1][id] + az * vb[2][id]);
            }
#pragma omp parallel for schedule(static)
    for (int z = 2; z < nz - 2; z++)
        for (int y = 2; y < ny - 2; y++)
            for (int x = 2; x < nx - 2; x++) {
                size_t id = IDX(x, y, z);
                sb[0][id] -= k * dmd(w[0] + id, 1);
                sb[3][id] -= k * dmd(w[1] + id, sy);
                sb[5][id] -= k * dmd(w[2] + id, sz);
                sb[1][id] -= k * (dpd(w[0] + id, sy) + dpd(w[1] + id, 1));
                sb[2][id] -= k * (dpd(w[0] + id, sz) + dpd(w[2] + id, 1));
                sb[4][id] -= k * (dpd(w[1] + id, sz) + dpd(w[2] + id, sy));
            }
#undef INW
    for (int i = 0; i < 6; ++i) free(q[i]);
    for (int i = 0; i < 3; ++i) free(w[i]);
}
