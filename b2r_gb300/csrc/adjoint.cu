// adjoint.cu -- hand-written discrete adjoint of the staggered elastic-wave
// time stepping (no reference counterpart) and the receiver misfit gradient
// with respect to lambda, mu and rho, with wavefield checkpointing.
//
// Forward step n (eqwp.cu STAG stage kernels), on the interior window W:
//   v'  = v + dt*b*(Dsigma)          velocity stage (Dp/Dm staggered FD4)
//   s'  = s + dt*C(lambda,mu)*E(v') + src_n   stress stage
//   d_n = vy'(receivers)
// Misfit J = 1/2 sum_n sum_r (d_n,r - obs_n,r)^2.  Reverse step n, with
// (vb, sb) the adjoints of (v', s'):
//   1. vb_y(rec) += d_n - obs_n
//   2. stress stage: q = C*sb on W (0 elsewhere);  vb += dt*E^T q;
//      g_lambda += dt*tr(E v')*tr(sb), g_mu += dt*(2 e_ii sb_ii + gamma_ij sb_ij)
//   3. velocity stage: w = b*vb on W (0 elsewhere);  sb += dt*D^T w;
//      g_b += dt*(D s)*vb on W
// with Dp^T = -Dm and Dm^T = -Dp for the 4th-order staggered differences.
// Gradients accumulate in FP64.  g_rho = -g_b / rho^2 at the end.
#include <cstdio>
#include <vector>

#include "b2r_common.cuh"
#include "eqwp.h"

namespace b2r {
namespace {

constexpr float C1 = 1.125f, C2 = -1.f / 24.f;

__device__ __forceinline__ float dpf(const float* f, long long s)
{
    return C1 * (f[s] - f[0]) + C2 * (f[2 * s] - f[-s]);
}
__device__ __forceinline__ float dmf(const float* f, long long s)
{
    return C1 * (f[0] - f[-s]) + C2 * (f[s] - f[-2 * s]);
}

struct Adj {
    float* vb[3];          // adjoint velocity
    float* sb[6];          // adjoint stress: xx, xy, xz, yy, yz, zz
    float* q[6];           // C*sb on W
    float* w[3];           // b*vb on W
    const float* v[3];     // forward velocity v^{n+1}
    const float* s[6];     // forward stress s^n (for the velocity-stage gradient)
    const float* lam;
    const float* mu;
    const float* buoy;
    double* g_lam;
    double* g_mu;
    double* g_b;
    float dt_h;            // dt / h
    int lo[3], hi[3];      // window W (inclusive)
};

__device__ __forceinline__ bool cell_of(const BlockLayout& L, long long e, int& x, int& y, int& z)
{
    x = (int)(e % L.n[0]);
    const long long r = e / L.n[0];
    y = (int)(r % L.n[1]);
    z = (int)(r / L.n[1]);
    return true;
}

__device__ __forceinline__ bool in_w(const Adj& A, int x, int y, int z)
{
    return x >= A.lo[0] && x <= A.hi[0] && y >= A.lo[1] && y <= A.hi[1] && z >= A.lo[2] && z <= A.hi[2];
}

// 2a: q = C*sb on W, 0 elsewhere; lambda / mu gradients on W (uses v^{n+1})
__global__ void adj_q_kernel(Adj A, const BlockLayout L)
{
    const long long total = (long long)L.n[0] * L.n[1] * L.n[2];
    const long long P = L.P, S = L.plane;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        cell_of(L, e, x, y, z);
        const long long id = (long long)z * S + (long long)y * P + L.xoff + x;
        if (!in_w(A, x, y, z)) {
            for (int k = 0; k < 6; ++k) A.q[k][id] = 0.f;
            continue;
        }
        const float l = A.lam[id], m = A.mu[id];
        const float sxx = A.sb[0][id], sxy = A.sb[1][id], sxz = A.sb[2][id];
        const float syy = A.sb[3][id], syz = A.sb[4][id], szz = A.sb[5][id];
        const float tr = sxx + syy + szz;
        A.q[0][id] = 2.f * m * sxx + l * tr;
        A.q[3][id] = 2.f * m * syy + l * tr;
        A.q[5][id] = 2.f * m * szz + l * tr;
        A.q[1][id] = m * sxy;
        A.q[2][id] = m * sxz;
        A.q[4][id] = m * syz;
        // strain of v^{n+1} (the forward stress stage, eqwp.cu STAG)
        const float* vx = A.v[0] + id;
        const float* vy = A.v[1] + id;
        const float* vz = A.v[2] + id;
        const float exx = dmf(vx, 1), eyy = dmf(vy, P), ezz = dmf(vz, S);
        const float gxy = dpf(vx, P) + dpf(vy, 1);
        const float gxz = dpf(vx, S) + dpf(vz, 1);
        const float gyz = dpf(vy, S) + dpf(vz, P);
        const double k = (double)A.dt_h;
        A.g_lam[id] += k * ((double)exx + eyy + ezz) * (double)tr;
        A.g_mu[id] += k * (2.0 * ((double)exx * sxx + (double)eyy * syy + (double)ezz * szz) +
                           (double)gxy * sxy + (double)gxz * sxz + (double)gyz * syz);
    }
}

// 2b: vb += dt*E^T q  (E: exx = Dm_x vx, eyy = Dm_y vy, ezz = Dm_z vz,
// gxy = Dp_y vx + Dp_x vy, gxz = Dp_z vx + Dp_x vz, gyz = Dp_z vy + Dp_y vz)
__global__ void adj_vb_kernel(Adj A, const BlockLayout L)
{
    const long long total = (long long)L.n[0] * L.n[1] * L.n[2];
    const long long P = L.P, S = L.plane;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        cell_of(L, e, x, y, z);
        if (x < 2 || y < 2 || z < 2 || x > L.n[0] - 3 || y > L.n[1] - 3 || z > L.n[2] - 3) continue;
        const long long id = (long long)z * S + (long long)y * P + L.xoff + x;
        const float* qxx = A.q[0] + id;
        const float* qxy = A.q[1] + id;
        const float* qxz = A.q[2] + id;
        const float* qyy = A.q[3] + id;
        const float* qyz = A.q[4] + id;
        const float* qzz = A.q[5] + id;
        const float k = A.dt_h;
        A.vb[0][id] -= k * (dpf(qxx, 1) + dmf(qxy, P) + dmf(qxz, S));
        A.vb[1][id] -= k * (dpf(qyy, P) + dmf(qxy, 1) + dmf(qyz, S));
        A.vb[2][id] -= k * (dpf(qzz, S) + dmf(qxz, 1) + dmf(qyz, P));
    }
}

// 3a: w = b*vb on W (0 elsewhere); g_b += dt*(D s^n).vb on W
__global__ void adj_w_kernel(Adj A, const BlockLayout L)
{
    const long long total = (long long)L.n[0] * L.n[1] * L.n[2];
    const long long P = L.P, S = L.plane;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        cell_of(L, e, x, y, z);
        const long long id = (long long)z * S + (long long)y * P + L.xoff + x;
        if (!in_w(A, x, y, z)) {
            for (int k = 0; k < 3; ++k) A.w[k][id] = 0.f;
            continue;
        }
        const float b = A.buoy[id];
        const float vbx = A.vb[0][id], vby = A.vb[1][id], vbz = A.vb[2][id];
        A.w[0][id] = b * vbx;
        A.w[1][id] = b * vby;
        A.w[2][id] = b * vbz;
        const float* sxx = A.s[0] + id;
        const float* sxy = A.s[1] + id;
        const float* sxz = A.s[2] + id;
        const float* syy = A.s[3] + id;
        const float* syz = A.s[4] + id;
        const float* szz = A.s[5] + id;
        const float ax = dpf(sxx, 1) + dmf(sxy, P) + dmf(sxz, S);
        const float ay = dmf(sxy, 1) + dpf(syy, P) + dmf(syz, S);
        const float az = dmf(sxz, 1) + dmf(syz, P) + dpf(szz, S);
        A.g_b[id] += (double)A.dt_h * ((double)ax * vbx + (double)ay * vby + (double)az * vbz);
    }
}

// 3b: sb += dt*D^T w  (velocity stage: ax = Dp_x sxx + Dm_y sxy + Dm_z sxz, ...)
__global__ void adj_sb_kernel(Adj A, const BlockLayout L)
{
    const long long total = (long long)L.n[0] * L.n[1] * L.n[2];
    const long long P = L.P, S = L.plane;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        cell_of(L, e, x, y, z);
        if (x < 2 || y < 2 || z < 2 || x > L.n[0] - 3 || y > L.n[1] - 3 || z > L.n[2] - 3) continue;
        const long long id = (long long)z * S + (long long)y * P + L.xoff + x;
        const float* wx = A.w[0] + id;
        const float* wy = A.w[1] + id;
        const float* wz = A.w[2] + id;
        const float k = A.dt_h;
        A.sb[0][id] -= k * dmf(wx, 1);
        A.sb[3][id] -= k * dmf(wy, P);
        A.sb[5][id] -= k * dmf(wz, S);
        A.sb[1][id] -= k * (dpf(wx, P) + dpf(wy, 1));
        A.sb[2][id] -= k * (dpf(wx, S) + dpf(wz, 1));
        A.sb[4][id] -= k * (dpf(wy, S) + dpf(wz, P));
    }
}

__global__ void rec_sample_kernel(const float* vy, const long long* idx, int nrec, float* out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrec) out[r] = vy[idx[r]];
}

__global__ void rec_inject_kernel(float* vby, const long long* idx, int nrec, const float* res)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrec) atomicAdd(&vby[idx[r]], res[r]);
}

// g_rho = -g_b * b^2 ; copy interior gradients out (x fastest, env cells)
__global__ void grad_out_kernel(const double* g, const float* buoy, int rho, const BlockLayout L,
                                double* out)
{
    const long long total = (long long)L.B[0] * L.B[1] * L.B[2];
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(e % L.B[0]);
        const long long r = e / L.B[0];
        const int y = (int)(r % L.B[1]);
        const int z = (int)(r / L.B[1]);
        const long long id = (long long)(z + L.H) * L.plane + (long long)(y + L.H) * L.P + L.xoff + x + L.H;
        double v = g[id];
        if (rho) {
            const double b = buoy[id];
            v = -v * b * b;
        }
        out[e] = v;
    }
}

inline int grid_for(long long work)
{
    long long g = (work + 255) / 256;
    if (g > 152LL * 16) g = 152LL * 16;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

// ---------------------------------------------------------------- driver
// All device buffers of one gradient computation.
struct AdjointRun {
    BlockLayout L;
    size_t fb = 0;
    std::vector<float*> ckpt;        // 9 fields per checkpoint
    std::vector<float*> replay;      // 9 fields per replayed state
    float* tmp[18] = {};             // vb(3) sb(6) q(6) w(3)
    double* g[3] = {};
    long long* d_idx = nullptr;
    float* d_rec = nullptr;          // nsteps*nrec synthetic data
    float* d_res = nullptr;          // nsteps*nrec residual
    ~AdjointRun()
    {
        for (float* p : ckpt) cudaFree(p);
        for (float* p : replay) cudaFree(p);
        for (float* p : tmp) if (p) cudaFree(p);
        for (double* p : g) if (p) cudaFree(p);
        if (d_idx) cudaFree(d_idx);
        if (d_rec) cudaFree(d_rec);
        if (d_res) cudaFree(d_res);
    }
};

cudaError_t adjoint_sample(const float* vy, const long long* d_idx, int nrec, float* out, cudaStream_t st)
{
    rec_sample_kernel<<<(nrec + 127) / 128, 128, 0, st>>>(vy, d_idx, nrec, out);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t adjoint_inject(float* vby, const long long* d_idx, int nrec, const float* res, cudaStream_t st)
{
    rec_inject_kernel<<<(nrec + 127) / 128, 128, 0, st>>>(vby, d_idx, nrec, res);
    count_launches(1);
    return cudaGetLastError();
}

// One reverse step.  fwd_v: v^{n+1} (3 fields), fwd_s: s^n (6 fields in the
// order xx, xy, xz, yy, yz, zz).
cudaError_t adjoint_step(float* const* tmp, const float* const* fwd_v, const float* const* fwd_s,
                         const float* const* mat, double* const* g, const BlockLayout& L, float dt_h,
                         const int lo[3], const int hi[3], cudaStream_t st)
{
    Adj A;
    for (int k = 0; k < 3; ++k) {
        A.vb[k] = tmp[k];
        A.w[k] = tmp[15 + k];
        A.v[k] = fwd_v[k];
    }
    for (int k = 0; k < 6; ++k) {
        A.sb[k] = tmp[3 + k];
        A.q[k] = tmp[9 + k];
        A.s[k] = fwd_s[k];
    }
    A.lam = mat[0];
    A.mu = mat[1];
    A.buoy = mat[2];
    A.g_lam = g[0];
    A.g_mu = g[1];
    A.g_b = g[2];
    A.dt_h = dt_h;
    for (int a = 0; a < 3; ++a) {
        A.lo[a] = lo[a];
        A.hi[a] = hi[a];
    }
    const int grid = grid_for((long long)L.n[0] * L.n[1] * L.n[2]);
    adj_q_kernel<<<grid, 256, 0, st>>>(A, L);
    adj_vb_kernel<<<grid, 256, 0, st>>>(A, L);
    adj_w_kernel<<<grid, 256, 0, st>>>(A, L);
    adj_sb_kernel<<<grid, 256, 0, st>>>(A, L);
    count_launches(4);
    return cudaGetLastError();
}

cudaError_t adjoint_grad_out(const double* g, const float* buoy, int rho, const BlockLayout& L,
                             double* out, cudaStream_t st)
{
    grad_out_kernel<<<grid_for((long long)L.B[0] * L.B[1] * L.B[2]), 256, 0, st>>>(g, buoy, rho, L, out);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace b2r
