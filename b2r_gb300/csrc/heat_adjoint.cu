// heat_adjoint.cu -- receiver-misfit gradient of the heat model with respect
// to a per-cell conductivity field kappa (no reference counterpart).
//
// Differentiable form of the heat step (delta D, one block, fixed shell):
//   u^{n+1} = u^n + kappa * (L u^n)          on the interior window W
// where L is the reference's FD Laplacian of order 2D times alpha*dt/dx^2
// per axis (the stencil of fdm_heat_diffuse_deltaD, heat-3D.cu:15-28): with
// kappa = 1 this is the plain heat step.  d_n = u^{n+1}(receivers),
// J = 1/2 sum_n sum_r (d_n,r - obs_n,r)^2.  Reverse step n, lam = adjoint
// of u^{n+1}:
//   lam(rec) += d_n - obs_n
//   g_kappa  += lam * (L u^n)                 on W   (FP32 increment, FP64 sum)
//   y         = kappa * lam on W, 0 elsewhere
//   lam      += L^T y = L y                   on W   (L is symmetric)
// u^n is replayed from checkpoints every K steps.
#include <algorithm>
#include <vector>

#include "b2r_common.cuh"
#include "heat.h"

namespace b2r {

namespace {

// L u at one cell (D compile time): w0 u + sum_k (wx_k (u[x+k] + u[x-k]) +
// wy_k (...) + wz_k (...))
template <int D>
__device__ __forceinline__ float lap(const float* u, long long P, long long S, const HeatLap& c)
{
    float acc = c.w0 * u[0];
#pragma unroll
    for (int k = 1; k <= D; ++k) {
        acc += c.wx[k - 1] * (u[k] + u[-k]);
        acc += c.wy[k - 1] * (u[k * P] + u[-k * P]);
        acc += c.wz[k - 1] * (u[k * S] + u[-k * S]);
    }
    return acc;
}

struct Win3 {
    int lo[3], hi[3];
};

// thread = one (x, y) column of the window, marching z
template <int D>
__global__ void heat_kappa_step_kernel(const float* __restrict__ in, float* __restrict__ out,
                                       const float* __restrict__ kappa, const BlockLayout L, HeatLap c,
                                       Win3 w)
{
    const int x = w.lo[0] + blockIdx.x * blockDim.x + threadIdx.x;
    const int y = w.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    if (x > w.hi[0] || y > w.hi[1]) return;
    const long long P = L.P, S = L.plane;
    const long long col = (long long)y * P + L.xoff + x;
    for (int z = w.lo[2]; z <= w.hi[2]; ++z) {
        const long long i = col + (long long)z * S;
        out[i] = in[i] + kappa[i] * lap<D>(in + i, P, S, c);
    }
}

// y = kappa * lam on W (0 elsewhere, never written there); g += lam * L u^n
template <int D>
__global__ void heat_adj_y_kernel(const float* __restrict__ lam, const float* __restrict__ u,
                                  const float* __restrict__ kappa, float* __restrict__ yb, double* g,
                                  const BlockLayout L, HeatLap c, Win3 w)
{
    const int x = w.lo[0] + blockIdx.x * blockDim.x + threadIdx.x;
    const int y = w.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    if (x > w.hi[0] || y > w.hi[1]) return;
    const long long P = L.P, S = L.plane;
    const long long col = (long long)y * P + L.xoff + x;
    for (int z = w.lo[2]; z <= w.hi[2]; ++z) {
        const long long i = col + (long long)z * S;
        const float l = lam[i];
        yb[i] = kappa[i] * l;
        g[i] += (double)(l * lap<D>(u + i, P, S, c));
    }
}

// lam += L y on W
template <int D>
__global__ void heat_adj_lam_kernel(float* __restrict__ lam, const float* __restrict__ yb, const BlockLayout L,
                                    HeatLap c, Win3 w)
{
    const int x = w.lo[0] + blockIdx.x * blockDim.x + threadIdx.x;
    const int y = w.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    if (x > w.hi[0] || y > w.hi[1]) return;
    const long long P = L.P, S = L.plane;
    const long long col = (long long)y * P + L.xoff + x;
    for (int z = w.lo[2]; z <= w.hi[2]; ++z) {
        const long long i = col + (long long)z * S;
        lam[i] += lap<D>(yb + i, P, S, c);
    }
}

Win3 interior(const BlockLayout& L)
{
    Win3 w;
    for (int a = 0; a < 3; ++a) {
        w.lo[a] = L.H;
        w.hi[a] = L.n[a] - 1 - L.H;
    }
    return w;
}

dim3 col_grid(const Win3& w, dim3 b)
{
    return dim3((w.hi[0] - w.lo[0] + 1 + b.x - 1) / b.x, (w.hi[1] - w.lo[1] + 1 + b.y - 1) / b.y);
}

__global__ void fill_kernel(float* p, size_t n, float v)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

}  // namespace

cudaError_t launch_fill(float* p, size_t n, float v, cudaStream_t st)
{
    const size_t blocks = std::min<size_t>((n + 255) / 256, 152 * 16);
    fill_kernel<<<(unsigned)std::max<size_t>(blocks, 1), 256, 0, st>>>(p, n, v);
    count_launches(1);
    return cudaGetLastError();
}

HeatLap heat_lap(int D, double alpha_dt, double dx, double dy, double dz)
{
    static const double cw[5][5] = {
        {0, 0, 0, 0, 0},
        {-2.0, 1.0, 0, 0, 0},
        {-5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0, 0, 0},
        {-49.0 / 18.0, 3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0, 0},
        {-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0}};
    const double wx = alpha_dt / (dx * dx), wy = alpha_dt / (dy * dy), wz = alpha_dt / (dz * dz);
    HeatLap c{};
    c.w0 = (float)(cw[D][0] * (wx + wy + wz));
    for (int k = 1; k <= D; ++k) {
        c.wx[k - 1] = (float)(wx * cw[D][k]);
        c.wy[k - 1] = (float)(wy * cw[D][k]);
        c.wz[k - 1] = (float)(wz * cw[D][k]);
    }
    return c;
}

#define B2R_HEAT_ADJ_DISPATCH(D, CALL) \
    switch (D) {                       \
    case 1: CALL(1); break;            \
    case 2: CALL(2); break;            \
    case 3: CALL(3); break;            \
    case 4: CALL(4); break;            \
    default: return cudaErrorInvalidValue; \
    }

cudaError_t launch_heat_kappa_step(const float* in, float* out, const float* kappa, const BlockLayout& L, int D,
                                   const HeatLap& c, cudaStream_t st)
{
    const Win3 w = interior(L);
    const dim3 b(32, 8), g = col_grid(w, b);
#define CALL(DD) heat_kappa_step_kernel<DD><<<g, b, 0, st>>>(in, out, kappa, L, c, w)
    B2R_HEAT_ADJ_DISPATCH(D, CALL)
#undef CALL
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_heat_adjoint_step(float* lam, float* yb, const float* u, const float* kappa, double* g,
                                     const BlockLayout& L, int D, const HeatLap& c, cudaStream_t st)
{
    const Win3 w = interior(L);
    const dim3 b(32, 8), gr = col_grid(w, b);
#define CALL(DD)                                                                        \
    do {                                                                                \
        heat_adj_y_kernel<DD><<<gr, b, 0, st>>>(lam, u, kappa, yb, g, L, c, w);         \
        heat_adj_lam_kernel<DD><<<gr, b, 0, st>>>(lam, yb, L, c, w);                    \
    } while (0)
    B2R_HEAT_ADJ_DISPATCH(D, CALL)
#undef CALL
    count_launches(2);
    return cudaGetLastError();
}

}  // namespace b2r
