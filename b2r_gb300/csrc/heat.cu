// heat.cu -- explicit 3-D heat diffusion, stencil radius D = 1..4.
//
// Replaces fdm_heat_diffuse_delta1..4 (heat-3D.cu:173-521) and the
// edge-freezing fdm_heat_diffuse_delta1_verify (heat-3D.cu:57-158).  Scheme
// (heat-3D.cu:228-231, 315-318, 410-413, 514-517):
//     u' = u + alpha_dt * (Lx/dx^2 + Ly/dy^2 + Lz/dz^2)
// with the order-2D central second differences L of heat-3D.cu:15-28, folded
// here into   u' = a0*u + sum_k [ax_k (u[x-k]+u[x+k]) + ay_k (..y..) + az_k (..z..)].
//
// Kernel shape: 2.5-D sweep.  A CTA owns a 128 x TY tile of one block in xy
// (lane = 4 consecutive x cells, warp = RY rows) and a chunk of z planes.
// Every input plane of the tile plus a D-row / 4-column skirt arrives in
// shared memory by one TMA load into an S-deep ring (mbarrier completion);
// each thread keeps its 2D+1 planes of float4 in a register queue along z
// and reads the xy neighbours of the current plane from shared memory.
// One HBM read and one write per cell and sub-step; the skirt re-reads hit L2.
#include <cstdio>

#include "b2r_common.cuh"
#include "heat.h"

namespace b2r {

namespace {

constexpr int kTX = 128;     // tile width (cells): 32 lanes x float4
constexpr int kWarps = 8;
constexpr int kThreads = 32 * kWarps;

template <int D, int RY, int S>
struct HeatCfg {
    static constexpr int TY = kWarps * RY;
    static constexpr int BW = kTX + 8;       // 4-cell skirt on both sides (D <= 4)
    static constexpr int BH = TY + 2 * D;
    static constexpr int PLANE = BW * BH;    // floats of one tile plane
    static constexpr int SLOT = (PLANE + 31) / 32 * 32;   // ring slot stride: 128-byte aligned
    // ring, then S mbarriers, then the abort flag, plus 128 B to align the base
    static constexpr size_t SMEM = size_t(S) * SLOT * sizeof(float) + S * sizeof(uint64_t) + 16 + 128;
};

template <int D, int RY, int S>
__global__ void __launch_bounds__(kThreads)
heat_sweep_kernel(const __grid_constant__ CUtensorMap tin, float* __restrict__ out,
                  const BlockLayout L, const int step_i, const int nzc, const HeatCoef C,
                  int* __restrict__ status)
{
    using Cfg = HeatCfg<D, RY, S>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // TMA destinations must be 128-byte aligned: align the base by hand
    float* smem = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + S * Cfg::SLOT);
    int& abort_flag = *reinterpret_cast<int*>(bar + S);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const int edge = edge_bits(L, blk);
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) stage_region(L, edge, a, D * (step_i + 1), lo[a], hi[a]);

    const int xs_begin = (L.xoff + D) & ~3;
    const int xs0 = xs_begin + blockIdx.x * kTX;        // storage x of tile column 0
    const int y0 = D + blockIdx.y * Cfg::TY;            // block y of tile row 0
    // uniform early exits (before any barrier is initialised)
    if (xs0 - L.xoff > hi[0] || xs0 + kTX - 1 - L.xoff < lo[0]) return;
    if (y0 > hi[1] || y0 + Cfg::TY - 1 < lo[1]) return;
    const int nz_out = hi[2] - lo[2] + 1;
    const int per = (nz_out + nzc - 1) / nzc;
    const int zs = lo[2] + zc * per;
    const int ze = min(hi[2], zs + per - 1);
    if (nz_out <= 0 || zs > ze) return;

    const int first = zs - D;                 // first input plane
    const int np = (ze + D) - first + 1;      // input planes streamed

    if (tid == 0) {
        abort_flag = 0;
#pragma unroll
        for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < S && s < np; ++s) {
            mbar_expect_tx(&bar[s], Cfg::PLANE * sizeof(float));
            tma_load_4d(smem + s * Cfg::SLOT, &tin, xs0 - 4, y0 - D, first + s, blk, &bar[s]);
        }
    }

    // coefficients in registers
    const float a0 = C.a0;
    float ax[D], ay[D], az[D];
#pragma unroll
    for (int k = 0; k < D; ++k) { ax[k] = C.ax[k]; ay[k] = C.ay[k]; az[k] = C.az[k]; }

    const int xb = xs0 + 4 * lane - L.xoff;             // block x of this lane's first cell
    bool vx[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) vx[j] = (xb + j >= lo[0]) && (xb + j <= hi[0]);
    const bool vx_all = vx[0] && vx[1] && vx[2] && vx[3];
    const bool vx_any = vx[0] || vx[1] || vx[2] || vx[3];

    float4 q[RY][2 * D + 1];
    float* const outb = out + (long long)blk * L.bstride + xs0 + 4 * lane;

    int pr = 0;
    for (; pr < np; ++pr) {
        const int slot = pr % S;
        if (!mbar_wait_bounded(&bar[slot], (pr / S) & 1)) {
            abort_flag = 1;
        }
        const float* pl = smem + slot * Cfg::SLOT;
#pragma unroll
        for (int r = 0; r < RY; ++r) {
#pragma unroll
            for (int k = 0; k < 2 * D; ++k) q[r][k] = q[r][k + 1];
            const int row = D + warp * RY + r;
            q[r][2 * D] = *reinterpret_cast<const float4*>(pl + row * Cfg::BW + 4 + 4 * lane);
        }
        if (pr >= 2 * D && vx_any) {
            const int z = first + pr - D;
            const float* pc = smem + ((pr - D) % S) * Cfg::SLOT;
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                const int y = y0 + warp * RY + r;
                if (y < lo[1] || y > hi[1]) continue;
                const int row = D + warp * RY + r;
                const float* prow = pc + row * Cfg::BW + 4 * lane;
                const float4 xl = *reinterpret_cast<const float4*>(prow);
                const float4 c4 = q[r][D];
                const float4 xr = *reinterpret_cast<const float4*>(prow + 8);
                const float v[12] = {xl.x, xl.y, xl.z, xl.w, c4.x, c4.y, c4.z, c4.w,
                                     xr.x, xr.y, xr.z, xr.w};
                float res[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) res[j] = a0 * v[4 + j];
#pragma unroll
                for (int k = 1; k <= D; ++k) {
                    const float4 ym = *reinterpret_cast<const float4*>(prow + 4 - k * Cfg::BW);
                    const float4 yp = *reinterpret_cast<const float4*>(prow + 4 + k * Cfg::BW);
                    const float4 zm = q[r][D - k];
                    const float4 zp = q[r][D + k];
                    const float ys[4] = {ym.x + yp.x, ym.y + yp.y, ym.z + yp.z, ym.w + yp.w};
                    const float zsum[4] = {zm.x + zp.x, zm.y + zp.y, zm.z + zp.z, zm.w + zp.w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        res[j] = fmaf(ax[k - 1], v[4 + j - k] + v[4 + j + k], res[j]);
                        res[j] = fmaf(ay[k - 1], ys[j], res[j]);
                        res[j] = fmaf(az[k - 1], zsum[j], res[j]);
                    }
                }
                float* dst = outb + (long long)z * L.plane + (long long)y * L.P;
                if (vx_all) {
                    *reinterpret_cast<float4*>(dst) = make_float4(res[0], res[1], res[2], res[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (vx[j]) dst[j] = res[j];
                }
            }
        }
        __syncthreads();
        if (abort_flag) break;
        if (tid == 0 && pr >= D) {
            const int nxt = pr - D + S;
            if (nxt < np) {
                const int s2 = (pr - D) % S;
                mbar_expect_tx(&bar[s2], Cfg::PLANE * sizeof(float));
                tma_load_4d(smem + s2 * Cfg::SLOT, &tin, xs0 - 4, y0 - D, first + nxt, blk,
                            &bar[s2]);
            }
        }
    }
    if (abort_flag && tid == 0) {
        report(status, DEV_TIMEOUT);
        // drain the loads still in flight (bounded) before the CTA retires
        const int issued = min(np, (pr >= D ? pr - D + S : S));
        for (int p = pr; p < issued; ++p) mbar_wait_bounded(&bar[p % S], (p / S) & 1, 100000000ull);
    }
}

template <int D, int RY, int S>
cudaError_t launch_t(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                     const HeatCoef& c, int* status, cudaStream_t st, int nzc)
{
    using Cfg = HeatCfg<D, RY, S>;
    auto kern = heat_sweep_kernel<D, RY, S>;
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)Cfg::SMEM);
        if (e != cudaSuccess) return e;
        attr_done = true;
    }
    const int xs_begin = (L.xoff + D) & ~3;
    const int xs_end = L.xoff + L.n[0] - D;              // exclusive
    const int ntx = (xs_end - xs_begin + kTX - 1) / kTX;
    const int nty = (L.n[1] - 2 * D + Cfg::TY - 1) / Cfg::TY;
    dim3 grid(ntx, nty, L.nblk * nzc);
    kern<<<grid, kThreads, Cfg::SMEM, st>>>(*tin, out, L, step_i, nzc, c, status);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace

int heat_box_h(int D) { return kWarps * 2 + 2 * D; }
int heat_box_w() { return kTX + 8; }

HeatCoef heat_coef(int D, double alpha_dt, double dx, double dy, double dz)
{
    // central second-difference weights c0..c4 of heat-3D.cu:15-28 (exact)
    static const double cw[5][5] = {
        {0, 0, 0, 0, 0},
        {-2.0, 1.0, 0, 0, 0},
        {-5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0, 0, 0},
        {-49.0 / 18.0, 3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0, 0},
        {-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0}};
    const double wx = alpha_dt / (dx * dx), wy = alpha_dt / (dy * dy), wz = alpha_dt / (dz * dz);
    HeatCoef c{};
    c.a0 = (float)(1.0 + cw[D][0] * (wx + wy + wz));
    for (int k = 1; k <= D; ++k) {
        c.ax[k - 1] = (float)(wx * cw[D][k]);
        c.ay[k - 1] = (float)(wy * cw[D][k]);
        c.az[k - 1] = (float)(wz * cw[D][k]);
    }
    return c;
}

int heat_default_nzc(const BlockLayout& L, int D)
{
    // enough CTAs for ~4 waves of 5 resident CTAs on 152 SMs, chunks >= 32 planes
    const int TY = kWarps * 2;
    const int xs_begin = (L.xoff + D) & ~3;
    const int ntx = (L.xoff + L.n[0] - D - xs_begin + kTX - 1) / kTX;
    const int nty = (L.n[1] - 2 * D + TY - 1) / TY;
    const long long tiles = (long long)ntx * nty * L.nblk;
    const long long want = 152LL * 5 * 4;
    int nzc = (int)((want + tiles - 1) / tiles);
    const int nz_out = L.n[2] - 2 * D;
    int maxc = nz_out / 32;
    if (maxc < 1) maxc = 1;
    if (nzc > maxc) nzc = maxc;
    if (nzc < 1) nzc = 1;
    return nzc;
}

cudaError_t launch_heat_substep(const CUtensorMap* tin, float* out, const BlockLayout& L, int D,
                                int step_i, const HeatCoef& c, int* status, cudaStream_t st,
                                int nzc)
{
    if (nzc <= 0) nzc = heat_default_nzc(L, D);
    switch (D) {
    case 1: return launch_t<1, 2, 4>(tin, out, L, step_i, c, status, st, nzc);
    case 2: return launch_t<2, 2, 5>(tin, out, L, step_i, c, status, st, nzc);
    case 3: return launch_t<3, 2, 6>(tin, out, L, step_i, c, status, st, nzc);
    case 4: return launch_t<4, 2, 7>(tin, out, L, step_i, c, status, st, nzc);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace b2r
