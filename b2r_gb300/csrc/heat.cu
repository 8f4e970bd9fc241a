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

// Work schedule of one launch: units = (block, z-chunk of Lz output planes,
// tile row, tile column) numbered with the tile column fastest, dealt
// round-robin to gridDim.x CTAs.  Units that run at the same time are
// neighbouring tiles of the same planes, so whole DRAM rows are fetched
// together and the tile skirts hit L2.  gridDim.x = number of units gives one
// unit per CTA; a smaller grid makes the CTAs persistent.
struct HeatSched {
    int ntx, nty;            // tile columns / rows per block
    int NZ, Lz, nzc;         // output planes per column, planes per chunk, chunks
    long long U;             // units
};

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }

template <int D, int RY, int S>
__global__ void __launch_bounds__(kThreads)
heat_sweep_kernel(const __grid_constant__ CUtensorMap tin, float* __restrict__ out,
                  const BlockLayout L, const int step_i, const HeatCoef C, const HeatSched sch,
                  int* __restrict__ status)
{
    using Cfg = HeatCfg<D, RY, S>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // TMA destinations must be 128-byte aligned: align the base by hand
    float* smem = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + S * Cfg::SLOT);
    int& abort_flag = *reinterpret_cast<int*>(bar + S);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        abort_flag = 0;
#pragma unroll
        for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    // the input was written by the previous launch on this stream
    pdl_wait();
    pdl_trigger();

    const float a0 = C.a0;
    float ax[D], ay[D], az[D];
#pragma unroll
    for (int k = 0; k < D; ++k) { ax[k] = C.ax[k]; ay[k] = C.ay[k]; az[k] = C.az[k]; }

    unsigned gp = 0;             // ring position: planes streamed by this CTA so far
    bool aborted = false;
    int pr = 0, np = 0;
    unsigned issued_hi = 0;
    for (long long u = blockIdx.x; u < sch.U && !aborted; u += gridDim.x) {
        const int tx = (int)(u % sch.ntx);
        long long r = u / sch.ntx;
        const int ty = (int)(r % sch.nty);
        r /= sch.nty;
        const int zc = (int)(r % sch.nzc);
        const int blk = (int)(r / sch.nzc);
        const int zi0 = zc * sch.Lz;
        const int zi1 = min(sch.NZ, zi0 + sch.Lz);

        const int edge = edge_bits(L, blk);
        int lo[3], hi[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) stage_region(L, edge, a, D * (step_i + 1), lo[a], hi[a]);
        const int xs0 = ((L.xoff + D) & ~3) + tx * kTX;      // storage x of tile column 0
        const int y0 = D + ty * Cfg::TY;                     // block y of tile row 0
        if (xs0 - L.xoff > hi[0] || xs0 + kTX - 1 - L.xoff < lo[0]) continue;
        if (y0 > hi[1] || y0 + Cfg::TY - 1 < lo[1]) continue;
        const int zs = max(D + zi0, lo[2]);
        const int ze = min(D + zi1 - 1, hi[2]);
        if (zs > ze) continue;

        const int first = zs - D;               // first input plane
        np = (ze + D) - first + 1;              // input planes streamed
        if (tid == 0) {
            for (int s = 0; s < S && s < np; ++s) {
                const unsigned g = gp + s;
                mbar_expect_tx(&bar[g % S], Cfg::PLANE * sizeof(float));
                tma_load_4d(smem + (g % S) * Cfg::SLOT, &tin, xs0 - 4, y0 - D, first + s, blk,
                            &bar[g % S]);
            }
        }
        issued_hi = gp + min(S, np);

        const int xb = xs0 + 4 * lane - L.xoff;             // block x of this lane's first cell
        bool vx[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) vx[j] = (xb + j >= lo[0]) && (xb + j <= hi[0]);
        const bool vx_all = vx[0] && vx[1] && vx[2] && vx[3];
        const bool vx_any = vx[0] || vx[1] || vx[2] || vx[3];

        float4 q[RY][2 * D + 1];
        float* const outb = out + (long long)blk * L.bstride + xs0 + 4 * lane;

        for (pr = 0; pr < np; ++pr) {
            const unsigned g = gp + pr;
            if (!mbar_wait_bounded(&bar[g % S], (g / S) & 1)) abort_flag = 1;
            const float* pl = smem + (g % S) * Cfg::SLOT;
#pragma unroll
            for (int r2 = 0; r2 < RY; ++r2) {
#pragma unroll
                for (int k = 0; k < 2 * D; ++k) q[r2][k] = q[r2][k + 1];
                const int row = D + warp * RY + r2;
                q[r2][2 * D] = *reinterpret_cast<const float4*>(pl + row * Cfg::BW + 4 + 4 * lane);
            }
            if (pr >= 2 * D && vx_any) {
                const int z = first + pr - D;
                const float* pc = smem + ((g - D) % S) * Cfg::SLOT;
#pragma unroll
                for (int r2 = 0; r2 < RY; ++r2) {
                    const int y = y0 + warp * RY + r2;
                    if (y < lo[1] || y > hi[1]) continue;
                    const int row = D + warp * RY + r2;
                    const float* prow = pc + row * Cfg::BW + 4 * lane;
                    const float4 xl = *reinterpret_cast<const float4*>(prow);
                    const float4 c4 = q[r2][D];
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
                        const float4 zm = q[r2][D - k];
                        const float4 zp = q[r2][D + k];
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
            if (abort_flag) {
                aborted = true;
                break;
            }
            if (pr >= D) {
                const int nxt = pr - D + S;
                if (nxt < np) {
                    const unsigned g2 = gp + nxt;
                    if (tid == 0) {
                        mbar_expect_tx(&bar[g2 % S], Cfg::PLANE * sizeof(float));
                        tma_load_4d(smem + (g2 % S) * Cfg::SLOT, &tin, xs0 - 4, y0 - D, first + nxt,
                                    blk, &bar[g2 % S]);
                    }
                    issued_hi = g2 + 1;
                }
            }
        }
        if (!aborted) gp += np;
    }
    if (aborted && tid == 0) {
        report(status, DEV_TIMEOUT);
        // drain the loads still in flight (bounded) before the CTA retires
        for (unsigned g = gp + pr; g < issued_hi; ++g)
            mbar_wait_bounded(&bar[g % S], (g / S) & 1, 100000000ull);
    }
}

template <int D, int RY, int S>
cudaError_t launch_t(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                     const HeatCoef& c, int* status, cudaStream_t st, const HeatTune& tune)
{
    using Cfg = HeatCfg<D, RY, S>;
    auto kern = heat_sweep_kernel<D, RY, S>;
    static int resident = 0;    // CTAs resident on the whole GPU
    static int resident_per_sm = 0;
    if (resident == 0) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)Cfg::SMEM);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0, occ = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kThreads, Cfg::SMEM);
        if (e != cudaSuccess) return e;
        resident_per_sm = occ > 0 ? occ : 1;
        resident = resident_per_sm * (sms > 0 ? sms : 1);
    }
    HeatSched sch;
    const int xs_begin = (L.xoff + D) & ~3;
    const int xs_end = L.xoff + L.n[0] - D;              // exclusive
    sch.ntx = (xs_end - xs_begin + kTX - 1) / kTX;
    sch.nty = (L.n[1] - 2 * D + Cfg::TY - 1) / Cfg::TY;
    sch.NZ = L.n[2] - 2 * D;
    const long long tiles = (long long)sch.ntx * sch.nty * L.nblk;
    int Lz = tune.zchunk;
    if (Lz <= 0) {
        // default: chunks of 16 planes (the fastest on 512^3 D=1 of every
        // schedule the autotuner tries), fewer when the grid would be small
        Lz = 16;
        if (tiles * ((sch.NZ + 15) / 16) < 2LL * resident) {
            long long nzc = (2LL * resident + tiles - 1) / tiles;
            if (nzc > sch.NZ / 4) nzc = sch.NZ / 4 > 0 ? sch.NZ / 4 : 1;
            Lz = (int)((sch.NZ + nzc - 1) / nzc);
        }
    }
    if (Lz > sch.NZ) Lz = sch.NZ;
    if (Lz < 1) Lz = 1;
    sch.Lz = Lz;
    sch.nzc = (sch.NZ + Lz - 1) / Lz;
    sch.U = tiles * sch.nzc;
    long long G = sch.U;                                 // one unit per CTA
    if (tune.ctas_per_sm > 0) {                          // persistent
        const long long cap = (long long)resident / (resident_per_sm > 0 ? resident_per_sm : 1) *
                              (tune.ctas_per_sm < resident_per_sm ? tune.ctas_per_sm : resident_per_sm);
        if (G > cap) G = cap;
    }
    if (G < 1) G = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)G);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = tune.pdl ? 1 : 0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, *tin, out, L, step_i, c, sch, status);
    count_launches(1);
    if (e != cudaSuccess) return e;
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

cudaError_t launch_heat_substep(const CUtensorMap* tin, float* out, const BlockLayout& L, int D,
                                int step_i, const HeatCoef& c, int* status, cudaStream_t st,
                                const HeatTune& tune)
{
    switch (D) {
    case 1: return launch_t<1, 2, 4>(tin, out, L, step_i, c, status, st, tune);
    case 2: return launch_t<2, 2, 5>(tin, out, L, step_i, c, status, st, tune);
    case 3: return launch_t<3, 2, 6>(tin, out, L, step_i, c, status, st, tune);
    case 4: return launch_t<4, 2, 7>(tin, out, L, step_i, c, status, st, tune);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace b2r
