// heat_unit.cuh -- one work unit of the heat sweep: one 128 x TY tile of one
// block over a chunk of output planes, one sub-step.  Shared by the plain
// sweep (heat.cu) and the batched persistent kernel (batch.cu).
//
// Every input plane of the tile plus a D-row / 4-column skirt arrives in
// shared memory by one TMA 4-D box (x, y, z, block) into an S-deep ring with
// one mbarrier per slot; each thread holds 4 consecutive x cells of RY rows
// and keeps 2D+1 planes of them in a float4 register queue along z; the xy
// neighbours of the current plane come from shared memory.  The ring position
// (planes streamed so far) carries over from unit to unit, so a persistent
// CTA keeps its barriers' phases consistent across units.
//
// Scheme (heat-3D.cu:228-231, 315-318, 410-413, 514-517), folded:
//     u' = a0*u + sum_k [ax_k (u[x-k]+u[x+k]) + ay_k (..y..) + az_k (..z..)].
#pragma once
#include "b2r_common.cuh"
#include "heat.h"

namespace b2r {
namespace heatk {

constexpr int kTX = 128;     // tile width (cells): 32 lanes x float4
constexpr int kWarps = 8;
constexpr int kThreads = 32 * kWarps;

// ring geometry for radius D, RY row slots per warp, S slots of SLOT floats,
// LPR lanes per tile row: a tile is 4*LPR cells wide (128, 64 or 32) and a
// warp covers 32/LPR rows per row slot
template <int D, int RY, int S, int SLOT_ = 0, int LPR = 32>
struct Cfg {
    static constexpr int TXW = 4 * LPR;
    static constexpr int RPW = 32 / LPR;
    static constexpr int TY = kWarps * RY * RPW;
    static constexpr int BW = TXW + 8;       // 4-cell skirt on both sides (D <= 4)
    static constexpr int BH = TY + 2 * D;
    static constexpr int PLANE = BW * BH;    // floats of one tile plane
    static constexpr int SLOT = SLOT_ > 0 ? SLOT_ : (PLANE + 31) / 32 * 32;   // 128-byte aligned
    // ring, then S mbarriers, then the abort flag, plus 128 B to align the base
    static constexpr size_t SMEM = size_t(S) * SLOT * sizeof(float) + S * sizeof(uint64_t) + 16 + 128;
};

// Per-CTA ring state in shared memory / registers.
struct Ring {
    float* smem;
    uint64_t* bar;
    int* abort_flag;
    unsigned gp;          // planes streamed by this CTA so far (ring position)
    unsigned issued_hi;   // ring position one past the last plane issued
    unsigned stop;        // ring position where an abort happened
};

template <int S, int SLOT>
__device__ __forceinline__ void ring_init(Ring& rg, unsigned char* smem_raw)
{
    // TMA destinations must be 128-byte aligned: align the base by hand
    rg.smem = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    rg.bar = reinterpret_cast<uint64_t*>(rg.smem + S * SLOT);
    rg.abort_flag = reinterpret_cast<int*>(rg.bar + S);
    rg.gp = rg.issued_hi = rg.stop = 0;
    if (threadIdx.x == 0) {
        *rg.abort_flag = 0;
#pragma unroll
        for (int s = 0; s < S; ++s) mbar_init(&rg.bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
}

// After an abort: thread 0 waits (bounded) for the loads still in flight.
template <int S>
__device__ __forceinline__ void ring_drain(const Ring& rg)
{
    if (threadIdx.x == 0)
        for (unsigned g = rg.stop; g < rg.issued_hi; ++g)
            mbar_wait_bounded(&rg.bar[g % S], (g / S) & 1, 100000000ull);
}

// Sweep one unit.  Returns false if a bounded wait gave up (all threads
// agree: the decision is taken after a __syncthreads on a shared flag).
// LPR = 0: the tile shape is the run-time lpr (32, 16 or 8 lanes per tile
// row), so that one kernel serves instances of different tile shapes; the
// tensor map's box must match it.
template <int D, int RY, int S, int SLOT, int LPR = 32>
__device__ __forceinline__ bool sweep_unit(const CUtensorMap* tmap, float* __restrict__ out,
                                           const BlockLayout& L, int step_i, const HeatCoef& C,
                                           int blk, int tx, int ty, int zi0, int zi1, Ring& rg, int lpr = LPR)
{
    if (LPR > 0) lpr = LPR;
    const int lg = lpr == 32 ? 5 : (lpr == 16 ? 4 : 3);   // log2(lpr)
    const int kTXW = 4 * lpr, kRPW = 32 >> lg;
    const int kTY = kWarps * RY * kRPW, kBW = kTXW + 8;
    const int kPLANE = kBW * (kTY + 2 * D);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int lane = (tid & 31) & (lpr - 1);  // x group of this thread in its row
    const int sr = (tid & 31) >> lg;          // row of this thread within a row slot
    const int edge = edge_bits(L, blk);
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) stage_region(L, edge, a, D * (step_i + 1), lo[a], hi[a]);
    const int xs0 = ((L.xoff + D) & ~3) + tx * kTXW;     // storage x of tile column 0
    const int y0 = D + ty * kTY;                       // block y of tile row 0
    if (xs0 - L.xoff > hi[0] || xs0 + kTXW - 1 - L.xoff < lo[0]) return true;
    if (y0 > hi[1] || y0 + kTY - 1 < lo[1]) return true;
    const int zs = max(D + zi0, lo[2]);
    const int ze = min(D + zi1 - 1, hi[2]);
    if (zs > ze) return true;

    const float a0 = C.a0;
    float ax[D], ay[D], az[D];
#pragma unroll
    for (int k = 0; k < D; ++k) { ax[k] = C.ax[k]; ay[k] = C.ay[k]; az[k] = C.az[k]; }

    const unsigned gp = rg.gp;
    const int first = zs - D;                // first input plane
    const int np = (ze + D) - first + 1;     // input planes streamed
    if (tid == 0) {
        for (int s = 0; s < S && s < np; ++s) {
            const unsigned g = gp + s;
            mbar_expect_tx(&rg.bar[g % S], kPLANE * sizeof(float));
            tma_load_4d(rg.smem + (g % S) * SLOT, tmap, xs0 - 4, y0 - D, first + s, blk, &rg.bar[g % S]);
        }
    }
    rg.issued_hi = gp + min(S, np);

    const int xb = xs0 + 4 * lane - L.xoff;             // block x of this lane's first cell
    bool vx[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) vx[j] = (xb + j >= lo[0]) && (xb + j <= hi[0]);
    const bool vx_all = vx[0] && vx[1] && vx[2] && vx[3];
    const bool vx_any = vx[0] || vx[1] || vx[2] || vx[3];

    float4 q[RY][2 * D + 1];
    float* const outb = out + (long long)blk * L.bstride + xs0 + 4 * lane;

    // unrolled by the queue depth, so the queue rotation becomes register
    // renaming instead of 2D float4 moves per row and plane (not at D = 4
    // with two rows per warp, where the unrolled loop spills)
#ifndef B2R_SWEEP_UNROLL
#define B2R_SWEEP_UNROLL 1
#endif
#ifndef B2R_HEAT4_UNROLL
#define B2R_HEAT4_UNROLL 0
#endif
    constexpr int kUnroll = (B2R_SWEEP_UNROLL && (D <= 3 || RY == 1 || B2R_HEAT4_UNROLL)) ? 2 * D + 1 : 1;
#pragma unroll kUnroll
    for (int pr = 0; pr < np; ++pr) {
        const unsigned g = gp + pr;
        if (!mbar_wait_bounded(&rg.bar[g % S], (g / S) & 1)) *rg.abort_flag = 1;
        const float* pl = rg.smem + (g % S) * SLOT;
#pragma unroll
        for (int r2 = 0; r2 < RY; ++r2) {
#pragma unroll
            for (int k = 0; k < 2 * D; ++k) q[r2][k] = q[r2][k + 1];
            const int row = D + (warp * RY + r2) * kRPW + sr;
            q[r2][2 * D] = *reinterpret_cast<const float4*>(pl + row * kBW + 4 + 4 * lane);
        }
        if (pr >= 2 * D && vx_any) {
            const int z = first + pr - D;
            const float* pc = rg.smem + ((g - D) % S) * SLOT;
#pragma unroll
            for (int r2 = 0; r2 < RY; ++r2) {
                const int y = y0 + (warp * RY + r2) * kRPW + sr;
                if (y < lo[1] || y > hi[1]) continue;
                const int row = D + (warp * RY + r2) * kRPW + sr;
                const float* prow = pc + row * kBW + 4 * lane;
                const float4 xl = *reinterpret_cast<const float4*>(prow);
                const float4 c4 = q[r2][D];
                const float4 xr = *reinterpret_cast<const float4*>(prow + 8);
                const float v[12] = {xl.x, xl.y, xl.z, xl.w, c4.x, c4.y, c4.z, c4.w,
                                     xr.x, xr.y, xr.z, xr.w};
                // cells (0, 1) and (2, 3) in packed two-lane FP32 operations,
                // each lane the scalar round-to-nearest one (heat_upd.cuh)
                float2 lo = __fmul2_rn(make_float2(a0, a0), make_float2(v[4], v[5]));
                float2 hi = __fmul2_rn(make_float2(a0, a0), make_float2(v[6], v[7]));
#pragma unroll
                for (int k = 1; k <= D; ++k) {
                    const float4 ym = *reinterpret_cast<const float4*>(prow + 4 - k * kBW);
                    const float4 yp = *reinterpret_cast<const float4*>(prow + 4 + k * kBW);
                    const float4 zm = q[r2][D - k];
                    const float4 zp = q[r2][D + k];
                    const float2 cx = make_float2(ax[k - 1], ax[k - 1]), cy = make_float2(ay[k - 1], ay[k - 1]),
                                 cz = make_float2(az[k - 1], az[k - 1]);
                    lo = __ffma2_rn(cx, make_float2(v[4 - k] + v[4 + k], v[5 - k] + v[5 + k]), lo);
                    hi = __ffma2_rn(cx, make_float2(v[6 - k] + v[6 + k], v[7 - k] + v[7 + k]), hi);
                    lo = __ffma2_rn(cy, __fadd2_rn(make_float2(ym.x, ym.y), make_float2(yp.x, yp.y)), lo);
                    hi = __ffma2_rn(cy, __fadd2_rn(make_float2(ym.z, ym.w), make_float2(yp.z, yp.w)), hi);
                    lo = __ffma2_rn(cz, __fadd2_rn(make_float2(zm.x, zm.y), make_float2(zp.x, zp.y)), lo);
                    hi = __ffma2_rn(cz, __fadd2_rn(make_float2(zm.z, zm.w), make_float2(zp.z, zp.w)), hi);
                }
                const float res[4] = {lo.x, lo.y, hi.x, hi.y};
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
        if (*rg.abort_flag) {
            rg.stop = g;
            return false;
        }
        if (pr >= D) {
            const int nxt = pr - D + S;
            if (nxt < np) {
                const unsigned g2 = gp + nxt;
                if (tid == 0) {
                    mbar_expect_tx(&rg.bar[g2 % S], kPLANE * sizeof(float));
                    tma_load_4d(rg.smem + (g2 % S) * SLOT, tmap, xs0 - 4, y0 - D, first + nxt, blk,
                                &rg.bar[g2 % S]);
                }
                rg.issued_hi = g2 + 1;
            }
        }
    }
    rg.gp = gp + np;
    return true;
}

}  // namespace heatk
}  // namespace b2r
