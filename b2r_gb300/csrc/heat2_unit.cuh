// heat2_unit.cuh -- one work unit of the two-step heat pass (radius 1): one
// 120 x 14 output tile of one block over a chunk of output planes, two
// sub-steps per HBM pass.  Shared by heat2_kernel (heat2.cu) and the batched
// persistent kernel (batch.cu), which streams its units through the same
// mbarrier ring as its one-step units.
//
// B2R's deep halo turned inward: a CTA reads a tile of the field once,
// advances it two sub-steps on chip and writes it once, so HBM traffic per
// lattice-site update halves.  Bit-identical to two launches of the plain
// sweep: every cell runs the same FMA sequence on the same inputs
// (heat-3D.cu:228-231 folded as in heat.cu).
//
// Shape.  Thread = 4 consecutive x cells (float4) of 2 rows; CTA = 8 warps =
// 128 x 16 stage-1 cells; output tile = lanes 1..30 x rows 1..14 = 120 x 14
// cells.  Per input plane p (TMA 4-D box 128 x 18 into an S-deep mbarrier
// ring):
//   stage 1 (sub-step i) at plane p-1: x neighbours by warp shuffles, y
//     neighbours from the thread's other row (registers) or the tile plane in
//     shared memory, z neighbours from a 3-plane float4 register queue;
//   stage 2 (sub-step i+1) at plane p-2: the same on stage-1 values -- x by
//     shuffles, y by registers or a 2-slot shared stage-1 plane (rows of other
//     warps), z by a second 3-plane register queue -- then stored to HBM.
// Cells outside a stage's window keep their value (fixed shell, B2R window).
// A unit in single-step mode stores the stage-1 values of its output tile
// and skips stage 2 (the last step of a run with an odd step count).
#pragma once
#include "b2r_common.cuh"
#include "heat.h"
#include "heat_upd.cuh"

namespace b2r {
namespace h2k {

constexpr int kW = 8;                 // warps
constexpr int kT2 = 32 * kW;          // threads
constexpr int kBoxW = 128;            // TMA box width (cells)
constexpr int kRows1 = 2 * kW;        // stage-1 rows (16)
constexpr int kBoxH = kRows1 + 2;     // input rows (18)
constexpr int kOutW = 120;            // output cells per tile row
constexpr int kOutH = kRows1 - 2;     // output rows (14)
constexpr int kPlane = kBoxW * kBoxH; // floats per input plane
constexpr int kP1 = kBoxW * kRows1;   // floats per stage-1 plane

// Per-CTA state of the plane loop.  The 3-plane queues rotate by index:
// at loop phase PH (= pr mod 3) the newest plane goes to slot PH, so the
// planes p-2, p-1, p sit in slots (PH+1)%3, (PH+2)%3, PH and no register is
// moved.  gp / issued_hi / stop are ring positions (planes streamed by this
// CTA), carried over from unit to unit.
struct H2Ctx {
    float4 q0[2][3], q1[2][3];
    const float* ring;
    float* s1;
    uint64_t* bar;
    int* abort_flag;
    float* outb;                 // out + block + lane's storage x
    const CUtensorMap* tmap;
    HeatCoef C;
    long long plane, P;
    unsigned gp;
    int np, first, zs, ze, xs0, y0, blk, ya, warp, lane, tid;
    int lo1z, hi1z, lo2z, hi2z;
    bool m1[2][4];               // stage-1 window, x and y part
    bool in2y[2], st_all, st_any;
    bool in2x[4];
    bool in1y[2], st1_all, st1_any;   // single-step mode: stored stage-1 cells
    bool in1x[4];
    bool single;
    unsigned issued_hi;
    bool aborted;
    unsigned stop;
};

__device__ __forceinline__ void h2_store(float* dst, float4 v, bool all, const bool (&m)[4])
{
    if (all) {
        *reinterpret_cast<float4*>(dst) = v;
    } else {
        if (m[0]) dst[0] = v.x;
        if (m[1]) dst[1] = v.y;
        if (m[2]) dst[2] = v.z;
        if (m[3]) dst[3] = v.w;
    }
}

// S ring slots of SLOT floats (SLOT >= kPlane)
template <int PH, int S, int SLOT>
__device__ __forceinline__ void h2_iter(H2Ctx& c, int pr)
{
    constexpr int CZ = (PH + 2) % 3, MZ = (PH + 1) % 3, NZ = PH;
    const unsigned g = c.gp + pr;
    if (!mbar_wait_bounded(&c.bar[g % S], (g / S) & 1)) *c.abort_flag = 1;
    const float* pl = c.ring + (g % S) * SLOT;
#pragma unroll
    for (int rr = 0; rr < 2; ++rr)
        c.q0[rr][NZ] = *reinterpret_cast<const float4*>(pl + (2 * c.warp + 1 + rr) * kBoxW + 4 * c.lane);
    const int p = c.first + pr;
    // ---- stage 1 at plane z1 = p-1
    if (pr >= 2) {
        const int z1 = p - 1;
        const float* pc = c.ring + ((g - 1) % S) * SLOT;
        const float4 up = *reinterpret_cast<const float4*>(pc + (2 * c.warp) * kBoxW + 4 * c.lane);
        const float4 dn = *reinterpret_cast<const float4*>(pc + (2 * c.warp + 3) * kBoxW + 4 * c.lane);
        const bool zin = z1 >= c.lo1z && z1 <= c.hi1z;
        float* s1p = c.s1 + (z1 & 1) * kP1;
        const bool st1 = c.single && zin && z1 >= c.zs && z1 <= c.ze && c.st1_any;
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const float4 ce = c.q0[rr][CZ];
            const float l = __shfl_up_sync(0xffffffffu, ce.w, 1);
            const float rt = __shfl_down_sync(0xffffffffu, ce.x, 1);
            const float4 ym = rr == 0 ? up : c.q0[0][CZ];
            const float4 yp = rr == 0 ? c.q0[1][CZ] : dn;
            const float4 v = heat_upd4(c.C, ce, l, rt, ym, yp, c.q0[rr][MZ], c.q0[rr][NZ]);
            float4 res;
            if (zin) {
                res.x = c.m1[rr][0] ? v.x : ce.x;
                res.y = c.m1[rr][1] ? v.y : ce.y;
                res.z = c.m1[rr][2] ? v.z : ce.z;
                res.w = c.m1[rr][3] ? v.w : ce.w;
            } else {
                res = ce;
            }
            if (st1 && c.in1y[rr])
                h2_store(c.outb + (long long)z1 * c.plane + (long long)(c.ya + rr) * c.P, res, c.st1_all, c.in1x);
            *reinterpret_cast<float4*>(s1p + (2 * c.warp + rr) * kBoxW + 4 * c.lane) = res;
            c.q1[rr][NZ] = res;
        }
    }
    // ---- stage 2 at plane z2 = p-2 (stage-1 planes p-3, p-2, p-1 in q1)
    if (pr >= 4 && !c.single) {
        const int z2 = p - 2;
        const float* sp = c.s1 + (z2 & 1) * kP1;
        const int wu = 2 * c.warp - 1, wd = 2 * c.warp + 2;
        const float4 up = *reinterpret_cast<const float4*>(sp + (wu < 0 ? 0 : wu) * kBoxW + 4 * c.lane);
        const float4 dn = *reinterpret_cast<const float4*>(sp + (wd >= kRows1 ? kRows1 - 1 : wd) * kBoxW + 4 * c.lane);
        const bool zin = z2 >= c.lo2z && z2 <= c.hi2z && z2 >= c.zs && z2 <= c.ze;
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const float4 ce = c.q1[rr][CZ];
            const float l = __shfl_up_sync(0xffffffffu, ce.w, 1);
            const float rt = __shfl_down_sync(0xffffffffu, ce.x, 1);
            const float4 ym = rr == 0 ? up : c.q1[0][CZ];
            const float4 yp = rr == 0 ? c.q1[1][CZ] : dn;
            const float4 v = heat_upd4(c.C, ce, l, rt, ym, yp, c.q1[rr][MZ], c.q1[rr][NZ]);
            if (zin && c.in2y[rr] && c.st_any)
                h2_store(c.outb + (long long)z2 * c.plane + (long long)(c.ya + rr) * c.P, v, c.st_all, c.in2x);
        }
    }
    __syncthreads();
    if (*c.abort_flag) {
        c.aborted = true;
        c.stop = g;
        return;
    }
    // plane p-1 is no longer needed: refill its slot with plane p-1+S
    if (pr >= 1) {
        const int nxt = pr - 1 + S;
        if (nxt < c.np) {
            const unsigned g2 = c.gp + nxt;
            if (c.tid == 0) {
                mbar_expect_tx(&c.bar[g2 % S], kPlane * 4);
                tma_load_4d(const_cast<float*>(c.ring) + (g2 % S) * SLOT, c.tmap, c.xs0, c.y0 - 2,
                            c.first + nxt, c.blk, &c.bar[g2 % S]);
            }
            c.issued_hi = g2 + 1;
        }
    }
}

// Tile columns / rows of a block for the two-step units: out0 = storage x of
// tile column 0's first output cell (the aligned float4 holding x = 1).
__host__ __device__ inline int h2_out0(const BlockLayout& L) { return (L.xoff + 1) & ~3; }
__host__ __device__ inline int h2_ntx(const BlockLayout& L)
{
    return (L.xoff + L.n[0] - 1 - h2_out0(L) + kOutW - 1) / kOutW;
}
__host__ __device__ inline int h2_nty(const BlockLayout& L) { return (L.n[1] - 2 + kOutH - 1) / kOutH; }

// One unit: tile (tx, ty) of block blk, output planes [1 + zi0, zi0 + Lz]
// clipped to the window, sub-steps step_i and step_i + 1 (single: step_i
// only).  c.ring/s1/bar/abort_flag/tid/lane/warp/C/plane/P and the ring
// position must be set.  Returns false if a bounded wait gave up (c.stop
// holds where).
template <int S, int SLOT>
__device__ __forceinline__ bool h2_unit(H2Ctx& c, const CUtensorMap* tmap, float* out, const BlockLayout& L,
                                        int step_i, int blk, int tx, int ty, int zi0, int Lz, bool single)
{
    c.tmap = tmap;
    c.blk = blk;
    c.single = single;
    const int edge = edge_bits(L, blk);
    int lo1[3], hi1[3], lo2[3], hi2[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        stage_region(L, edge, a, step_i + 1, lo1[a], hi1[a]);
        stage_region(L, edge, a, step_i + 2, lo2[a], hi2[a]);
    }
    // the stored window: stage 2's, or stage 1's in single-step mode
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = single ? lo1[a] : lo2[a];
        hi[a] = single ? hi1[a] : hi2[a];
    }
    c.xs0 = h2_out0(L) - 4 + tx * kOutW;             // storage x of lane 0's first cell
    c.y0 = 1 + ty * kOutH;                           // block y of output row 0
    c.zs = max(1 + zi0, lo[2]);
    c.ze = min(zi0 + Lz, hi[2]);                     // output planes [zs, ze]
    if (c.zs > c.ze) return true;
    if (c.xs0 + 4 - L.xoff > hi[0] || c.xs0 + 123 - L.xoff < lo[0]) return true;
    if (c.y0 > hi[1] || c.y0 + kOutH - 1 < lo[1]) return true;
    c.first = c.zs - 2;                              // first input plane
    c.np = c.ze + (single ? 1 : 2) - c.first + 1;
    c.lo1z = lo1[2];
    c.hi1z = hi1[2];
    c.lo2z = lo2[2];
    c.hi2z = hi2[2];
    if (c.tid == 0)
        for (int s = 0; s < S && s < c.np; ++s) {
            const unsigned g = c.gp + s;
            mbar_expect_tx(&c.bar[g % S], kPlane * 4);
            tma_load_4d(const_cast<float*>(c.ring) + (g % S) * SLOT, tmap, c.xs0, c.y0 - 2, c.first + s, blk,
                        &c.bar[g % S]);
        }
    c.issued_hi = c.gp + min(S, c.np);

    // this thread's cells: storage x xs0+4*lane.., stage-1 rows 2w, 2w+1
    const int xb = c.xs0 + 4 * c.lane - L.xoff;      // block x of the first cell
    c.ya = c.y0 - 1 + 2 * c.warp;                    // block y of stage-1 row 2w
    bool in1x[4];
    const bool lane_out = c.lane >= 1 && c.lane <= 30;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        in1x[j] = xb + j >= lo1[0] && xb + j <= hi1[0];
        c.in2x[j] = xb + j >= lo2[0] && xb + j <= hi2[0] && lane_out;
        c.in1x[j] = in1x[j] && lane_out;
    }
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
        const bool y1 = c.ya + rr >= lo1[1] && c.ya + rr <= hi1[1];
#pragma unroll
        for (int j = 0; j < 4; ++j) c.m1[rr][j] = y1 && in1x[j];
    }
    c.in2y[0] = c.ya >= lo2[1] && c.ya <= hi2[1] && 2 * c.warp >= 1;
    c.in2y[1] = c.ya + 1 >= lo2[1] && c.ya + 1 <= hi2[1] && 2 * c.warp + 1 <= kOutH;
    c.in1y[0] = c.ya >= lo1[1] && c.ya <= hi1[1] && 2 * c.warp >= 1;
    c.in1y[1] = c.ya + 1 >= lo1[1] && c.ya + 1 <= hi1[1] && 2 * c.warp + 1 <= kOutH;
    c.st_all = c.in2x[0] && c.in2x[1] && c.in2x[2] && c.in2x[3];
    c.st_any = c.in2x[0] || c.in2x[1] || c.in2x[2] || c.in2x[3];
    c.st1_all = c.in1x[0] && c.in1x[1] && c.in1x[2] && c.in1x[3];
    c.st1_any = c.in1x[0] || c.in1x[1] || c.in1x[2] || c.in1x[3];
    c.outb = out + (long long)blk * L.bstride + c.xs0 + 4 * c.lane;

    for (int pr = 0; pr < c.np;) {
        h2_iter<0, S, SLOT>(c, pr++);
        if (c.aborted || pr >= c.np) break;
        h2_iter<1, S, SLOT>(c, pr++);
        if (c.aborted || pr >= c.np) break;
        h2_iter<2, S, SLOT>(c, pr++);
        if (c.aborted) break;
    }
    if (c.aborted) return false;
    c.gp += c.np;
    return true;
}

}  // namespace h2k
}  // namespace b2r
