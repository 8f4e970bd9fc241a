// heat2.cu -- two heat time steps per HBM pass (temporal blocking), radius 1.
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
#include "b2r_common.cuh"
#include "heat.h"

namespace b2r {
namespace {

constexpr int kW = 8;                 // warps
constexpr int kT2 = 32 * kW;          // threads
constexpr int kBoxW = 128;            // TMA box width (cells)
constexpr int kRows1 = 2 * kW;        // stage-1 rows (16)
constexpr int kBoxH = kRows1 + 2;     // input rows (18)
constexpr int kOutW = 120;            // output cells per tile row
constexpr int kOutH = kRows1 - 2;     // output rows (14)
constexpr int kS2 = 4;                // input ring slots
constexpr int kPlane = kBoxW * kBoxH; // floats per input plane
constexpr int kP1 = kBoxW * kRows1;   // floats per stage-1 plane
constexpr size_t kSmem2 = size_t(kS2) * kPlane * 4 + 2 * size_t(kP1) * 4 + kS2 * 8 + 16 + 128;

__device__ __forceinline__ void pdl_wait2() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger2() { asm volatile("griddepcontrol.launch_dependents;"); }

struct H2Sched {
    int ntx, nty, NZ, Lz, nzc;
    int out0;          // storage x of the first output cell of tile column 0
    long long U;
};

// one folded D = 1 update of 4 cells: c centre, l/r = x-1 / x+4 cells,
// ym/yp/zm/zp neighbour float4s
__device__ __forceinline__ float4 upd(const HeatCoef& C, float4 c, float l, float r, float4 ym,
                                      float4 yp, float4 zm, float4 zp)
{
    float4 o;
    o.x = C.a0 * c.x;
    o.y = C.a0 * c.y;
    o.z = C.a0 * c.z;
    o.w = C.a0 * c.w;
    o.x = fmaf(C.ax[0], l + c.y, o.x);
    o.y = fmaf(C.ax[0], c.x + c.z, o.y);
    o.z = fmaf(C.ax[0], c.y + c.w, o.z);
    o.w = fmaf(C.ax[0], c.z + r, o.w);
    o.x = fmaf(C.ay[0], ym.x + yp.x, o.x);
    o.y = fmaf(C.ay[0], ym.y + yp.y, o.y);
    o.z = fmaf(C.ay[0], ym.z + yp.z, o.z);
    o.w = fmaf(C.ay[0], ym.w + yp.w, o.w);
    o.x = fmaf(C.az[0], zm.x + zp.x, o.x);
    o.y = fmaf(C.az[0], zm.y + zp.y, o.y);
    o.z = fmaf(C.az[0], zm.z + zp.z, o.z);
    o.w = fmaf(C.az[0], zm.w + zp.w, o.w);
    return o;
}

__device__ __forceinline__ float4 sel(const bool (&m)[4], float4 a, float4 b)
{
    return make_float4(m[0] ? a.x : b.x, m[1] ? a.y : b.y, m[2] ? a.z : b.z, m[3] ? a.w : b.w);
}

__global__ void __launch_bounds__(kT2, 2)
heat2_kernel(const __grid_constant__ CUtensorMap tin, float* __restrict__ out, const BlockLayout L,
             const int step_i, const HeatCoef C, const H2Sched sch, int* __restrict__ status)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    float* s1 = ring + kS2 * kPlane;                      // 2 stage-1 planes
    uint64_t* bar = reinterpret_cast<uint64_t*>(s1 + 2 * kP1);
    int* abort_flag = reinterpret_cast<int*>(bar + kS2);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        *abort_flag = 0;
        for (int s = 0; s < kS2; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    pdl_wait2();
    pdl_trigger2();

    unsigned gp = 0, issued_hi = 0, stop = 0;
    bool aborted = false;
    for (long long u = blockIdx.x; u < sch.U && !aborted; u += gridDim.x) {
        const int tx = (int)(u % sch.ntx);
        long long r = u / sch.ntx;
        const int ty = (int)(r % sch.nty);
        r /= sch.nty;
        const int zc = (int)(r % sch.nzc);
        const int blk = (int)(r / sch.nzc);
        const int edge = edge_bits(L, blk);
        int lo1[3], hi1[3], lo2[3], hi2[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            stage_region(L, edge, a, step_i + 1, lo1[a], hi1[a]);
            stage_region(L, edge, a, step_i + 2, lo2[a], hi2[a]);
        }
        const int xs0 = sch.out0 - 4 + tx * kOutW;       // storage x of lane 0's first cell
        const int y0 = 1 + ty * kOutH;                   // block y of output row 0
        const int zi0 = zc * sch.Lz;
        const int zs = max(1 + zi0, lo2[2]);
        const int ze = min(zi0 + sch.Lz, hi2[2]);        // output planes [zs, ze]
        if (zs > ze) continue;
        if (xs0 + 4 - L.xoff > hi2[0] || xs0 + 123 - L.xoff < lo2[0]) continue;
        if (y0 > hi2[1] || y0 + kOutH - 1 < lo2[1]) continue;
        const int first = zs - 2;                        // first input plane
        const int np = ze + 2 - first + 1;
        if (tid == 0)
            for (int s = 0; s < kS2 && s < np; ++s) {
                const unsigned g = gp + s;
                mbar_expect_tx(&bar[g % kS2], kPlane * 4);
                tma_load_4d(ring + (g % kS2) * kPlane, &tin, xs0, y0 - 2, first + s, blk, &bar[g % kS2]);
            }
        issued_hi = gp + min(kS2, np);

        // this thread's cells: storage x xs0+4*lane.., stage-1 rows 2w, 2w+1
        const int xb = xs0 + 4 * lane - L.xoff;          // block x of the first cell
        const int ya = y0 - 1 + 2 * warp;                // block y of stage-1 row 2w
        bool in1x[4], in2x[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            in1x[j] = xb + j >= lo1[0] && xb + j <= hi1[0];
            in2x[j] = xb + j >= lo2[0] && xb + j <= hi2[0] && lane >= 1 && lane <= 30;
        }
        const bool in1y[2] = {ya >= lo1[1] && ya <= hi1[1], ya + 1 >= lo1[1] && ya + 1 <= hi1[1]};
        const bool in2y[2] = {ya >= lo2[1] && ya <= hi2[1] && 2 * warp >= 1,
                              ya + 1 >= lo2[1] && ya + 1 <= hi2[1] && 2 * warp + 1 <= kOutH};
        const bool st_all = in2x[0] && in2x[1] && in2x[2] && in2x[3];
        const bool st_any = in2x[0] || in2x[1] || in2x[2] || in2x[3];

        float4 q0[2][3], q1[2][3];       // [row][plane]: input / stage-1 queues (z-1, z, z+1)
        float* const outb = out + (long long)blk * L.bstride + xs0 + 4 * lane;

        for (int pr = 0; pr < np; ++pr) {
            const unsigned g = gp + pr;
            if (!mbar_wait_bounded(&bar[g % kS2], (g / kS2) & 1)) *abort_flag = 1;
            const float* pl = ring + (g % kS2) * kPlane;
            // push input plane p (box rows 2w+1, 2w+2 = stage-1 rows 2w, 2w+1)
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                q0[rr][0] = q0[rr][1];
                q0[rr][1] = q0[rr][2];
                q0[rr][2] = *reinterpret_cast<const float4*>(pl + (2 * warp + 1 + rr) * kBoxW + 4 * lane);
            }
            const int p = first + pr;
            // ---- stage 1 at plane z1 = p-1
            if (pr >= 2) {
                const int z1 = p - 1;
                const float* pc = ring + ((g - 1) % kS2) * kPlane;   // input plane z1
                const float4 up = *reinterpret_cast<const float4*>(pc + (2 * warp) * kBoxW + 4 * lane);
                const float4 dn = *reinterpret_cast<const float4*>(pc + (2 * warp + 3) * kBoxW + 4 * lane);
                const bool zin = z1 >= lo1[2] && z1 <= hi1[2];
                float4 res[2];
#pragma unroll
                for (int rr = 0; rr < 2; ++rr) {
                    const float4 c = q0[rr][1];
                    const float l = __shfl_up_sync(0xffffffffu, c.w, 1);
                    const float rt = __shfl_down_sync(0xffffffffu, c.x, 1);
                    const float4 ym = rr == 0 ? up : q0[0][1];
                    const float4 yp = rr == 0 ? q0[1][1] : dn;
                    const float4 v = upd(C, c, l, rt, ym, yp, q0[rr][0], q0[rr][2]);
                    bool m[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) m[j] = zin && in1y[rr] && in1x[j];
                    res[rr] = sel(m, v, c);
                }
                float* s1p = s1 + (z1 & 1) * kP1;
                *reinterpret_cast<float4*>(s1p + (2 * warp) * kBoxW + 4 * lane) = res[0];
                *reinterpret_cast<float4*>(s1p + (2 * warp + 1) * kBoxW + 4 * lane) = res[1];
#pragma unroll
                for (int rr = 0; rr < 2; ++rr) {
                    q1[rr][0] = q1[rr][1];
                    q1[rr][1] = q1[rr][2];
                    q1[rr][2] = res[rr];
                }
            }
            // ---- stage 2 at plane z2 = p-2 (stage-1 planes z2-1 .. z2+1 in q1)
            if (pr >= 4) {
                const int z2 = p - 2;
                const float* sp = s1 + (z2 & 1) * kP1;              // stage-1 plane z2
                const int wu = 2 * warp - 1, wd = 2 * warp + 2;     // rows of other warps
                const float4 up = wu >= 0 ? *reinterpret_cast<const float4*>(sp + wu * kBoxW + 4 * lane)
                                          : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 dn = wd < kRows1 ? *reinterpret_cast<const float4*>(sp + wd * kBoxW + 4 * lane)
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
                const bool zin = z2 >= lo2[2] && z2 <= hi2[2] && z2 >= zs && z2 <= ze;
#pragma unroll
                for (int rr = 0; rr < 2; ++rr) {
                    const float4 c = q1[rr][1];
                    const float l = __shfl_up_sync(0xffffffffu, c.w, 1);
                    const float rt = __shfl_down_sync(0xffffffffu, c.x, 1);
                    const float4 ym = rr == 0 ? up : q1[0][1];
                    const float4 yp = rr == 0 ? q1[1][1] : dn;
                    const float4 v = upd(C, c, l, rt, ym, yp, q1[rr][0], q1[rr][2]);
                    if (zin && in2y[rr] && st_any) {
                        float* dst = outb + (long long)z2 * L.plane + (long long)(ya + rr) * L.P;
                        if (st_all) {
                            *reinterpret_cast<float4*>(dst) = v;
                        } else {
                            if (in2x[0]) dst[0] = v.x;
                            if (in2x[1]) dst[1] = v.y;
                            if (in2x[2]) dst[2] = v.z;
                            if (in2x[3]) dst[3] = v.w;
                        }
                    }
                }
            }
            __syncthreads();
            if (*abort_flag) {
                aborted = true;
                stop = g;
                break;
            }
            // plane p-1 is no longer needed: refill its slot with plane p-1+S
            if (pr >= 1) {
                const int nxt = pr - 1 + kS2;
                if (nxt < np) {
                    const unsigned g2 = gp + nxt;
                    if (tid == 0) {
                        mbar_expect_tx(&bar[g2 % kS2], kPlane * 4);
                        tma_load_4d(ring + (g2 % kS2) * kPlane, &tin, xs0, y0 - 2, first + nxt, blk,
                                    &bar[g2 % kS2]);
                    }
                    issued_hi = g2 + 1;
                }
            }
        }
        if (!aborted) gp += np;
    }
    if (aborted && tid == 0) {
        report(status, DEV_TIMEOUT);
        for (unsigned g = stop; g < issued_hi; ++g) mbar_wait_bounded(&bar[g % kS2], (g / kS2) & 1, 100000000ull);
    }
}

}  // namespace

int heat2_box_w() { return kBoxW; }
int heat2_box_h() { return kBoxH; }

cudaError_t launch_heat_substep2(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                                 const HeatCoef& c, int* status, cudaStream_t st, int zchunk)
{
    static int resident = 0;
    if (resident == 0) {
        cudaError_t e = cudaFuncSetAttribute(heat2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kSmem2);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0, occ = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, heat2_kernel, kT2, kSmem2);
        if (e != cudaSuccess) return e;
        resident = (occ > 0 ? occ : 1) * (sms > 0 ? sms : 1);
    }
    H2Sched sch;
    sch.out0 = (L.xoff + 1) & ~3;                       // aligned float4 holding x = 1
    const int xend = L.xoff + L.n[0] - 1;               // storage x one past the last region cell
    sch.ntx = (xend - sch.out0 + kOutW - 1) / kOutW;
    sch.nty = (L.n[1] - 2 + kOutH - 1) / kOutH;
    sch.NZ = L.n[2] - 2;
    const long long tiles = (long long)sch.ntx * sch.nty * L.nblk;
    int Lz = zchunk > 0 ? zchunk : 16;
    if (zchunk <= 0 && tiles * ((sch.NZ + 15) / 16) < 2LL * resident) {
        long long nzc = (2LL * resident + tiles - 1) / tiles;
        if (nzc > sch.NZ / 4) nzc = sch.NZ / 4 > 0 ? sch.NZ / 4 : 1;
        Lz = (int)((sch.NZ + nzc - 1) / nzc);
    }
    if (Lz > sch.NZ) Lz = sch.NZ;
    sch.Lz = Lz;
    sch.nzc = (sch.NZ + Lz - 1) / Lz;
    sch.U = tiles * sch.nzc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(sch.U < 1 ? 1 : sch.U));
    cfg.blockDim = dim3(kT2);
    cfg.dynamicSmemBytes = kSmem2;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, heat2_kernel, *tin, out, L, step_i, c, sch, status);
    count_launches(1);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace b2r
