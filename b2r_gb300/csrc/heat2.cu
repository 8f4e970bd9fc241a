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

// Per-unit state of the plane loop.  The 3-plane queues rotate by index:
// at loop phase PH (= pr mod 3) the newest plane goes to slot PH, so the
// planes p-2, p-1, p sit in slots (PH+1)%3, (PH+2)%3, PH and no register is
// moved.
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
    unsigned issued_hi;
    bool aborted;
    unsigned stop;
};

template <int PH>
__device__ __forceinline__ void h2_iter(H2Ctx& c, int pr)
{
    constexpr int CZ = (PH + 2) % 3, MZ = (PH + 1) % 3, NZ = PH;
    const unsigned g = c.gp + pr;
    if (!mbar_wait_bounded(&c.bar[g % kS2], (g / kS2) & 1)) *c.abort_flag = 1;
    const float* pl = c.ring + (g % kS2) * kPlane;
#pragma unroll
    for (int rr = 0; rr < 2; ++rr)
        c.q0[rr][NZ] = *reinterpret_cast<const float4*>(pl + (2 * c.warp + 1 + rr) * kBoxW + 4 * c.lane);
    const int p = c.first + pr;
    // ---- stage 1 at plane z1 = p-1
    if (pr >= 2) {
        const int z1 = p - 1;
        const float* pc = c.ring + ((g - 1) % kS2) * kPlane;
        const float4 up = *reinterpret_cast<const float4*>(pc + (2 * c.warp) * kBoxW + 4 * c.lane);
        const float4 dn = *reinterpret_cast<const float4*>(pc + (2 * c.warp + 3) * kBoxW + 4 * c.lane);
        const bool zin = z1 >= c.lo1z && z1 <= c.hi1z;
        float* s1p = c.s1 + (z1 & 1) * kP1;
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const float4 ce = c.q0[rr][CZ];
            const float l = __shfl_up_sync(0xffffffffu, ce.w, 1);
            const float rt = __shfl_down_sync(0xffffffffu, ce.x, 1);
            const float4 ym = rr == 0 ? up : c.q0[0][CZ];
            const float4 yp = rr == 0 ? c.q0[1][CZ] : dn;
            const float4 v = upd(c.C, ce, l, rt, ym, yp, c.q0[rr][MZ], c.q0[rr][NZ]);
            float4 res;
            if (zin) {
                res.x = c.m1[rr][0] ? v.x : ce.x;
                res.y = c.m1[rr][1] ? v.y : ce.y;
                res.z = c.m1[rr][2] ? v.z : ce.z;
                res.w = c.m1[rr][3] ? v.w : ce.w;
            } else {
                res = ce;
            }
            *reinterpret_cast<float4*>(s1p + (2 * c.warp + rr) * kBoxW + 4 * c.lane) = res;
            c.q1[rr][NZ] = res;
        }
    }
    // ---- stage 2 at plane z2 = p-2 (stage-1 planes p-3, p-2, p-1 in q1)
    if (pr >= 4) {
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
            const float4 v = upd(c.C, ce, l, rt, ym, yp, c.q1[rr][MZ], c.q1[rr][NZ]);
            if (zin && c.in2y[rr] && c.st_any) {
                float* dst = c.outb + (long long)z2 * c.plane + (long long)(c.ya + rr) * c.P;
                if (c.st_all) {
                    *reinterpret_cast<float4*>(dst) = v;
                } else {
                    if (c.in2x[0]) dst[0] = v.x;
                    if (c.in2x[1]) dst[1] = v.y;
                    if (c.in2x[2]) dst[2] = v.z;
                    if (c.in2x[3]) dst[3] = v.w;
                }
            }
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
        const int nxt = pr - 1 + kS2;
        if (nxt < c.np) {
            const unsigned g2 = c.gp + nxt;
            if (c.tid == 0) {
                mbar_expect_tx(&c.bar[g2 % kS2], kPlane * 4);
                tma_load_4d(const_cast<float*>(c.ring) + (g2 % kS2) * kPlane, c.tmap, c.xs0, c.y0 - 2,
                            c.first + nxt, c.blk, &c.bar[g2 % kS2]);
            }
            c.issued_hi = g2 + 1;
        }
    }
}

__global__ void __launch_bounds__(kT2, 2)
heat2_kernel(const __grid_constant__ CUtensorMap tin, float* __restrict__ out, const BlockLayout L,
             const int step_i, const HeatCoef C, const H2Sched sch, int* __restrict__ status)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    H2Ctx c;
    float* ring = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    c.ring = ring;
    c.s1 = ring + kS2 * kPlane;                          // 2 stage-1 planes
    c.bar = reinterpret_cast<uint64_t*>(c.s1 + 2 * kP1);
    c.abort_flag = reinterpret_cast<int*>(c.bar + kS2);
    c.tid = threadIdx.x;
    c.lane = c.tid & 31;
    c.warp = c.tid >> 5;
    c.tmap = &tin;
    c.C = C;
    c.plane = L.plane;
    c.P = L.P;
    if (c.tid == 0) {
        *c.abort_flag = 0;
        for (int s = 0; s < kS2; ++s) mbar_init(&c.bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    pdl_wait2();
    pdl_trigger2();

    c.gp = 0;
    c.issued_hi = 0;
    c.stop = 0;
    c.aborted = false;
    for (long long u = blockIdx.x; u < sch.U && !c.aborted; u += gridDim.x) {
        const int tx = (int)(u % sch.ntx);
        long long r = u / sch.ntx;
        const int ty = (int)(r % sch.nty);
        r /= sch.nty;
        const int zc = (int)(r % sch.nzc);
        c.blk = (int)(r / sch.nzc);
        const int edge = edge_bits(L, c.blk);
        int lo1[3], hi1[3], lo2[3], hi2[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            stage_region(L, edge, a, step_i + 1, lo1[a], hi1[a]);
            stage_region(L, edge, a, step_i + 2, lo2[a], hi2[a]);
        }
        c.xs0 = sch.out0 - 4 + tx * kOutW;               // storage x of lane 0's first cell
        c.y0 = 1 + ty * kOutH;                           // block y of output row 0
        const int zi0 = zc * sch.Lz;
        c.zs = max(1 + zi0, lo2[2]);
        c.ze = min(zi0 + sch.Lz, hi2[2]);                // output planes [zs, ze]
        if (c.zs > c.ze) continue;
        if (c.xs0 + 4 - L.xoff > hi2[0] || c.xs0 + 123 - L.xoff < lo2[0]) continue;
        if (c.y0 > hi2[1] || c.y0 + kOutH - 1 < lo2[1]) continue;
        c.first = c.zs - 2;                              // first input plane
        c.np = c.ze + 2 - c.first + 1;
        c.lo1z = lo1[2];
        c.hi1z = hi1[2];
        c.lo2z = lo2[2];
        c.hi2z = hi2[2];
        if (c.tid == 0)
            for (int s = 0; s < kS2 && s < c.np; ++s) {
                const unsigned g = c.gp + s;
                mbar_expect_tx(&c.bar[g % kS2], kPlane * 4);
                tma_load_4d(ring + (g % kS2) * kPlane, &tin, c.xs0, c.y0 - 2, c.first + s, c.blk,
                            &c.bar[g % kS2]);
            }
        c.issued_hi = c.gp + min(kS2, c.np);

        // this thread's cells: storage x xs0+4*lane.., stage-1 rows 2w, 2w+1
        const int xb = c.xs0 + 4 * c.lane - L.xoff;      // block x of the first cell
        c.ya = c.y0 - 1 + 2 * c.warp;                    // block y of stage-1 row 2w
        bool in1x[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            in1x[j] = xb + j >= lo1[0] && xb + j <= hi1[0];
            c.in2x[j] = xb + j >= lo2[0] && xb + j <= hi2[0] && c.lane >= 1 && c.lane <= 30;
        }
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const bool y1 = c.ya + rr >= lo1[1] && c.ya + rr <= hi1[1];
#pragma unroll
            for (int j = 0; j < 4; ++j) c.m1[rr][j] = y1 && in1x[j];
        }
        c.in2y[0] = c.ya >= lo2[1] && c.ya <= hi2[1] && 2 * c.warp >= 1;
        c.in2y[1] = c.ya + 1 >= lo2[1] && c.ya + 1 <= hi2[1] && 2 * c.warp + 1 <= kOutH;
        c.st_all = c.in2x[0] && c.in2x[1] && c.in2x[2] && c.in2x[3];
        c.st_any = c.in2x[0] || c.in2x[1] || c.in2x[2] || c.in2x[3];
        c.outb = out + (long long)c.blk * L.bstride + c.xs0 + 4 * c.lane;

        for (int pr = 0; pr < c.np;) {
            h2_iter<0>(c, pr++);
            if (c.aborted || pr >= c.np) break;
            h2_iter<1>(c, pr++);
            if (c.aborted || pr >= c.np) break;
            h2_iter<2>(c, pr++);
            if (c.aborted) break;
        }
        if (!c.aborted) c.gp += c.np;
    }
    if (c.aborted && c.tid == 0) {
        report(status, DEV_TIMEOUT);
        for (unsigned g = c.stop; g < c.issued_hi; ++g)
            mbar_wait_bounded(&c.bar[g % kS2], (g / kS2) & 1, 100000000ull);
    }
}

}  // namespace

int heat2_box_w() { return kBoxW; }
int heat2_box_h() { return kBoxH; }

cudaError_t launch_heat_substep2(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                                 const HeatCoef& c, int* status, cudaStream_t st, int zchunk)
{
    static KernelSetup setup;
    int resident = 0;                          // CTAs resident on the whole GPU
    if (cudaError_t e = kernel_setup(setup, heat2_kernel, kT2, kSmem2, nullptr, &resident)) return e;
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
