// heat_tb.cu -- T = 2, 3 or 4 heat time steps per HBM pass (temporal
// blocking), radius 1.
//
// B2R's deep halo turned inward, deeper than heat2.cu: a CTA reads a tile of
// the field once, advances it T sub-steps on chip and writes it once, so HBM
// traffic per lattice-site update falls to 8/T bytes.  Bit-identical to T
// launches of the plain sweep: every cell runs the same float operations on
// the same inputs (heat-3D.cu:228-231 folded as in heat.cu).
//
// Shape.  CTA = 16 warps; thread = 4 consecutive x cells (float4) of 2 rows;
// a row of the tile is LX lanes (4*LX cells: 128 with LX = 32, 64 with
// LX = 16, a warp then holding two row pairs), so the CTA computes
// 4*LX x 1024/LX cells per stage.  Per input plane p (one TMA 4-D box into an
// S-deep mbarrier ring: the computed cells, 4 more on each side in x for the
// first stage's edge neighbours, 1 more row on each side in y):
//   stage s (sub-step i+s-1), s = 1..T, computes plane p-s: z neighbours from
//   a 3-plane float4 register queue of stage s-1 (its newest plane computed
//   in this same iteration), x neighbours by shuffles within the row's lanes
//   (stage 1's end lanes read the box's extra columns), y neighbours from the
//   thread's other row or, across row pairs, from stage s-1's plane in shared
//   memory (stage 1: the input box; later stages: a 2-plane exchange buffer
//   written one iteration earlier), so one barrier per plane orders
//   everything; stage T stores the cells still valid (T-1 from every edge).
// The valid region shrinks by one cell per stage on each side; on fixed faces
// the shell layer next to the window keeps its value at every stage
// (nothing else outside a window can reach a stored cell).  With T = 4 the
// input queue would not fit the register budget, so stage 1 reads its three
// input planes from the ring (two more slots).
#include <climits>

#include "b2r_common.cuh"
#include "heat.h"
#include "heat_upd.cuh"

namespace b2r {
namespace {

constexpr int kWarps = 16;
constexpr int kThreads = 32 * kWarps;   // 512

template <int T, int LX>
struct TbCfg {
    static constexpr int SEG = 32 / LX;                 // row pairs per warp
    static constexpr int CW = 4 * LX;                   // computed cells per row
    static constexpr int ROWS = 2 * kWarps * SEG;       // computed rows
    static constexpr int BW = CW + 8, BH = ROWS + 2;    // TMA box (cells)
    static constexpr int SLOT = (BW * BH + 31) / 32 * 32;   // floats per ring slot (128-byte multiple)
    static constexpr int XP = CW * ROWS;                // floats per exchange plane
    static constexpr int OW = (CW - 2 * (T - 1)) & ~3;  // output cells per tile row (a 16-byte multiple)
    static constexpr int OH = ROWS + 2 - 2 * T;         // output rows: T-1 .. ROWS-T
    static constexpr bool INQ = T <= 3;                 // input planes queued in registers
    static constexpr int S = INQ ? 4 : 6;               // ring slots
    static constexpr int NQ = INQ ? T : T - 1;          // register queues (stage 0 = input)
    static constexpr size_t SMEM = size_t(S) * SLOT * 4 + size_t(T - 1) * 2 * XP * 4 + S * 8 + 16 + 128;
};

struct TbSched {
    int ntx, nty, nzc, Lz;
    int x0;            // storage x of tile column 0's first computed cell (a multiple of 4)
    long long U;
};

__device__ __forceinline__ void pdl_wait_tb() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger_tb() { asm volatile("griddepcontrol.launch_dependents;"); }

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

// Which cells must keep their value.  A stage's window shrinks by one cell
// per step on an interior face, so in-window cells of a stage use only
// in-window cells of the stage before, and whatever the out-of-window cells
// hold never reaches a stored cell.  On a fixed face the window stays put at
// the shell depth H, and the window's first cells use the shell layer next
// to it (cell H-1, or n-H on the high side): that layer must keep its value
// at every stage.  Deeper shell cells and cells beyond the block are never
// used.  So the only mask is that layer: a plane (the same for the whole
// CTA), a row (the same for a row's lanes) or, in x, cells of one lane;
// bit j of m is cell j of the thread's 4.
__device__ __forceinline__ float4 restore_x(unsigned m, float4 v, float4 c)
{
    return make_float4((m & 1u) ? c.x : v.x, (m & 2u) ? c.y : v.y, (m & 4u) ? c.z : v.z, (m & 8u) ? c.w : v.w);
}

template <int T, int LX>
struct TbCtx {
    using Cfg = TbCfg<T, LX>;
    float4 q[Cfg::NQ][3][2];   // [queue][slot][row]: queue k holds stage k (INQ) or stage k+1
    const float* ring;
    float* xch;                 // [stage 1..T-1][parity] exchange planes
    uint64_t* bar;
    int* abort_flag;
    float* outb;                // out + block + this thread's storage x
    const CUtensorMap* tmap;
    HeatCoef C;
    long long plane, P;
    unsigned gp;
    int np, first, zs, ze, X0, Y0, blk, ya, wrow, lx, tid;
    int zk0, zk1;               // the fixed-shell layer planes (restored at every stage), or INT_MIN
    bool yk[2];                 // this thread's rows in the fixed-shell layer
    bool xkw;                   // some lane of the thread's warp holds a shell cell in x
    unsigned xkm;               // this thread's cells in the fixed-shell layer in x (restore_x())
    unsigned mst;               // cells stored by stage T (its window, the valid lanes and rows)
    unsigned issued_hi;
    bool aborted;
    unsigned stop;
};

// queue index of stage k's output (k >= 1) and of the input (k = 0)
template <int T, int LX>
__device__ __forceinline__ constexpr int qi(int k) { return TbCfg<T, LX>::INQ ? k : k - 1; }

template <int T, int LX>
__device__ __forceinline__ float4 fix(const TbCtx<T, LX>& c, bool zk, int rr, float4 v, float4 ce)
{
    if (zk || c.yk[rr]) return ce;
    if (c.xkm) return restore_x(c.xkm, v, ce);
    return v;
}

template <int T, int LX, int PH>
__device__ __forceinline__ void tb_iter(TbCtx<T, LX>& c, int pr)
{
    using Cfg = TbCfg<T, LX>;
    constexpr int S = Cfg::S, BW = Cfg::BW, CW = Cfg::CW;
    constexpr int NEW = PH, CUR = (PH + 2) % 3, OLD = (PH + 1) % 3;   // planes p, p-1, p-2 of a queue
    const unsigned g = c.gp + pr;
    if (!mbar_wait_bounded(&c.bar[g % S], (g / S) & 1)) *c.abort_flag = 1;
    const int p = c.first + pr;
    const int wrow = c.wrow;
    const int col = 4 + 4 * c.lx;                        // box column of the thread's first cell
    if constexpr (Cfg::INQ) {
        const float* pl = c.ring + (g % S) * Cfg::SLOT + col;
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) c.q[0][NEW][rr] = ld4(pl + (wrow + 1 + rr) * BW);
    }
    // ---- stage 1 at plane p-1
    if (pr >= 2) {
        const int z = p - 1;
        const float* pc = c.ring + ((g - 1) % S) * Cfg::SLOT;
        const float4 up = ld4(pc + wrow * BW + col);
        const float4 dn = ld4(pc + (wrow + 3) * BW + col);
        float4 in[3][2];     // input planes p-2, p-1, p of this thread's rows
        if constexpr (Cfg::INQ) {
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                in[0][rr] = c.q[0][OLD][rr];
                in[1][rr] = c.q[0][CUR][rr];
                in[2][rr] = c.q[0][NEW][rr];
            }
        } else {
            const float* p0 = c.ring + ((g - 2) % S) * Cfg::SLOT + col;
            const float* p2 = c.ring + (g % S) * Cfg::SLOT + col;
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                in[0][rr] = ld4(p0 + (wrow + 1 + rr) * BW);
                in[1][rr] = ld4(pc + (wrow + 1 + rr) * BW + col);
                in[2][rr] = ld4(p2 + (wrow + 1 + rr) * BW);
            }
        }
        const bool zk = z == c.zk0 || z == c.zk1;
        float* xo = c.xch + (size_t)(z & 1) * Cfg::XP + 4 * c.lx;
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const float4 ce = in[1][rr];
            float l = __shfl_up_sync(0xffffffffu, ce.w, 1, LX);
            float r = __shfl_down_sync(0xffffffffu, ce.x, 1, LX);
            if (c.lx == 0) l = pc[(wrow + 1 + rr) * BW + 3];
            if (c.lx == LX - 1) r = pc[(wrow + 1 + rr) * BW + 4 + CW];
            const float4 ym = rr == 0 ? up : in[1][0];
            const float4 yp = rr == 0 ? in[1][1] : dn;
            const float4 v = fix(c, zk, rr, heat_upd4(c.C, ce, l, r, ym, yp, in[0][rr], in[2][rr]), ce);
            c.q[qi<T, LX>(1)][NEW][rr] = v;
            st4(xo + (wrow + rr) * CW, v);
        }
    }
    // ---- stages 2..T at planes p-2 .. p-T
#pragma unroll
    for (int s = 2; s <= T; ++s) {
        if (pr >= 2 * s) {
            const int z = p - s;
            const int qa = qi<T, LX>(s - 1);
            const float* xi = c.xch + (size_t)((s - 2) * 2 + (z & 1)) * Cfg::XP + 4 * c.lx;
            const int ru = wrow - 1 < 0 ? 0 : wrow - 1;
            const int rd = wrow + 2 >= Cfg::ROWS ? Cfg::ROWS - 1 : wrow + 2;
            const float4 up = ld4(xi + ru * CW);
            const float4 dn = ld4(xi + rd * CW);
            const bool zk = s < T && (z == c.zk0 || z == c.zk1);   // stage T stores no shell cell
            float4 res[2];
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const float4 ce = c.q[qa][CUR][rr];
                const float l = __shfl_up_sync(0xffffffffu, ce.w, 1, LX);
                const float r = __shfl_down_sync(0xffffffffu, ce.x, 1, LX);
                const float4 ym = rr == 0 ? up : c.q[qa][CUR][0];
                const float4 yp = rr == 0 ? c.q[qa][CUR][1] : dn;
                const float4 v = heat_upd4(c.C, ce, l, r, ym, yp, c.q[qa][OLD][rr], c.q[qa][NEW][rr]);
                res[rr] = s < T ? fix(c, zk, rr, v, ce) : v;
            }
            if (s < T) {
                float* xo = c.xch + (size_t)((s - 1) * 2 + (z & 1)) * Cfg::XP + 4 * c.lx;
#pragma unroll
                for (int rr = 0; rr < 2; ++rr) {
                    c.q[qi<T, LX>(s)][NEW][rr] = res[rr];
                    st4(xo + (wrow + rr) * CW, res[rr]);
                }
            } else if (z >= c.zs && z <= c.ze && c.mst) {
                float* dst = c.outb + (long long)z * c.plane + (long long)c.ya * c.P;
#pragma unroll
                for (int rr = 0; rr < 2; ++rr) {
                    const unsigned b = (c.mst >> (4 * rr)) & 15u;
                    float* d = dst + rr * c.P;
                    if (b == 15u) {
                        st4(d, res[rr]);
                    } else if (b) {
                        if (b & 1u) d[0] = res[rr].x;
                        if (b & 2u) d[1] = res[rr].y;
                        if (b & 4u) d[2] = res[rr].z;
                        if (b & 8u) d[3] = res[rr].w;
                    }
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
    // the oldest plane still held is no longer needed: refill its slot
    constexpr int lag = Cfg::INQ ? 1 : 2;
    if (pr >= lag) {
        const int nxt = pr - lag + S;
        if (nxt < c.np) {
            const unsigned g2 = c.gp + nxt;
            if (c.tid == 0) {
                mbar_expect_tx(&c.bar[g2 % S], Cfg::BW * Cfg::BH * 4);
                tma_load_4d(const_cast<float*>(c.ring) + (g2 % S) * Cfg::SLOT, c.tmap, c.X0 - 4, c.Y0 - 1,
                            c.first + nxt, c.blk, &c.bar[g2 % S]);
            }
            c.issued_hi = g2 + 1;
        }
    }
}

template <int T, int LX>
__global__ void __launch_bounds__(kThreads, 1)
heat_tb_kernel(const __grid_constant__ CUtensorMap tin, float* __restrict__ out, const BlockLayout L,
               const int step_i, const HeatCoef C, const TbSched sch, int* __restrict__ status)
{
    using Cfg = TbCfg<T, LX>;
    constexpr int S = Cfg::S;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TbCtx<T, LX> c;
    float* ring = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    c.ring = ring;
    c.xch = ring + S * Cfg::SLOT;
    c.bar = reinterpret_cast<uint64_t*>(c.xch + (T - 1) * 2 * Cfg::XP);
    c.abort_flag = reinterpret_cast<int*>(c.bar + S);
    c.tid = threadIdx.x;
    const int lane = c.tid & 31, warp = c.tid >> 5;
    c.lx = lane % LX;                                   // the thread's lane within its row
    c.wrow = 2 * (warp * Cfg::SEG + lane / LX);         // its first computed row
    c.tmap = &tin;
    c.C = C;
    c.plane = L.plane;
    c.P = L.P;
    if (c.tid == 0) {
        *c.abort_flag = 0;
        for (int s = 0; s < S; ++s) mbar_init(&c.bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    pdl_wait_tb();
    pdl_trigger_tb();

    c.gp = 0;
    c.issued_hi = 0;
    c.stop = 0;
    c.aborted = false;
    for (long long u = blockIdx.x; u < sch.U && !c.aborted; u += gridDim.x) {
        const int tx = (int)(u % sch.ntx);
        long long rem = u / sch.ntx;
        const int ty = (int)(rem % sch.nty);
        rem /= sch.nty;
        const int zc = (int)(rem % sch.nzc);
        c.blk = (int)(rem / sch.nzc);
        const int edge = edge_bits(L, c.blk);
        int lo[3], hi[3];           // window of the last stage: the stored cells
#pragma unroll
        for (int a = 0; a < 3; ++a) stage_region(L, edge, a, step_i + T, lo[a], hi[a]);
        c.X0 = sch.x0 + tx * Cfg::OW;                   // storage x of the first computed cell
        c.Y0 = 1 + ty * Cfg::OH - (T - 1);              // block y of computed row 0
        const int zi0 = zc * sch.Lz;
        c.zs = max(1 + zi0, lo[2]);
        c.ze = min(zi0 + sch.Lz, hi[2]);                // output planes [zs, ze]
        if (c.zs > c.ze) continue;
        const int ox0 = c.X0 + T - 1 - L.xoff, oy0 = c.Y0 + T - 1;   // first output cell (block x, y)
        if (ox0 > hi[0] || ox0 + Cfg::OW - 1 < lo[0]) continue;
        if (oy0 > hi[1] || oy0 + Cfg::OH - 1 < lo[1]) continue;
        c.first = c.zs - T;
        c.np = c.ze + T - c.first + 1;
        // the fixed-shell layer next to the window on fixed faces (restore_x())
        c.zk0 = ((edge >> 4) & 1) ? L.H - 1 : INT_MIN;
        c.zk1 = ((edge >> 5) & 1) ? L.n[2] - L.H : INT_MIN;
        if (c.tid == 0)
            for (int s = 0; s < S && s < c.np; ++s) {
                const unsigned g = c.gp + s;
                mbar_expect_tx(&c.bar[g % S], Cfg::BW * Cfg::BH * 4);
                tma_load_4d(ring + (g % S) * Cfg::SLOT, &tin, c.X0 - 4, c.Y0 - 1, c.first + s, c.blk, &c.bar[g % S]);
            }
        c.issued_hi = c.gp + min(S, c.np);

        const int cx = 4 * c.lx;                        // the thread's first computed column
        const int xb = c.X0 + cx - L.xoff;              // its block x
        c.ya = c.Y0 + c.wrow;                           // block y of its first row
        unsigned xkm = 0, mst = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int x = xb + j;
            const bool xk = ((edge & 1) && x == L.H - 1) || (((edge >> 1) & 1) && x == L.n[0] - L.H);
            xkm |= (xk ? 1u : 0u) << j;
        }
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const int y = c.ya + rr;
            c.yk[rr] = (((edge >> 2) & 1) && y == L.H - 1) || (((edge >> 3) & 1) && y == L.n[1] - L.H);
            // stored: the last stage's window, the columns and rows still valid
            const bool yin = y >= lo[1] && y <= hi[1] && c.wrow + rr >= T - 1 && c.wrow + rr <= Cfg::ROWS - T;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                mst |= (yin && cx + j >= T - 1 && cx + j <= T - 2 + Cfg::OW && xb + j >= lo[0] && xb + j <= hi[0]
                            ? 1u : 0u) << (4 * rr + j);
        }
        c.xkm = xkm;
        c.xkw = __any_sync(0xffffffffu, xkm != 0);
        c.mst = mst;
        c.outb = out + (long long)c.blk * L.bstride + c.X0 + cx;

        for (int pr = 0; pr < c.np;) {
            tb_iter<T, LX, 0>(c, pr++);
            if (c.aborted || pr >= c.np) break;
            tb_iter<T, LX, 1>(c, pr++);
            if (c.aborted || pr >= c.np) break;
            tb_iter<T, LX, 2>(c, pr++);
            if (c.aborted) break;
        }
        if (!c.aborted) c.gp += c.np;
    }
    if (c.aborted && c.tid == 0) {
        report(status, DEV_TIMEOUT);
        for (unsigned g = c.stop; g < c.issued_hi; ++g)
            mbar_wait_bounded(&c.bar[g % S], (g / S) & 1, 100000000ull);
    }
}

template <int T, int LX>
cudaError_t launch_tb(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i, const HeatCoef& c,
                      int* status, cudaStream_t st, int zchunk)
{
    using Cfg = TbCfg<T, LX>;
    static KernelSetup setup;
    int resident = 0;
    if (cudaError_t e = kernel_setup(setup, heat_tb_kernel<T, LX>, kThreads, Cfg::SMEM, nullptr, &resident))
        return e;
    TbSched sch;
    // tile column 0 outputs from block x = 1 at the latest; its first computed
    // cell (T - 1 before its first output) on a 16-byte boundary
    sch.x0 = (L.xoff + 1 - (T - 1)) & ~3;
    const int xend = L.xoff + L.n[0] - 1;               // storage x one past the last region cell
    sch.ntx = (xend - (sch.x0 + T - 1) + Cfg::OW - 1) / Cfg::OW;
    sch.nty = (L.n[1] - 2 + Cfg::OH - 1) / Cfg::OH;
    const int NZ = L.n[2] - 2;
    const long long tiles = (long long)sch.ntx * sch.nty * L.nblk;
    int Lz = zchunk > 0 ? zchunk : 64;
    if (zchunk <= 0 && tiles * ((NZ + Lz - 1) / Lz) < 2LL * resident) {
        long long nzc = (2LL * resident + tiles - 1) / tiles;
        if (nzc > NZ / 8) nzc = NZ / 8 > 0 ? NZ / 8 : 1;
        Lz = (int)((NZ + nzc - 1) / nzc);
    }
    if (Lz > NZ) Lz = NZ;
    sch.Lz = Lz;
    sch.nzc = (NZ + Lz - 1) / Lz;
    sch.U = tiles * sch.nzc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(sch.U < 1 ? 1 : sch.U));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, heat_tb_kernel<T, LX>, *tin, out, L, step_i, c, sch, status);
    count_launches(1);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace

int heat_tb_box_w(int narrow) { return narrow ? TbCfg<3, 16>::BW : TbCfg<3, 32>::BW; }
int heat_tb_box_h(int narrow) { return narrow ? TbCfg<3, 16>::BH : TbCfg<3, 32>::BH; }

cudaError_t launch_heat_substep_tb(int T, int narrow, const CUtensorMap* tin, float* out, const BlockLayout& L,
                                   int step_i, const HeatCoef& c, int* status, cudaStream_t st, int zchunk)
{
    switch (T * 2 + (narrow ? 1 : 0)) {
    case 4: return launch_tb<2, 32>(tin, out, L, step_i, c, status, st, zchunk);
    case 5: return launch_tb<2, 16>(tin, out, L, step_i, c, status, st, zchunk);
    case 6: return launch_tb<3, 32>(tin, out, L, step_i, c, status, st, zchunk);
    case 7: return launch_tb<3, 16>(tin, out, L, step_i, c, status, st, zchunk);
    case 8: return launch_tb<4, 32>(tin, out, L, step_i, c, status, st, zchunk);
    case 9: return launch_tb<4, 16>(tin, out, L, step_i, c, status, st, zchunk);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace b2r
