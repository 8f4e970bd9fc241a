// heat_tb2.cu -- two heat time steps per HBM pass at stencil radius 2
// (fdm_heat_diffuse_delta2, heat-3D.cu:250-335: the 13-point Laplacian of
// 4th order), temporal blocking as in heat_tb.cu for radius 1.
//
// A CTA reads a tile of the field once, advances it two sub-steps on chip
// and writes it once: 4 B of HBM traffic per lattice-site update instead of
// 8.  Bit-identical to two launches of the one-step sweep (heat_unit.cuh):
// every cell runs the same float operations in the same order (a0*u, then per
// distance k = 1, 2 the x, y and z pair sums in fused multiply-adds).
//
// Shape.  CTA = 16 warps; thread = 4 consecutive x cells (float4) of 2 rows;
// a tile row is 16 lanes (64 cells, a warp holding two row pairs), so the CTA
// computes 64 x 64 cells per stage.  Per input plane p (one TMA 4-D box of
// 72 x 68 cells -- the computed cells, 4 more on each side in x and 2 more
// rows on each side in y -- into an S-deep mbarrier ring):
//   stage 1 (sub-step i) computes plane p-2 from the input planes p-4 .. p,
//   read from the ring: x neighbours by shuffles within the row's lanes (the
//   end lanes read the box's extra columns), y neighbours from the box rows;
//   stage 2 (sub-step i+1) computes plane p-4 from stage-1 planes p-6 .. p-2:
//   z neighbours from a 5-plane float4 register queue (its newest plane
//   computed in this iteration), x neighbours by shuffles, y neighbours from
//   the thread's other row or from a 4-plane exchange buffer of stage-1
//   planes written two iterations earlier -- so one barrier per plane orders
//   everything; stage 2 stores the cells still valid (2 from every edge).
// On fixed faces the two shell layers next to the window keep their value at
// stage 1 (the window's first cells use them); nothing else outside a window
// reaches a stored cell.
#include <climits>

#include "b2r_common.cuh"
#include "heat.h"

namespace b2r {
namespace {

constexpr int kD = 2;                     // stencil radius
constexpr int kT = 2;                     // sub-steps per pass
constexpr int kWarps = 16;
constexpr int kThreads = 32 * kWarps;     // 512
constexpr int kLX = 16;                   // lanes per tile row
constexpr int kSEG = 32 / kLX;            // row pairs per warp
constexpr int kCW = 4 * kLX;              // computed cells per row (64)
constexpr int kROWS = 2 * kWarps * kSEG;  // computed rows (64)
constexpr int kBW = kCW + 8, kBH = kROWS + 2 * kD;       // TMA box (72 x 68)
constexpr int kSLOT = (kBW * kBH + 31) / 32 * 32;        // floats per ring slot
constexpr int kS = 7;                     // ring slots: planes p-4 .. p and two ahead
constexpr int kXP = kCW * kROWS;          // floats per exchange plane
constexpr int kNX = 4;                    // exchange planes (by z mod 4)
constexpr int kV = kD * (kT - 1);         // cells lost per side by the last stage (2)
constexpr int kOW = (kCW - 2 * kV) & ~3;  // output cells per tile row (60)
constexpr int kOH = kROWS - 2 * kV;       // output rows (60)
constexpr size_t kSmem = size_t(kS) * kSLOT * 4 + size_t(kNX) * kXP * 4 + kS * 8 + 16 + 128;

struct Tb2Sched {
    int ntx, nty, nzc, Lz;
    int x0;            // storage x of tile column 0's first computed cell (a multiple of 4)
    long long U;
};

__device__ __forceinline__ void pdl_wait2r() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger2r() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

// The radius-2 update of 4 cells in the sweep's order: c centre; l2 l1 /
// r1 r2 = the cells 2 and 1 left of x / 1 and 2 right of x+3; y / z pair
// sums at distance 1 and 2 as float4s.  Packed two-lane FP32 operations
// (each lane the scalar round-to-nearest one, as the sweep computes it).
__device__ __forceinline__ float4 upd2(const HeatCoef& C, float4 c, float l2, float l1, float r1, float r2,
                                       float4 ys1, float4 zs1, float4 ys2, float4 zs2)
{
    const float2 a0 = make_float2(C.a0, C.a0);
    float2 lo = __fmul2_rn(a0, make_float2(c.x, c.y));
    float2 hi = __fmul2_rn(a0, make_float2(c.z, c.w));
    // distance 1
    float2 k = make_float2(C.ax[0], C.ax[0]);
    lo = __ffma2_rn(k, make_float2(l1 + c.y, c.x + c.z), lo);
    hi = __ffma2_rn(k, make_float2(c.y + c.w, c.z + r1), hi);
    k = make_float2(C.ay[0], C.ay[0]);
    lo = __ffma2_rn(k, make_float2(ys1.x, ys1.y), lo);
    hi = __ffma2_rn(k, make_float2(ys1.z, ys1.w), hi);
    k = make_float2(C.az[0], C.az[0]);
    lo = __ffma2_rn(k, make_float2(zs1.x, zs1.y), lo);
    hi = __ffma2_rn(k, make_float2(zs1.z, zs1.w), hi);
    // distance 2
    k = make_float2(C.ax[1], C.ax[1]);
    lo = __ffma2_rn(k, make_float2(l2 + c.z, l1 + c.w), lo);
    hi = __ffma2_rn(k, make_float2(c.x + r1, c.y + r2), hi);
    k = make_float2(C.ay[1], C.ay[1]);
    lo = __ffma2_rn(k, make_float2(ys2.x, ys2.y), lo);
    hi = __ffma2_rn(k, make_float2(ys2.z, ys2.w), hi);
    k = make_float2(C.az[1], C.az[1]);
    lo = __ffma2_rn(k, make_float2(zs2.x, zs2.y), lo);
    hi = __ffma2_rn(k, make_float2(zs2.z, zs2.w), hi);
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

__device__ __forceinline__ float4 sum4(float4 a, float4 b)
{
    const float2 lo = __fadd2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
    const float2 hi = __fadd2_rn(make_float2(a.z, a.w), make_float2(b.z, b.w));
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// bit j of m: cell j of the thread's 4 keeps its value
__device__ __forceinline__ float4 restore_x(unsigned m, float4 v, float4 c)
{
    return make_float4((m & 1u) ? c.x : v.x, (m & 2u) ? c.y : v.y, (m & 4u) ? c.z : v.z, (m & 8u) ? c.w : v.w);
}

struct Tb2Ctx {
    float4 q[5][2];             // stage-1 planes, slot (plane mod 5) by loop phase; [row]
    const float* ring;
    float* xch;                 // kNX stage-1 exchange planes (by z mod 4)
    uint64_t* bar;
    int* abort_flag;
    float* outb;                // out + block + this thread's storage x
    const CUtensorMap* tmap;
    HeatCoef C;
    long long plane, P;
    unsigned gp;
    int np, first, zs, ze, X0, Y0, blk, ya, wrow, lx, tid;
    int zk[4];                  // the two fixed-shell layer planes on each fixed z face, or INT_MIN
    bool yk[2];                 // this thread's rows in a fixed-shell layer
    unsigned xkm;               // this thread's cells in a fixed-shell layer in x
    unsigned mst;               // cells stored by stage 2 (its window, the valid lanes and rows)
    unsigned issued_hi;
    bool aborted;
    unsigned stop;
};

// x neighbours of a row's 4 cells within the tile row's lanes: the left
// lane's last two and the right lane's first two cells
__device__ __forceinline__ void xnb(float4 v, float& l2, float& l1, float& r1, float& r2)
{
    l2 = __shfl_up_sync(0xffffffffu, v.z, 1, kLX);
    l1 = __shfl_up_sync(0xffffffffu, v.w, 1, kLX);
    r1 = __shfl_down_sync(0xffffffffu, v.x, 1, kLX);
    r2 = __shfl_down_sync(0xffffffffu, v.y, 1, kLX);
}

// PH = pr mod 5: stage-1 plane z sits in queue slot (z - first) mod 5
template <int PH>
__device__ __forceinline__ void tb2_iter(Tb2Ctx& c, int pr)
{
    const unsigned g = c.gp + pr;
    if (!mbar_wait_bounded(&c.bar[g % kS], (g / kS) & 1)) *c.abort_flag = 1;
    const int p = c.first + pr;
    const int wrow = c.wrow;
    const int col = 4 + 4 * c.lx;                        // box column of the thread's first cell
    // ---- stage 1 at plane z1 = p-2 (input planes p-4 .. p from the ring)
    if (pr >= 2 * kD) {
        const int z1 = p - kD;
        const float* pm2 = c.ring + ((g - 4) % kS) * kSLOT + col;
        const float* pm1 = c.ring + ((g - 3) % kS) * kSLOT + col;
        const float* pc = c.ring + ((g - 2) % kS) * kSLOT;
        const float* pp1 = c.ring + ((g - 1) % kS) * kSLOT + col;
        const float* pp2 = c.ring + (g % kS) * kSLOT + col;
        const float* pcc = pc + col;
        // box rows of the thread's rows: wrow + 2 + rr
        const float4 c0 = ld4(pcc + (wrow + 2) * kBW), c1 = ld4(pcc + (wrow + 3) * kBW);
        const float4 um2 = ld4(pcc + wrow * kBW), um1 = ld4(pcc + (wrow + 1) * kBW);
        const float4 dp1 = ld4(pcc + (wrow + 4) * kBW), dp2 = ld4(pcc + (wrow + 5) * kBW);
        bool zk = false;
#pragma unroll
        for (int i = 0; i < 4; ++i) zk = zk || z1 == c.zk[i];
        float* xo = c.xch + (size_t)(z1 & (kNX - 1)) * kXP + 4 * c.lx;
        constexpr int NEW = (PH + 3) % 5;               // slot of plane z1 = p - 2
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const float4 ce = rr == 0 ? c0 : c1;
            const int brow = (wrow + 2 + rr) * kBW;
            float l2, l1, r1, r2;
            xnb(ce, l2, l1, r1, r2);
            if (c.lx == 0) {
                l2 = pc[brow + 2];
                l1 = pc[brow + 3];
            }
            if (c.lx == kLX - 1) {
                r1 = pc[brow + 4 + kCW];
                r2 = pc[brow + 5 + kCW];
            }
            const float4 ys1 = rr == 0 ? sum4(um1, c1) : sum4(c0, dp1);
            const float4 ys2 = rr == 0 ? sum4(um2, dp1) : sum4(um1, dp2);
            const float4 zs1 = sum4(ld4(pm1 + (wrow + 2 + rr) * kBW), ld4(pp1 + (wrow + 2 + rr) * kBW));
            const float4 zs2 = sum4(ld4(pm2 + (wrow + 2 + rr) * kBW), ld4(pp2 + (wrow + 2 + rr) * kBW));
            float4 v = upd2(c.C, ce, l2, l1, r1, r2, ys1, zs1, ys2, zs2);
            if (zk || c.yk[rr]) v = ce;
            else if (c.xkm) v = restore_x(c.xkm, v, ce);
            c.q[NEW][rr] = v;
            st4(xo + (wrow + rr) * kCW, v);
        }
    }
    // ---- stage 2 at plane z2 = p-4 (stage-1 planes p-6 .. p-2)
    if (pr >= 4 * kD) {
        const int z2 = p - 2 * kD;
        constexpr int M2 = (PH + 4) % 5, M1 = PH, C0 = (PH + 1) % 5, P1 = (PH + 2) % 5, P2 = (PH + 3) % 5;
        const float* xi = c.xch + (size_t)(z2 & (kNX - 1)) * kXP + 4 * c.lx;
        const int rm2 = wrow - 2 < 0 ? 0 : wrow - 2, rm1 = wrow - 1 < 0 ? 0 : wrow - 1;
        const int rp2 = wrow + 2 >= kROWS ? kROWS - 1 : wrow + 2, rp3 = wrow + 3 >= kROWS ? kROWS - 1 : wrow + 3;
        const float4 um2 = ld4(xi + rm2 * kCW), um1 = ld4(xi + rm1 * kCW);
        const float4 dp1 = ld4(xi + rp2 * kCW), dp2 = ld4(xi + rp3 * kCW);
        const float4 c0 = c.q[C0][0], c1 = c.q[C0][1];
        float4 res[2];
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const float4 ce = rr == 0 ? c0 : c1;
            float l2, l1, r1, r2;
            xnb(ce, l2, l1, r1, r2);       // every lane: the shuffles are warp-wide
            const float4 ys1 = rr == 0 ? sum4(um1, c1) : sum4(c0, dp1);
            const float4 ys2 = rr == 0 ? sum4(um2, dp1) : sum4(um1, dp2);
            const float4 zs1 = sum4(c.q[M1][rr], c.q[P1][rr]);
            const float4 zs2 = sum4(c.q[M2][rr], c.q[P2][rr]);
            res[rr] = upd2(c.C, ce, l2, l1, r1, r2, ys1, zs1, ys2, zs2);
        }
        if (z2 >= c.zs && z2 <= c.ze && c.mst) {
            float* dst = c.outb + (long long)z2 * c.plane + (long long)c.ya * c.P;
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
    __syncthreads();
    if (*c.abort_flag) {
        c.aborted = true;
        c.stop = g;
        return;
    }
    // input plane p-4 is no longer needed: refill its slot with plane p-4+S
    if (pr >= 2 * kD) {
        const int nxt = pr - 2 * kD + kS;
        if (nxt < c.np) {
            const unsigned g2 = c.gp + nxt;
            if (c.tid == 0) {
                mbar_expect_tx(&c.bar[g2 % kS], kBW * kBH * 4);
                tma_load_4d(const_cast<float*>(c.ring) + (g2 % kS) * kSLOT, c.tmap, c.X0 - 4, c.Y0 - kD,
                            c.first + nxt, c.blk, &c.bar[g2 % kS]);
            }
            c.issued_hi = g2 + 1;
        }
    }
}

__global__ void __launch_bounds__(kThreads, 1)
heat_tb2_kernel(const __grid_constant__ CUtensorMap tin, float* __restrict__ out, const BlockLayout L,
                const int step_i, const HeatCoef C, const Tb2Sched sch, int* __restrict__ status)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Tb2Ctx c;
    float* ring = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    c.ring = ring;
    c.xch = ring + kS * kSLOT;
    c.bar = reinterpret_cast<uint64_t*>(c.xch + kNX * kXP);
    c.abort_flag = reinterpret_cast<int*>(c.bar + kS);
    c.tid = threadIdx.x;
    const int lane = c.tid & 31, warp = c.tid >> 5;
    c.lx = lane % kLX;                                  // the thread's lane within its row
    c.wrow = 2 * (warp * kSEG + lane / kLX);            // its first computed row
    c.tmap = &tin;
    c.C = C;
    c.plane = L.plane;
    c.P = L.P;
    if (c.tid == 0) {
        *c.abort_flag = 0;
        for (int s = 0; s < kS; ++s) mbar_init(&c.bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    pdl_wait2r();
    pdl_trigger2r();

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
        for (int a = 0; a < 3; ++a) stage_region(L, edge, a, kD * (step_i + kT), lo[a], hi[a]);
        c.X0 = sch.x0 + tx * kOW;                       // storage x of the first computed cell
        c.Y0 = kD + ty * kOH - kV;                      // block y of computed row 0
        const int zi0 = zc * sch.Lz;
        c.zs = max(kD + zi0, lo[2]);
        c.ze = min(kD - 1 + zi0 + sch.Lz, hi[2]);       // output planes [zs, ze]
        if (c.zs > c.ze) continue;
        const int ox0 = c.X0 + kV - L.xoff, oy0 = c.Y0 + kV;   // first output cell (block x, y)
        if (ox0 > hi[0] || ox0 + kOW - 1 < lo[0]) continue;
        if (oy0 > hi[1] || oy0 + kOH - 1 < lo[1]) continue;
        c.first = c.zs - kD * kT;
        c.np = c.ze + kD * kT - c.first + 1;
        // the fixed-shell layers next to the window on fixed faces
        c.zk[0] = ((edge >> 4) & 1) ? L.H - 2 : INT_MIN;
        c.zk[1] = ((edge >> 4) & 1) ? L.H - 1 : INT_MIN;
        c.zk[2] = ((edge >> 5) & 1) ? L.n[2] - L.H : INT_MIN;
        c.zk[3] = ((edge >> 5) & 1) ? L.n[2] - L.H + 1 : INT_MIN;
        if (c.tid == 0)
            for (int s = 0; s < kS && s < c.np; ++s) {
                const unsigned g = c.gp + s;
                mbar_expect_tx(&c.bar[g % kS], kBW * kBH * 4);
                tma_load_4d(ring + (g % kS) * kSLOT, &tin, c.X0 - 4, c.Y0 - kD, c.first + s, c.blk, &c.bar[g % kS]);
            }
        c.issued_hi = c.gp + min(kS, c.np);

        const int cx = 4 * c.lx;                        // the thread's first computed column
        const int xb = c.X0 + cx - L.xoff;              // its block x
        c.ya = c.Y0 + c.wrow;                           // block y of its first row
        unsigned xkm = 0, mst = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int x = xb + j;
            const bool xk = ((edge & 1) && (x == L.H - 1 || x == L.H - 2)) ||
                            (((edge >> 1) & 1) && (x == L.n[0] - L.H || x == L.n[0] - L.H + 1));
            xkm |= (xk ? 1u : 0u) << j;
        }
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
            const int y = c.ya + rr;
            c.yk[rr] = (((edge >> 2) & 1) && (y == L.H - 1 || y == L.H - 2)) ||
                       (((edge >> 3) & 1) && (y == L.n[1] - L.H || y == L.n[1] - L.H + 1));
            // stored: the last stage's window, the columns and rows still valid
            const bool yin = y >= lo[1] && y <= hi[1] && c.wrow + rr >= kV && c.wrow + rr <= kROWS - 1 - kV;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                mst |= (yin && cx + j >= kV && cx + j <= kV - 1 + kOW && xb + j >= lo[0] && xb + j <= hi[0]
                            ? 1u : 0u) << (4 * rr + j);
        }
        c.xkm = xkm;
        c.mst = mst;
        c.outb = out + (long long)c.blk * L.bstride + c.X0 + cx;

        for (int pr = 0; pr < c.np;) {
            tb2_iter<0>(c, pr++);
            if (c.aborted || pr >= c.np) break;
            tb2_iter<1>(c, pr++);
            if (c.aborted || pr >= c.np) break;
            tb2_iter<2>(c, pr++);
            if (c.aborted || pr >= c.np) break;
            tb2_iter<3>(c, pr++);
            if (c.aborted || pr >= c.np) break;
            tb2_iter<4>(c, pr++);
            if (c.aborted) break;
        }
        if (!c.aborted) c.gp += c.np;
    }
    if (c.aborted && c.tid == 0) {
        report(status, DEV_TIMEOUT);
        for (unsigned g = c.stop; g < c.issued_hi; ++g)
            mbar_wait_bounded(&c.bar[g % kS], (g / kS) & 1, 100000000ull);
    }
}

}  // namespace

int heat_tb2_box_w() { return kBW; }
int heat_tb2_box_h() { return kBH; }

cudaError_t launch_heat_substep_tb2(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                                    const HeatCoef& c, int* status, cudaStream_t st, int zchunk)
{
    static KernelSetup setup;
    int resident = 0;
    if (cudaError_t e = kernel_setup(setup, heat_tb2_kernel, kThreads, kSmem, nullptr, &resident)) return e;
    Tb2Sched sch;
    // tile column 0 outputs from block x = D at the latest; its first
    // computed cell (kV before its first output) on a 16-byte boundary
    sch.x0 = (L.xoff + kD - kV) & ~3;
    const int xend = L.xoff + L.n[0] - kD;              // storage x one past the last region cell
    sch.ntx = (xend - (sch.x0 + kV) + kOW - 1) / kOW;
    sch.nty = (L.n[1] - 2 * kD + kOH - 1) / kOH;
    const int NZ = L.n[2] - 2 * kD;
    const long long tiles = (long long)sch.ntx * sch.nty * L.nblk;
    int Lz = zchunk > 0 ? zchunk : 64;
    if (zchunk <= 0 && tiles * ((NZ + Lz - 1) / Lz) < 2LL * resident) {
        long long nzc = (2LL * resident + tiles - 1) / tiles;
        if (nzc > NZ / 8) nzc = NZ / 8 > 0 ? NZ / 8 : 1;
        Lz = (int)((NZ + nzc - 1) / nzc);
    }
    if (Lz > NZ) Lz = NZ;
    if (Lz < 1) Lz = 1;
    sch.Lz = Lz;
    sch.nzc = (NZ + Lz - 1) / Lz;
    sch.U = tiles * sch.nzc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(sch.U < 1 ? 1 : sch.U));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = kSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, heat_tb2_kernel, *tin, out, L, step_i, c, sch, status);
    count_launches(1);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace b2r
