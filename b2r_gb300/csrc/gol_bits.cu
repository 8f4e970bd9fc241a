// gol_bits.cu -- Game of Life generation with bit-sliced cells.
//
// Same rule and windows as gol.cu (gol-3D.cu:83-99: with n live neighbours
// out of 26, a live cell survives iff 2 <= n <= 7, a dead cell is born iff
// n == 5), computed 32 cells at a time.  A lane holds one 32-cell word of a
// row, one bit per cell (the byte cells of HBM are packed on load with one
// multiply per four cells and unpacked on store), for kRows rows plus one
// halo row above and below, and marches z with a three-plane queue (the
// next plane's bytes are loaded one iteration ahead).  Lanes form segments
// of GW consecutive words of a row (the first and last word of a segment
// only supply x neighbours); a warp holds 32/GW segments stacked in y; the
// four warps of a CTA take four z chunks of the same tile.  The 27-cell
// boxes are added with bit-sliced full adders:
//   * z: three planes -> a 2-bit count per cell of every row;
//   * y: rows r-1, r, r+1 -> a 4-bit count (0..9);
//   * x: the counts of the word and of its neighbour lanes' words shifted
//     by one cell (funnel shifts) -> the 27-cell total T, 5 bits;
//   * rule on T including the cell itself: live -> 3 <= T <= 8, dead ->
//     T == 5.
#include <mutex>
#include <algorithm>

#include "b2r_common.cuh"
#include "gol.h"

namespace b2r {

namespace {

constexpr int kRows = 4;          // output rows per segment
constexpr int kBWarps = 4;        // warps per CTA: four z chunks of the same tile

__device__ __forceinline__ uint32_t pack4(uint32_t w)
{
    // bytes c0..c3 in {0,1} at bits 0, 8, 16, 24 -> c_i at bit 28+i; the
    // other partial products land on distinct bits below 28 (no carries)
    return (w * 0x10204080u) >> 28;
}
__device__ __forceinline__ uint32_t unpack4(uint32_t n)
{
    // bits n0..n3 -> bytes 0/1: bit i lands on i + 7m (m = 0..3), all distinct
    return (n * 0x00204081u) & 0x01010101u;
}
__device__ __forceinline__ uint32_t pack32(const uint4& a, const uint4& b)
{
    return pack4(a.x) | (pack4(a.y) << 4) | (pack4(a.z) << 8) | (pack4(a.w) << 12) | (pack4(b.x) << 16) |
           (pack4(b.y) << 20) | (pack4(b.z) << 24) | (pack4(b.w) << 28);
}
__device__ __forceinline__ void unpack32(uint32_t v, uint4& a, uint4& b)
{
    a = make_uint4(unpack4(v & 15u), unpack4((v >> 4) & 15u), unpack4((v >> 8) & 15u), unpack4((v >> 12) & 15u));
    b = make_uint4(unpack4((v >> 16) & 15u), unpack4((v >> 20) & 15u), unpack4((v >> 24) & 15u),
                   unpack4(v >> 28));
}
__device__ __forceinline__ uint32_t xor3(uint32_t a, uint32_t b, uint32_t c) { return a ^ b ^ c; }
__device__ __forceinline__ uint32_t maj(uint32_t a, uint32_t b, uint32_t c) { return (a & b) | (c & (a ^ b)); }

struct GolBitsGeom {
    int kx0;      // first output word (32-byte units of the storage row) of tile 0
    int y0;       // first output row
    int nzc;      // z chunks per block
    int nzg;      // CTAs per block along z (kBWarps chunks each)
};

#ifndef B2R_GOLB_MINB
#define B2R_GOLB_MINB 5   // resident CTAs per SM the register budget is fitted to
#endif

template <int GW>
__global__ void __launch_bounds__(32 * kBWarps, B2R_GOLB_MINB)
gol_bits_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, const BlockLayout L, const int step_i,
                const GolBitsGeom G)
{
    constexpr int kOut = GW - 2, kSegs = 32 / GW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int l = lane % GW, sg = lane / GW;
    const int blk = blockIdx.z / G.nzg, zc = (blockIdx.z % G.nzg) * kBWarps + warp;
    const int edge = edge_bits(L, blk);
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) stage_region(L, edge, a, step_i + 1, lo[a], hi[a]);
    const int nz = hi[2] - lo[2] + 1;
    const int per = (nz + G.nzc - 1) / G.nzc;
    const int zs = lo[2] + zc * per, ze = min(hi[2], zs + per - 1);
    const int wy0 = G.y0 + blockIdx.y * kSegs * kRows;  // first row of the warp
    if (zc >= G.nzc || nz <= 0 || zs > ze || wy0 > hi[1]) return;   // warp-uniform: no barrier here
    const int y0 = wy0 + sg * kRows;                     // first output row of this lane's segment
    const int kw = G.kx0 + blockIdx.x * kOut + l - 1;    // this lane's word
    const int wpr = L.P >> 5;                            // 32-byte words per row
    const bool wload = kw >= 0 && kw < wpr;
    // bits of the x window in this word
    uint32_t xm = 0;
    {
        const int x0 = 32 * kw - L.xoff;
        const int a = max(lo[0] - x0, 0), b = min(hi[0] - x0, 31);
        if (a <= b) xm = (b - a == 31) ? 0xFFFFFFFFu : (((1u << (b - a + 1)) - 1u) << a);
    }
    const bool producer = l >= 1 && l <= kOut && xm != 0u;
    const uint8_t* inb = in + (long long)blk * L.bstride + 32LL * kw;
    uint8_t* outb = out + (long long)blk * L.bstride + 32LL * kw;

    // rows y0-1 .. y0+kRows of planes z-1, z, z+1 (packed) and of plane z+2
    // (raw bytes, loaded one iteration ahead and packed at its end)
    uint32_t qa[kRows + 2], qb[kRows + 2], qc[kRows + 2];
    uint4 ra[kRows + 2], rb[kRows + 2];
    bool rowok[kRows + 2];
#pragma unroll
    for (int r = 0; r < kRows + 2; ++r) {
        const int y = y0 - 1 + r;
        rowok[r] = wload && y >= 0 && y < L.n[1];
    }
    auto load_raw = [&](int z) {
        const uint8_t* p = inb + (long long)z * L.plane + (long long)(y0 - 1) * L.P;
#pragma unroll
        for (int r = 0; r < kRows + 2; ++r) {
            ra[r] = rb[r] = make_uint4(0u, 0u, 0u, 0u);
            if (rowok[r]) {
                const uint4* s = reinterpret_cast<const uint4*>(p + (long long)r * L.P);
                ra[r] = __ldg(s);
                rb[r] = __ldg(s + 1);
            }
        }
    };
    auto pack_raw = [&](uint32_t* q) {
#pragma unroll
        for (int r = 0; r < kRows + 2; ++r) q[r] = pack32(ra[r], rb[r]);
    };
    load_raw(zs - 1);
    pack_raw(qa);
    load_raw(zs);
    pack_raw(qb);
    load_raw(zs + 1);
    pack_raw(qc);
    for (int z = zs; z <= ze; ++z) {
        if (z + 2 <= ze + 1) load_raw(z + 2);
        // z: 2-bit column counts of every row
        uint32_t c0[kRows + 2], c1[kRows + 2];
#pragma unroll
        for (int r = 0; r < kRows + 2; ++r) {
            c0[r] = xor3(qa[r], qb[r], qc[r]);
            c1[r] = maj(qa[r], qb[r], qc[r]);
        }
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
            // y: rows r, r+1, r+2 (centre r+1) -> 4-bit counts v0..v3
            const uint32_t k1 = maj(c0[r], c0[r + 1], c0[r + 2]);
            const uint32_t t = xor3(c1[r], c1[r + 1], c1[r + 2]), d = maj(c1[r], c1[r + 1], c1[r + 2]);
            const uint32_t e = t & k1;
            const uint32_t v0 = xor3(c0[r], c0[r + 1], c0[r + 2]), v1 = t ^ k1, v2 = d ^ e, v3 = d & e;
            // x: the neighbour lanes' counts, shifted by one cell
            const uint32_t p0 = __shfl_up_sync(0xffffffffu, v0, 1, GW), n0 = __shfl_down_sync(0xffffffffu, v0, 1, GW);
            const uint32_t p1 = __shfl_up_sync(0xffffffffu, v1, 1, GW), n1 = __shfl_down_sync(0xffffffffu, v1, 1, GW);
            const uint32_t p2 = __shfl_up_sync(0xffffffffu, v2, 1, GW), n2 = __shfl_down_sync(0xffffffffu, v2, 1, GW);
            const uint32_t p3 = __shfl_up_sync(0xffffffffu, v3, 1, GW), n3 = __shfl_down_sync(0xffffffffu, v3, 1, GW);
            const uint32_t l0 = __funnelshift_l(p0, v0, 1), r0 = __funnelshift_r(v0, n0, 1);
            const uint32_t l1 = __funnelshift_l(p1, v1, 1), r1 = __funnelshift_r(v1, n1, 1);
            const uint32_t l2 = __funnelshift_l(p2, v2, 1), r2 = __funnelshift_r(v2, n2, 1);
            const uint32_t l3 = __funnelshift_l(p3, v3, 1), r3 = __funnelshift_r(v3, n3, 1);
            const uint32_t s0 = xor3(l0, v0, r0), kk1 = maj(l0, v0, r0);
            const uint32_t t1 = xor3(l1, v1, r1), m1 = maj(l1, v1, r1);
            const uint32_t s1 = t1 ^ kk1, k2 = t1 & kk1;
            const uint32_t t2 = xor3(l2, v2, r2), m2 = maj(l2, v2, r2);
            const uint32_t s2 = xor3(t2, m1, k2), k3 = maj(t2, m1, k2);
            const uint32_t t3 = xor3(l3, v3, r3), m3 = maj(l3, v3, r3);
            const uint32_t s3 = xor3(t3, m2, k3), k4 = maj(t3, m2, k3);
            const uint32_t s4 = m3 ^ k4;
            // T = s4..s0, the 27-cell total; live: 3 <= T <= 8, dead: T == 5
            const uint32_t born = ~s4 & ~s3 & s2 & ~s1 & s0;
            const uint32_t surv = ~s4 & ((~s3 & (s2 | (s1 & s0))) | (s3 & ~s2 & ~s1 & ~s0));
            const uint32_t cur = qb[r + 1];
            const int y = y0 + r;
            if (producer && y >= lo[1] && y <= hi[1]) {
                const uint32_t nxt = (cur & surv) | (~cur & born);
                const uint32_t res = (nxt & xm) | (cur & ~xm);
                uint4 a, b;
                unpack32(res, a, b);
                uint4* dst = reinterpret_cast<uint4*>(outb + (long long)z * L.plane + (long long)y * L.P);
                dst[0] = a;
                dst[1] = b;
            }
        }
#pragma unroll
        for (int r = 0; r < kRows + 2; ++r) {
            qa[r] = qb[r];
            qb[r] = qc[r];
        }
        if (z + 2 <= ze + 1) pack_raw(qc);
    }
}


// ---------------------------------------------------------------- several generations per pass
// Up to kBMaxGen generations of one B2R period in one launch, on bit-sliced
// cells.  A CTA owns a region of GW words of 32 cells (x; one halo word each
// side), PR rows (ng halo rows each side) and a z chunk.  Generation g of a
// plane (level g) is built from level g-1 planes z-1 .. z+1 held in a
// 4-plane ring of bit words per level in shared memory; level g runs 2 planes
// behind level g-1, so a time step reads only planes finished in earlier time
// steps and needs one barrier.  A thread holds one word of 4 rows: z sums
// from the ring, y sums in registers, x sums from the segment's neighbour
// lanes by shuffles.  Level 0 is read (bytes packed to bits) once and the
// last level written (unpacked) once per period.  Each level shrinks the
// valid region by one cell per side as the period's windows do; cells
// outside a sub-step's window keep their value.
constexpr int kBMaxGen = 4;
#ifndef B2R_GOLP_ROWS
#define B2R_GOLP_ROWS 32     // output rows per band at most
#endif
#ifndef B2R_GOLP_MINPER
#define B2R_GOLP_MINPER 3    // CTAs per SM on average the period kernel's grid keeps at least
#endif

struct GolBitsPeriod {
    int ng, i0;          // generations, first sub-step
    int kx0, OW;         // first output word (32-byte units of the row) of tile 0, output words per tile
    int y0, OR, PR;      // first output row, output rows per band, region rows (multiple of 4)
    int nzc;
    int push;            // the pass ends a period: push band cells into the neighbours' halos
};

// The halo exchange folded into the pass that ends a period: after its
// output is stored, each CTA copies the part of its output box that the
// halo gather (halo.cu) would send to the neighbour blocks.  Region d of
// block t is owner t + d's cells p with p_a in [B_a, B_a + H) for d_a < 0,
// [H, 2H) for d_a > 0 and any interior p_a for d_a = 0, stored at p + d B;
// no region crosses a non-periodic domain edge.  Every row piece moves in
// the widest vector that its length and both starts allow.
__device__ __forceinline__ void push_box(const BlockLayout& L, int blk, uint8_t* out, const int (&blo)[3],
                                         const int (&bhi)[3])
{
    const int H = L.H;
    const int bc[3] = {blk % L.nb[0], (blk / L.nb[0]) % L.nb[1], blk / (L.nb[0] * L.nb[1])};
    for (int r = 0; r < 27; ++r) {
        const int d[3] = {r % 3 - 1, (r / 3) % 3 - 1, r / 9 - 1};
        if (r == 13) continue;
        int lo[3], hi[3], t[3];
        bool ok = true;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int sl = d[q] < 0 ? L.B[q] : H, sh = d[q] < 0 ? L.B[q] + H - 1 : (d[q] > 0 ? 2 * H - 1 : H + L.B[q] - 1);
            lo[q] = max(sl, blo[q]);
            hi[q] = min(sh, bhi[q]);
            ok = ok && lo[q] <= hi[q];
            t[q] = bc[q] - d[q];
            if (t[q] < 0 || t[q] >= L.nb[q]) {
                if (!L.periodic) ok = false;
                t[q] = (t[q] + L.nb[q]) % L.nb[q];
            }
        }
        if (!ok) continue;     // uniform over the CTA
        const long long tb = t[0] + (long long)L.nb[0] * (t[1] + L.nb[1] * t[2]);
        const long long so = (long long)blk * L.bstride + L.xoff + lo[0];
        const long long doff = tb * L.bstride - (long long)blk * L.bstride +
                               (long long)d[2] * L.B[2] * L.plane + (long long)d[1] * L.B[1] * L.P + d[0] * L.B[0];
        const int len = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
        int vb = 16;
        while (vb > 1 && ((len % vb) || (so % vb) || ((so + doff) % vb))) vb >>= 1;
        const int nv = len / vb;
        const int total = nv * ny * nz;
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            const int v = e % nv, rr = e / nv;
            const int y = lo[1] + rr % ny, z = lo[2] + rr / ny;
            const long long s0 = so + (long long)z * L.plane + (long long)y * L.P + (long long)v * vb;
            uint8_t* dp = out + s0 + doff;
            const uint8_t* sp = out + s0;
            switch (vb) {
            case 16: *reinterpret_cast<uint4*>(dp) = __ldcg(reinterpret_cast<const uint4*>(sp)); break;
            case 8: *reinterpret_cast<uint2*>(dp) = __ldcg(reinterpret_cast<const uint2*>(sp)); break;
            case 4: *reinterpret_cast<uint32_t*>(dp) = __ldcg(reinterpret_cast<const unsigned int*>(sp)); break;
            case 2: *reinterpret_cast<uint16_t*>(dp) = __ldcg(reinterpret_cast<const unsigned short*>(sp)); break;
            default: *dp = __ldcg(reinterpret_cast<const unsigned char*>(sp)); break;
            }
        }
    }
}

template <int GW>
__global__ void __launch_bounds__(512)
gol_bits_period_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, const BlockLayout L,
                       const GolBitsPeriod G)
{
    extern __shared__ uint32_t bsm[];
    const int ng = G.ng, PR = G.PR;
    constexpr int WP = GW;                       // words per ring row (the region's words)
    const int RP = PR + 2;                       // padded rows (zero row each side)
    const int plane_w = WP * RP;
    uint32_t* ring = bsm;                        // [ng][4][RP][WP]: levels 0 .. ng-1
    const int tid = threadIdx.x;
    for (int i = tid; i < ng * 4 * plane_w; i += blockDim.x) bsm[i] = 0u;
    __syncthreads();
    const int w = tid % GW, yg = tid / GW;       // word of the region, group of 4 rows
    const bool active = yg < PR / 4;

    const int blk = blockIdx.z / G.nzc, zc = blockIdx.z % G.nzc;
    const int edge = edge_bits(L, blk);
    int lo[kBMaxGen + 1][3], hi[kBMaxGen + 1][3];
#pragma unroll
    for (int g = 1; g <= kBMaxGen; ++g)
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (g <= ng) stage_region(L, edge, a, G.i0 + g, lo[g][a], hi[g][a]);
    int flo[3], fhi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) stage_region(L, edge, a, G.i0 + ng, flo[a], fhi[a]);
    const int nzf = fhi[2] - flo[2] + 1;
    const int per = (nzf + G.nzc - 1) / G.nzc;
    const int zs = flo[2] + zc * per, ze = min(fhi[2], zs + per - 1);
    if (nzf <= 0 || zs > ze) return;                               // uniform
    const int kw = G.kx0 + blockIdx.x * G.OW - 1 + w;              // storage word of this lane
    const int yb = G.y0 - ng + blockIdx.y * G.OR;                  // block row of region row 0
    const int wpr = L.P >> 5;
    const bool wload = active && kw >= 0 && kw < wpr;
    const bool wout = active && w >= 1 && w <= G.OW && kw >= 0 && kw < wpr;
    // window bits of this word for every level
    uint32_t xm[kBMaxGen + 1];
#pragma unroll
    for (int g = 1; g <= kBMaxGen; ++g) {
        xm[g] = 0u;
        if (g <= ng) {
            const int x0 = 32 * kw - L.xoff;
            const int a = max(lo[g][0] - x0, 0), b = min(hi[g][0] - x0, 31);
            if (a <= b) xm[g] = (b - a == 31) ? 0xFFFFFFFFu : (((1u << (b - a + 1)) - 1u) << a);
        }
    }
    const uint8_t* inb = in + (long long)blk * L.bstride + 32LL * kw;
    uint8_t* outb = out + (long long)blk * L.bstride + 32LL * kw;

    // level-0 rows of the next plane, loaded one time step ahead
    uint4 pa[4], pb[4];
    auto load0 = [&](int z) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int y = yb + yg * 4 + k;
            pa[k] = pb[k] = make_uint4(0u, 0u, 0u, 0u);
            // planes and rows beyond the block read as dead: they feed only
            // cells outside the windows (a fixed shell shallower than the
            // generations of the pass), which keep their values
            if (wload && z >= 0 && z <= ze + ng && z < L.n[2] && y >= 0 && y < L.n[1]) {
                const uint4* s = reinterpret_cast<const uint4*>(inb + (long long)z * L.plane + (long long)y * L.P);
                pa[k] = __ldg(s);
                pb[k] = __ldg(s + 1);
            }
        }
    };
    load0(zs - ng);
    const int nt = ze - zs + 3 * ng + 1;
    for (int t = 0; t < nt; ++t) {
        __syncthreads();
        const int z0 = zs - ng + t;
        if (active && z0 <= ze + ng) {
            uint32_t* dst = ring + (z0 & 3) * plane_w + (yg * 4 + 1) * WP + w;
#pragma unroll
            for (int k = 0; k < 4; ++k) dst[k * WP] = pack32(pa[k], pb[k]);
        }
        load0(z0 + 1);
#pragma unroll
        for (int g = 1; g <= kBMaxGen; ++g) {
            const int zg = z0 - 2 * g;
            // uniform over the CTA: every lane takes part in the shuffles
            if (g > ng || zg < zs - (ng - g) || zg > ze + (ng - g)) continue;
            const uint32_t* src = ring + (g - 1) * 4 * plane_w + (yg * 4) * WP + w;   // padded row yg*4 = row -1
            const uint32_t* qa = src + ((zg - 1) & 3) * plane_w;
            const uint32_t* qb = src + (zg & 3) * plane_w;
            const uint32_t* qc = src + ((zg + 1) & 3) * plane_w;
            uint32_t c0[6], c1[6], cur[4];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const uint32_t a = active ? qa[k * WP] : 0u, b = active ? qb[k * WP] : 0u,
                               c = active ? qc[k * WP] : 0u;
                c0[k] = xor3(a, b, c);
                c1[k] = maj(a, b, c);
                if (k >= 1 && k <= 4) cur[k - 1] = b;
            }
            const bool zin = zg >= lo[g][2] && zg <= hi[g][2];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t k1 = maj(c0[k], c0[k + 1], c0[k + 2]);
                const uint32_t tt = xor3(c1[k], c1[k + 1], c1[k + 2]), d = maj(c1[k], c1[k + 1], c1[k + 2]);
                const uint32_t e = tt & k1;
                const uint32_t v0 = xor3(c0[k], c0[k + 1], c0[k + 2]), v1 = tt ^ k1, v2 = d ^ e, v3 = d & e;
                const uint32_t p0 = __shfl_up_sync(0xffffffffu, v0, 1, GW), n0 = __shfl_down_sync(0xffffffffu, v0, 1, GW);
                const uint32_t p1 = __shfl_up_sync(0xffffffffu, v1, 1, GW), n1 = __shfl_down_sync(0xffffffffu, v1, 1, GW);
                const uint32_t p2 = __shfl_up_sync(0xffffffffu, v2, 1, GW), n2 = __shfl_down_sync(0xffffffffu, v2, 1, GW);
                const uint32_t p3 = __shfl_up_sync(0xffffffffu, v3, 1, GW), n3 = __shfl_down_sync(0xffffffffu, v3, 1, GW);
                const uint32_t l0 = __funnelshift_l(p0, v0, 1), r0 = __funnelshift_r(v0, n0, 1);
                const uint32_t l1 = __funnelshift_l(p1, v1, 1), r1 = __funnelshift_r(v1, n1, 1);
                const uint32_t l2 = __funnelshift_l(p2, v2, 1), r2 = __funnelshift_r(v2, n2, 1);
                const uint32_t l3 = __funnelshift_l(p3, v3, 1), r3 = __funnelshift_r(v3, n3, 1);
                const uint32_t s0 = xor3(l0, v0, r0), kk1 = maj(l0, v0, r0);
                const uint32_t t1 = xor3(l1, v1, r1), m1 = maj(l1, v1, r1);
                const uint32_t s1 = t1 ^ kk1, k2 = t1 & kk1;
                const uint32_t t2 = xor3(l2, v2, r2), m2 = maj(l2, v2, r2);
                const uint32_t s2 = xor3(t2, m1, k2), k3 = maj(t2, m1, k2);
                const uint32_t t3 = xor3(l3, v3, r3), m3 = maj(l3, v3, r3);
                const uint32_t s3 = xor3(t3, m2, k3), k4 = maj(t3, m2, k3);
                const uint32_t s4 = m3 ^ k4;
                const uint32_t born = ~s4 & ~s3 & s2 & ~s1 & s0;
                const uint32_t surv = ~s4 & ((~s3 & (s2 | (s1 & s0))) | (s3 & ~s2 & ~s1 & ~s0));
                const uint32_t c = cur[k];
                const int r = yg * 4 + k, y = yb + r;
                const uint32_t m = (zin && y >= lo[g][1] && y <= hi[g][1]) ? xm[g] : 0u;
                const uint32_t nxt = (((c & surv) | (~c & born)) & m) | (c & ~m);
                if (!active) continue;
                if (g < ng) {
                    ring[(g * 4 + (zg & 3)) * plane_w + (r + 1) * WP + w] = nxt;
                } else if (wout && zg >= zs && zg <= ze && r >= ng && r < ng + G.OR && y >= flo[1] &&
                           y <= fhi[1] && xm[g]) {
                    uint4 a, b;
                    unpack32(nxt, a, b);
                    uint4* d = reinterpret_cast<uint4*>(outb + (long long)zg * L.plane + (long long)y * L.P);
                    d[0] = a;
                    d[1] = b;
                }
            }
        }
    }
    if (G.push) {
        // the pass ends a period: copy this CTA's band cells, just written
        // and still in L2, into the neighbours' halos
        __syncthreads();
        int box_lo[3], box_hi[3];
        const int kwa = G.kx0 + blockIdx.x * G.OW;
        box_lo[0] = max(32 * kwa - L.xoff, flo[0]);
        box_hi[0] = min(32 * (kwa + G.OW) - L.xoff - 1, fhi[0]);
        box_lo[1] = max(yb + ng, flo[1]);
        box_hi[1] = min(yb + ng + G.OR - 1, fhi[1]);
        box_lo[2] = zs;
        box_hi[2] = ze;
        push_box(L, blk, out, box_lo, box_hi);
    }
}

}  // namespace

cudaError_t launch_gol_bits_substep(const uint8_t* in, uint8_t* out, const BlockLayout& L, int step_i,
                                   cudaStream_t st)
{
    // output words and rows over the union of the blocks' windows
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-1, -1, -1};
    for (int b = 0; b < L.nblk; ++b) {
        const int e = edge_bits(L, b);
        for (int a = 0; a < 3; ++a) {
            int l, h;
            stage_region(L, e, a, step_i + 1, l, h);
            lo[a] = std::min(lo[a], l);
            hi[a] = std::max(hi[a], h);
        }
    }
    if (hi[0] < lo[0] || hi[1] < lo[1] || hi[2] < lo[2]) return cudaSuccess;
    GolBitsGeom G{};
    G.kx0 = (L.xoff + lo[0]) >> 5;
    const int nwt = ((L.xoff + hi[0]) >> 5) - G.kx0 + 1;    // output words per row
    // segment width: the fewest lanes per row (GW lanes give GW - 2 words)
    int GW = 32;
    for (int g : {8, 16, 32})
        if (((nwt + g - 3) / (g - 2)) * g < ((nwt + GW - 3) / (GW - 2)) * GW) GW = g;
    const int ntx = (nwt + GW - 3) / (GW - 2);
    G.y0 = lo[1];
    const int rows_per_warp = (32 / GW) * kRows;
    const int nty = (hi[1] - lo[1] + 1 + rows_per_warp - 1) / rows_per_warp;
    const int nz = hi[2] - lo[2] + 1;
    const long long cols = (long long)ntx * nty * L.nblk;
    // z chunks: about as many warps as fit on the SMs, chunks of at least 3 planes
    int nzc = (int)std::max(1LL, (152LL * kBWarps * B2R_GOLB_MINB + cols - 1) / cols);
    nzc = std::min(nzc, std::max(1, nz / 3));
    G.nzc = nzc;
    G.nzg = (nzc + kBWarps - 1) / kBWarps;
    const dim3 grid(ntx, nty, L.nblk * G.nzg);
    switch (GW) {
    case 8: gol_bits_kernel<8><<<grid, 32 * kBWarps, 0, st>>>(in, out, L, step_i, G); break;
    case 16: gol_bits_kernel<16><<<grid, 32 * kBWarps, 0, st>>>(in, out, L, step_i, G); break;
    default: gol_bits_kernel<32><<<grid, 32 * kBWarps, 0, st>>>(in, out, L, step_i, G); break;
    }
    count_launches(1);
    return cudaGetLastError();
}

int gol_bits_max_generations_per_pass() { return kBMaxGen; }

cudaError_t launch_gol_bits_period(const uint8_t* in, uint8_t* out, const BlockLayout& L, int i0, int ng,
                                   bool push_halos, cudaStream_t st, int rows)
{
    if (ng < 1 || ng > kBMaxGen) return cudaErrorInvalidValue;
    // a block row that is not a multiple of 32 cells ends in a word that the
    // pass stores whole, stale halo bytes included, which would race with
    // the fill from the neighbour block
    if (push_halos && L.B[0] % 32 != 0) return cudaErrorInvalidValue;
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-1, -1, -1};
    for (int b = 0; b < L.nblk; ++b) {
        const int e = edge_bits(L, b);
        for (int a = 0; a < 3; ++a) {
            int l, h;
            stage_region(L, e, a, i0 + ng, l, h);
            lo[a] = std::min(lo[a], l);
            hi[a] = std::max(hi[a], h);
        }
    }
    if (hi[0] < lo[0] || hi[1] < lo[1] || hi[2] < lo[2]) return cudaSuccess;
    GolBitsPeriod G{};
    G.ng = ng;
    G.i0 = i0;
    G.push = push_halos ? 1 : 0;
    G.kx0 = (L.xoff + lo[0]) >> 5;
    const int nwt = ((L.xoff + hi[0]) >> 5) - G.kx0 + 1;
    int GW = 32;
    for (int g : {8, 16, 32})
        if (((nwt + g - 3) / (g - 2)) * g < ((nwt + GW - 3) / (GW - 2)) * GW) GW = g;
    const int ntx = (nwt + GW - 3) / (GW - 2);
    G.OW = GW - 2;
    // bands of rows: at most `rows` output rows, split evenly
    const int H = hi[1] - lo[1] + 1;
    const int band = rows > 0 ? std::min(rows, H) : B2R_GOLP_ROWS;
    const int nty = (H + band - 1) / band;
    G.OR = (H + nty - 1) / nty;
    G.PR = (G.OR + 2 * ng + 3) / 4 * 4;
    if (GW * (G.PR / 4) > 512) G.PR = 512 / GW * 4, G.OR = G.PR - 2 * ng;
    const int nty2 = (H + G.OR - 1) / G.OR;
    G.y0 = lo[1];
    const long long tiles = (long long)ntx * nty2 * L.nblk;
    const int nz = hi[2] - lo[2] + 1;
    const size_t smem = (size_t)ng * 4 * GW * (G.PR + 2) * sizeof(uint32_t);
    const int threads = (GW * (G.PR / 4) + 31) / 32 * 32;   // whole warps: every lane takes part in the shuffles
    // raised only, per device, under a lock: handles on other host threads share the limit
    static SmemLimit attr[3];
    const int gi = GW == 8 ? 0 : (GW == 16 ? 1 : 2);
    const void* kern = GW == 8 ? (const void*)gol_bits_period_kernel<8>
                     : GW == 16 ? (const void*)gol_bits_period_kernel<16>
                                : (const void*)gol_bits_period_kernel<32>;
    if (cudaError_t e = raise_smem_limit(attr[gi], kern, std::max<size_t>(smem, 48 * 1024))) return e;
    // z chunks per block by the cost model of gol_period_chunks (the kernel
    // needs several CTAs per SM to hide its latencies).  Measured on the
    // 256^3 torus in 2 x 2 x 2 blocks: 987 GLUPS at the count this picks
    // (19), against 928 for 16 and 764-911 for the counts around them.
    int dev = 0, sms = 0, cap = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cap, kern, threads, smem);
    const int nzc = gol_period_chunks(tiles, nz, ng, sms, cap, B2R_GOLP_MINPER);
    G.nzc = nzc;
    const dim3 grid(ntx, nty2, L.nblk * nzc);
    switch (GW) {
    case 8: gol_bits_period_kernel<8><<<grid, threads, smem, st>>>(in, out, L, G); break;
    case 16: gol_bits_period_kernel<16><<<grid, threads, smem, st>>>(in, out, L, G); break;
    default: gol_bits_period_kernel<32><<<grid, threads, smem, st>>>(in, out, L, G); break;
    }
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace b2r
