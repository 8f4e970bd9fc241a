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

}  // namespace b2r
