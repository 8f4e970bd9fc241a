// gol.cu -- 3-D Game of Life generation on the resident blocks.
//
// Replaces gol_3d_kernel (gol-3D.cu:30-102).  Rule (gol-3D.cu:83-99 and its
// comment at gol-3D.cu:104-117): with n = number of live cells among the 26
// neighbours, a live cell with n <= 1 or n >= 8 dies, a dead cell with
// n == 5 is born, every other cell keeps its state (the reference leaves
// such cells unwritten, which with its ping-pong buffers yields the state of
// two generations back; this kernel writes the current state).
//
// Kernel shape: cells are bytes, processed four to a 32-bit word (SWAR).  A
// warp owns 32 consecutive words of a row (lanes 1..30 produce output, lanes
// 0 and 31 only supply the x neighbours), RY rows plus one halo row above
// and below, and marches z.  Per plane: the 3-plane column sum comes from a
// register queue (max 3 per byte), the 3-row sum from registers, the 3-cell
// x sum from two funnel shifts with the neighbour lanes' words (max 27 per
// byte, no carries), then the rule is applied to four cells at once with
// byte-wise compares.  Every load is a coalesced 128-byte warp row; the
// halo rows re-read by the next warp come from L1/L2.
#include "b2r_common.cuh"
#include "gol.h"

namespace b2r {

namespace {

constexpr int kRY = 8;           // output rows per warp
constexpr int kGolWarps = 4;     // warps per CTA, stacked in y
constexpr int kOutWords = 30;    // output words per warp row

__device__ __forceinline__ uint32_t ldw(const uint32_t* p) { return __ldg(p); }

// Per-byte rule on counts (0..26) and current states (0/1).
__device__ __forceinline__ uint32_t life_rule(uint32_t cnt, uint32_t cur)
{
    const uint32_t alive = cur * 0xFFu;                    // 0x00/0xFF per byte
    const uint32_t le1 = __vcmpleu4(cnt, 0x01010101u);
    const uint32_t ge8 = __vcmpgeu4(cnt, 0x08080808u);
    const uint32_t eq5 = __vcmpeq4(cnt, 0x05050505u);
    const uint32_t nxt = (alive & ~(le1 | ge8)) | (~alive & eq5);
    return nxt & 0x01010101u;
}

__global__ void __launch_bounds__(32 * kGolWarps)
gol_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, const BlockLayout L,
           const int step_i, const int nzc)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const int edge = edge_bits(L, blk);
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) stage_region(L, edge, a, step_i + 1, lo[a], hi[a]);

    const int wb = (L.xoff + 1) >> 2;                       // first word with an updatable cell
    const int w = wb + blockIdx.x * kOutWords + lane - 1;    // this lane's word (storage)
    const int y0 = 1 + (blockIdx.y * kGolWarps + warp) * kRY;
    const int nz_out = hi[2] - lo[2] + 1;
    const int per = (nz_out + nzc - 1) / nzc;
    const int zs = lo[2] + zc * per;
    const int ze = min(hi[2], zs + per - 1);
    if (nz_out <= 0 || zs > ze || y0 > hi[1]) return;       // warp-uniform

    // byte mask of cells of this word inside the x window
    const int xc = 4 * w - L.xoff;                          // block x of byte 0
    uint32_t xmask = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (xc + j >= lo[0] && xc + j <= hi[0]) xmask |= 0xFFu << (8 * j);
    const bool producer = lane >= 1 && lane <= kOutWords;

    const int wpr = L.P >> 2;                               // words per row
    const uint32_t* inw = reinterpret_cast<const uint32_t*>(in + (long long)blk * L.bstride);
    uint32_t* outw = reinterpret_cast<uint32_t*>(out + (long long)blk * L.bstride);
    const long long wplane = L.plane >> 2;

    // column queue: planes z-1, z, z+1 of rows y0-1 .. y0+kRY
    uint32_t qa[kRY + 2], qb[kRY + 2], qc[kRY + 2];
    auto load_plane = [&](int z, uint32_t* q) {
        const uint32_t* p = inw + (long long)z * wplane + w;
#pragma unroll
        for (int r = 0; r < kRY + 2; ++r) {
            const int y = y0 - 1 + r;
            q[r] = (y < L.n[1] && w < wpr) ? ldw(p + (long long)y * wpr) : 0u;
        }
    };
    load_plane(zs - 1, qa);
    load_plane(zs, qb);
    for (int z = zs; z <= ze; ++z) {
        load_plane(z + 1, qc);
        uint32_t s[kRY + 2];
#pragma unroll
        for (int r = 0; r < kRY + 2; ++r) s[r] = qa[r] + qb[r] + qc[r];
#pragma unroll
        for (int r = 0; r < kRY; ++r) {
            const uint32_t v = s[r] + s[r + 1] + s[r + 2];          // 3 rows x 3 planes
            const uint32_t vl = __shfl_up_sync(0xffffffffu, v, 1);
            const uint32_t vr = __shfl_down_sync(0xffffffffu, v, 1);
            const uint32_t box = v + __funnelshift_l(vl, v, 8) + __funnelshift_r(v, vr, 8);
            const uint32_t cur = qb[r + 1];
            const uint32_t nxt = life_rule(box - cur, cur);
            const int y = y0 + r;
            if (producer && xmask && y >= lo[1] && y <= hi[1]) {
                outw[(long long)z * wplane + (long long)y * wpr + w] = (nxt & xmask) | (cur & ~xmask);
            }
        }
#pragma unroll
        for (int r = 0; r < kRY + 2; ++r) {
            qa[r] = qb[r];
            qb[r] = qc[r];
        }
    }
}

}  // namespace

cudaError_t launch_gol_substep(const uint8_t* in, uint8_t* out, const BlockLayout& L, int step_i,
                               cudaStream_t st)
{
    const int wb = (L.xoff + 1) >> 2;
    const int we = (L.xoff + L.n[0] - 2) >> 2;              // last word with an updatable cell
    const int ntx = (we - wb + 1 + kOutWords - 1) / kOutWords;
    const int rows = L.n[1] - 2;
    const int nty = (rows + kRY * kGolWarps - 1) / (kRY * kGolWarps);
    const long long tiles = (long long)ntx * nty * L.nblk;
    // small blocks are latency bound (a generation of a 136^3 block is a few
    // microseconds of data): short z chunks, many CTAs
    const long long want = 152LL * 12;
    int nzc = (int)((want + tiles - 1) / tiles);
    const int maxc = (L.n[2] - 2) / 4 > 0 ? (L.n[2] - 2) / 4 : 1;
    if (nzc > maxc) nzc = maxc;
    if (nzc < 1) nzc = 1;
    dim3 grid(ntx, nty, L.nblk * nzc);
    gol_kernel<<<grid, 32 * kGolWarps, 0, st>>>(in, out, L, step_i, nzc);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace b2r
