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
#include <mutex>
#include <algorithm>

#include "b2r_common.cuh"
#include "gol.h"

namespace b2r {

namespace {

constexpr int kRY = 8;           // output rows per warp
constexpr int kGolWarps = 4;     // warps per CTA, stacked in y

__device__ __forceinline__ uint32_t ldw(const uint32_t* p) { return __ldg(p); }

// Per-byte rule on counts (0..26) and current states (0/1), in plain 32-bit
// logic: for a byte v < 128, (v + 0x7F) has bit 7 set iff v != 0, with no
// carry into the next byte.  Survive: live and n >= 2 (bits 1..4 of n not
// all zero) and n < 8 (bits 3..4 zero); birth: dead and n == 5.
__device__ __forceinline__ uint32_t life_rule(uint32_t cnt, uint32_t cur)
{
    const uint32_t ge2 = ((cnt & 0x1E1E1E1Eu) + 0x7F7F7F7Fu) & 0x80808080u;
    const uint32_t ge8 = ((cnt & 0x18181818u) + 0x7F7F7F7Fu) & 0x80808080u;
    const uint32_t ne5 = ((cnt ^ 0x05050505u) + 0x7F7F7F7Fu) & 0x80808080u;
    const uint32_t cur7 = cur << 7;
    const uint32_t nxt7 = (cur7 & ge2 & ~ge8) | (~cur7 & ~ne5 & 0x80808080u);
    return nxt7 >> 7;
}

// SEG = lanes per x segment: 32 (one segment per warp, 30 output words), or
// 16 (two segments of 14 output words, stacked in y) when that wastes fewer
// lanes on the row width (a 136-cell row is 34 words: 3 x 16 lanes instead
// of 2 x 32).
template <int SEG>
__global__ void __launch_bounds__(32 * kGolWarps)
gol_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, const BlockLayout L,
           const int step_i, const int nzc)
{
    constexpr int kOut = SEG - 2, kSegs = 32 / SEG;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int l = lane & (SEG - 1), sg = lane / SEG;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const int edge = edge_bits(L, blk);
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) stage_region(L, edge, a, step_i + 1, lo[a], hi[a]);

    const int wb = (L.xoff + 1) >> 2;                       // first word with an updatable cell
    const int w = wb + blockIdx.x * kOut + l - 1;           // this lane's word (storage)
    const int wy0 = 1 + (blockIdx.y * kGolWarps + warp) * kSegs * kRY;   // first row of the warp
    const int y0 = wy0 + sg * kRY;                           // first row of this lane's segment
    const int nz_out = hi[2] - lo[2] + 1;
    const int per = (nz_out + nzc - 1) / nzc;
    const int zs = lo[2] + zc * per;
    const int ze = min(hi[2], zs + per - 1);
    if (nz_out <= 0 || zs > ze || wy0 > hi[1]) return;      // warp-uniform

    // byte mask of cells of this word inside the x window
    const int xc = 4 * w - L.xoff;                          // block x of byte 0
    uint32_t xmask = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (xc + j >= lo[0] && xc + j <= hi[0]) xmask |= 0xFFu << (8 * j);
    const bool producer = l >= 1 && l <= kOut;

    const int wpr = L.P >> 2;                               // words per row
    const uint32_t* inw = reinterpret_cast<const uint32_t*>(in + (long long)blk * L.bstride);
    uint32_t* outw = reinterpret_cast<uint32_t*>(out + (long long)blk * L.bstride);
    const long long wplane = L.plane >> 2;

    // column queue: planes z-1, z, z+1 of rows y0-1 .. y0+kRY, and plane z+2
    // loaded one iteration ahead
    uint32_t qa[kRY + 2], qb[kRY + 2], qc[kRY + 2], qd[kRY + 2];
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
    load_plane(zs + 1, qc);
    for (int z = zs; z <= ze; ++z) {
        if (z + 2 <= ze + 1) load_plane(z + 2, qd);
        uint32_t s[kRY + 2];
#pragma unroll
        for (int r = 0; r < kRY + 2; ++r) s[r] = qa[r] + qb[r] + qc[r];
#pragma unroll
        for (int r = 0; r < kRY; ++r) {
            const uint32_t v = s[r] + s[r + 1] + s[r + 2];          // 3 rows x 3 planes
            const uint32_t vl = __shfl_up_sync(0xffffffffu, v, 1, SEG);
            const uint32_t vr = __shfl_down_sync(0xffffffffu, v, 1, SEG);
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
            qc[r] = qd[r];
        }
    }
}


// ---------------------------------------------------------------- several generations per pass
// Up to kMaxGen generations of one B2R period in one launch.  A CTA owns a
// region of WT words (x; one halo word each side unless at the block edge)
// by 32 rows (y) and marches a z chunk.  Generation g (level g) of a plane is
// built from level g-1 planes z-1 .. z+1, kept in a 4-plane ring per level
// in shared memory; level g runs 2 planes behind level g-1 (skew), so every
// level of a time step reads only planes finished in earlier time steps and
// one barrier per phase suffices.  Level 0 is read from HBM once, the last
// level is written to HBM once: a period costs one pass instead of R.
// Each level shrinks the valid region by one cell per side, as the windows
// of the period's sub-steps do; cells outside a sub-step's window carry
// their previous value, so shells and halos behave exactly as in the
// one-generation kernel.  Intermediate generations are never written to
// HBM: between exchanges only the final window of the period is current.
constexpr int kMaxGen = 4;
constexpr int kPRows = 32;              // region rows
constexpr int kPRowsT = 4;              // rows per thread
constexpr int kPGroups = kPRows / kPRowsT;
constexpr int kPMaxW = 64;              // region words at most

struct GolPeriod {
    int ng, i0;                         // generations, first sub-step
    int wx0, WT, OW;                    // first region word (storage), region / output words per tile
    int y0, OR;                         // first region row of tile 0, output rows per tile
    int nzc;
};

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
gol_period_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, const BlockLayout L,
                  const GolPeriod G)
{
    extern __shared__ uint32_t gsm[];
    const int WT = G.WT, ng = G.ng;
    const int WP = WT + 2;                           // padded words per row (zero word each side)
    const int RP = kPRows + 2;                       // padded rows (zero row each side)
    const int plane_w = WP * RP;
    uint32_t* ring = gsm;                            // [ng][4][RP][WP]: levels 0 .. ng-1
    uint32_t* vbuf = gsm + ng * 4 * plane_w;         // [ng][RP][WP]: column sums of levels 1 .. ng

    const int tid = threadIdx.x;
    const int nthreads = WT * kPGroups;
    // zero the padding once (never written afterwards)
    for (int i = tid; i < ng * 5 * plane_w; i += blockDim.x) gsm[i] = 0u;
    __syncthreads();
    const bool active = tid < nthreads;
    const int w = active ? tid % WT : 0, yg = active ? tid / WT : 0;

    const int blk = blockIdx.z / G.nzc, zc = blockIdx.z % G.nzc;
    const int edge = edge_bits(L, blk);
    int lo[kMaxGen + 1][3], hi[kMaxGen + 1][3];      // window of level g (g >= 1)
#pragma unroll
    for (int g = 1; g <= kMaxGen; ++g)
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (g <= ng) stage_region(L, edge, a, G.i0 + g, lo[g][a], hi[g][a]);
    int flo[3], fhi[3];                               // window of the last level
#pragma unroll
    for (int a = 0; a < 3; ++a) stage_region(L, edge, a, G.i0 + ng, flo[a], fhi[a]);
    const int nzf = fhi[2] - flo[2] + 1;
    const int per = (nzf + G.nzc - 1) / G.nzc;
    const int zs = flo[2] + zc * per, ze = min(fhi[2], zs + per - 1);
    const int wx = G.wx0 + blockIdx.x * G.OW - 1 + w;             // storage word of this thread
    const int yb = G.y0 + blockIdx.y * G.OR;                       // block row of region row 0
    if (nzf <= 0 || zs > ze) return;                               // uniform
    const int wpr = L.P >> 2;
    const long long wplane = L.plane >> 2;
    const uint32_t* inw = reinterpret_cast<const uint32_t*>(in + (long long)blk * L.bstride);
    uint32_t* outw = reinterpret_cast<uint32_t*>(out + (long long)blk * L.bstride);
    // byte masks of this word inside each level's x window; output words
    const int xc = 4 * wx - L.xoff;
    uint32_t xm[kMaxGen + 1];
#pragma unroll
    for (int g = 1; g <= kMaxGen; ++g) {
        xm[g] = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (g <= ng && xc + j >= lo[g][0] && xc + j <= hi[g][0]) xm[g] |= 0xFFu << (8 * j);
    }
    const bool wout = active && w >= 1 && w <= WT - 2 && wx >= 0 && wx < wpr;
    const bool wload = active && wx >= 0 && wx < wpr;

    const int nt = ze - zs + 3 * ng + 1;
    // level 0 rows of the next plane, loaded one time step ahead
    uint32_t pre[kPRowsT];
    auto load0 = [&](int z) {
#pragma unroll
        for (int k = 0; k < kPRowsT; ++k) {
            const int y = yb + yg * kPRowsT + k;
            // planes and rows beyond the block read as dead (see gol_bits.cu)
            pre[k] = (wload && z >= 0 && z <= ze + ng && z < L.n[2] && y >= 0 && y < L.n[1])
                         ? __ldg(inw + (long long)z * wplane + (long long)y * wpr + wx)
                         : 0u;
        }
    };
    load0(zs - ng);
    for (int t = 0; t < nt; ++t) {
        __syncthreads();
        // level 0: plane zs - ng + t
        const int z0 = zs - ng + t;
        if (active && z0 <= ze + ng) {
            uint32_t* dst = ring + (0 * 4 + (z0 & 3)) * plane_w + WP + 1 + w + (yg * kPRowsT) * WP;
#pragma unroll
            for (int k = 0; k < kPRowsT; ++k) dst[k * WP] = pre[k];
        }
        if (active) load0(z0 + 1);
        // levels 1 .. ng: column sums (3 rows x 3 planes) of level g-1 around plane z_g
#pragma unroll
        for (int g = 1; g <= kMaxGen; ++g) {
            const int zg = z0 - 2 * g;
            const bool need = g <= ng && active && zg >= zs - (ng - g) && zg <= ze + (ng - g);
            if (!need) continue;
            const uint32_t* src = ring + (g - 1) * 4 * plane_w + WP + 1 + w + (yg * kPRowsT) * WP;
            const uint32_t* pa = src + ((zg - 1) & 3) * plane_w;
            const uint32_t* pb = src + (zg & 3) * plane_w;
            const uint32_t* pc = src + ((zg + 1) & 3) * plane_w;
            uint32_t s[kPRowsT + 2];
#pragma unroll
            for (int k = 0; k < kPRowsT + 2; ++k) {
                const int o = (k - 1) * WP;
                s[k] = pa[o] + pb[o] + pc[o];
            }
            uint32_t* vd = vbuf + (g - 1) * plane_w + WP + 1 + w + (yg * kPRowsT) * WP;
#pragma unroll
            for (int k = 0; k < kPRowsT; ++k) {
                vd[k * WP] = s[k] + s[k + 1] + s[k + 2];
            }
        }
        __syncthreads();
        // levels 1 .. ng: x sums from the neighbour words' column sums, the rule
#pragma unroll
        for (int g = 1; g <= kMaxGen; ++g) {
            const int zg = z0 - 2 * g;
            const bool need = g <= ng && active && zg >= zs - (ng - g) && zg <= ze + (ng - g);
            if (!need) continue;
            const uint32_t* vn = vbuf + (g - 1) * plane_w + WP + 1 + w + (yg * kPRowsT) * WP;
            const uint32_t* cp = ring + ((g - 1) * 4 + (zg & 3)) * plane_w + WP + 1 + w + (yg * kPRowsT) * WP;
            const bool zin = zg >= lo[g][2] && zg <= hi[g][2];
#pragma unroll
            for (int k = 0; k < kPRowsT; ++k) {
                const int r = yg * kPRowsT + k, y = yb + r;
                const uint32_t v = vn[k * WP];
                const uint32_t box = v + __funnelshift_l(vn[k * WP - 1], v, 8) + __funnelshift_r(v, vn[k * WP + 1], 8);
                const uint32_t c = cp[k * WP];
                const uint32_t m = (zin && y >= lo[g][1] && y <= hi[g][1]) ? xm[g] : 0u;
                const uint32_t nxt = (life_rule(box - c, c) & m) | (c & ~m);
                if (g < ng) {
                    ring[(g * 4 + (zg & 3)) * plane_w + WP + 1 + w + r * WP] = nxt;
                } else if (wout && zg >= zs && zg <= ze && r >= ng && r < kPRows - ng && y <= fhi[1] &&
                           y >= flo[1]) {
                    outw[(long long)zg * wplane + (long long)y * wpr + wx] = nxt;
                }
            }
        }
    }
}

}  // namespace

cudaError_t launch_gol_substep(const uint8_t* in, uint8_t* out, const BlockLayout& L, int step_i,
                               cudaStream_t st)
{
    const int wb = (L.xoff + 1) >> 2;
    const int we = (L.xoff + L.n[0] - 2) >> 2;              // last word with an updatable cell
    const int nw = we - wb + 1;
    const bool seg16 = ((nw + 13) / 14) * 16 < ((nw + 29) / 30) * 32;
    const int out_words = seg16 ? 14 : 30, rows_per_warp = seg16 ? 2 * kRY : kRY;
    const int ntx = (nw + out_words - 1) / out_words;
    const int rows = L.n[1] - 2;
    const int nty = (rows + rows_per_warp * kGolWarps - 1) / (rows_per_warp * kGolWarps);
    const long long tiles = (long long)ntx * nty * L.nblk;
    // small blocks are latency bound (a generation of a 136^3 block is a few
    // microseconds of data): short z chunks, many CTAs
    const long long want = 152LL * 12;
    int nzc = (int)((want + tiles - 1) / tiles);
    const int maxc = (L.n[2] - 2) / 4 > 0 ? (L.n[2] - 2) / 4 : 1;
    if (nzc > maxc) nzc = maxc;
    if (nzc < 1) nzc = 1;
    dim3 grid(ntx, nty, L.nblk * nzc);
    if (seg16) gol_kernel<16><<<grid, 32 * kGolWarps, 0, st>>>(in, out, L, step_i, nzc);
    else gol_kernel<32><<<grid, 32 * kGolWarps, 0, st>>>(in, out, L, step_i, nzc);
    count_launches(1);
    return cudaGetLastError();
}

int gol_max_generations_per_pass() { return kMaxGen; }

cudaError_t launch_gol_period(const uint8_t* in, uint8_t* out, const BlockLayout& L, int i0, int ng,
                              cudaStream_t st)
{
    if (ng < 1 || ng > kMaxGen) return cudaErrorInvalidValue;
    // final window (last generation) over all blocks
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
    GolPeriod G{};
    G.ng = ng;
    G.i0 = i0;
    const int wfirst = (L.xoff + lo[0]) >> 2, wlast = (L.xoff + hi[0]) >> 2;
    const int nw = wlast - wfirst + 1;
    const int ntx = (nw + kPMaxW - 3) / (kPMaxW - 2);
    G.OW = (nw + ntx - 1) / ntx;
    G.WT = G.OW + 2;
    G.wx0 = wfirst;
    G.OR = kPRows - 2 * ng;
    G.y0 = lo[1] - ng;
    const int nty = (hi[1] - lo[1] + 1 + G.OR - 1) / G.OR;
    const long long tiles = (long long)ntx * nty * L.nblk;
    const int nz = hi[2] - lo[2] + 1;
    // z chunks: enough CTAs to fill the SMs, each chunk long enough that the
    // 3*ng planes of pipeline fill stay a small part of it
    int nzc = (int)std::max(1LL, (152LL * 2 + tiles - 1) / tiles);
    nzc = std::min(nzc, std::max(1, nz / (4 * ng)));
    G.nzc = nzc;
    const size_t smem = (size_t)ng * 5 * (G.WT + 2) * (kPRows + 2) * sizeof(uint32_t);
    const int threads = ((G.WT * kPGroups + 31) / 32) * 32;
    const dim3 grid(ntx, nty, L.nblk * nzc);
    // narrow regions: a variant with two resident CTAs per SM
    constexpr int kNarrowT = 36 * kPGroups;
    const bool narrow = threads <= kNarrowT;
    static SmemLimit attr[2];
    const void* kern = narrow ? (const void*)gol_period_kernel<kNarrowT, 2>
                              : (const void*)gol_period_kernel<kPMaxW * kPGroups, 1>;
    if (cudaError_t e = raise_smem_limit(attr[narrow], kern, std::max<size_t>(smem, 48 * 1024))) return e;
    if (narrow) gol_period_kernel<kNarrowT, 2><<<grid, threads, smem, st>>>(in, out, L, G);
    else gol_period_kernel<kPMaxW * kPGroups, 1><<<grid, threads, smem, st>>>(in, out, L, G);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace b2r
