// eqwp_tma.cu -- the staggered elastic wave's stress stage with every input
// streamed through TMA rings (the two-pass step's second pass).
//
// The plain-load stage (eqwp_stag.cuh) waits on its own first-touch loads
// each plane.  Here one thread of the CTA issues the tile's boxes a few
// planes ahead into shared memory, so the loads are in flight while the
// threads compute:
//   ring V: the three velocities of a plane (the tile, 4 more cells on each
//     side in x, 2 more rows on each side in y), 5 planes: the
//     plane being updated (x and y neighbours), the plane two ahead (its
//     columns feed the 5-plane z queues) and the planes between and ahead;
//   ring O: the six stresses and lambda, mu of the plane (the tile itself),
//     3 planes.
// CTA = 256 threads: tx x ty of them (tx = 8 .. 32, ty = 256 / tx, the tile
// shape the plain stage launch picks for the window, so that no tile column
// is mostly outside it), thread = 4 consecutive x cells (float4) of one row,
// tile = 4 tx x ty cells over a z chunk of one block; the velocity boxes are
// (4 tx + 8) x (ty + 4) cells, the own boxes 4 tx x ty.  The arithmetic is
// stag_stress_unit's, operation for operation (the same stencil helpers on
// the same values), so the result is bit-identical to it.
#include "b2r_common.cuh"
#include "eqwp.h"
#include "eqwp_tile.cuh"

namespace b2r {

namespace {

using namespace eqk;

constexpr int kThr = 256;
constexpr int kVF = 1632;                        // floats per velocity box slot: the largest box (136 x 12)
constexpr int kOF = 1024;                        // floats per own box slot: 4 * 256 cells
constexpr int kSV = 5, kSO = 3;                  // ring slots
constexpr size_t kSmemT = size_t(kSV) * 3 * kVF * 4 + size_t(kSO) * 8 * kOF * 4 + (kSV + kSO) * 8 + 16 + 128;

// tile geometry of a launch
struct TGeo {
    int tx, ty;             // threads per row, rows
    int vw, vh;             // velocity box (4 tx + 8) x (ty + 4)
    int ow, oh;             // own box 4 tx x ty
};

struct TmaArgs {
    float* out[6];          // stresses of the updated plane: xx, yy, zz, xy, xz, yz (stress_update order)
    float dt, ih, src_amp;
    int src[3];
    int* status;
};

__device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }

__global__ void __launch_bounds__(kThr, 1)
eqwp_stress_tma_kernel(const __grid_constant__ EqwpStressMaps maps, const TmaArgs A, const BlockLayout L,
                       const int step_i, const Tiles T, const TGeo G)
{
    const int kVW = G.vw, kOW = G.ow, kOH = G.oh;
    const uint32_t kVBytes = 3u * G.vw * G.vh * 4u, kOBytes = 8u * G.ow * G.oh * 4u;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* rv = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    float* ro = rv + kSV * 3 * kVF;
    uint64_t* barv = reinterpret_cast<uint64_t*>(ro + kSO * 8 * kOF);
    uint64_t* baro = barv + kSV;
    int* abort_flag = reinterpret_cast<int*>(baro + kSO);

    const int nzc = T.nzc;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 4);
    // the tile (uniform per CTA): storage x of its first cell, block row of its first row
    const int X0 = T.x0 + blockIdx.x * kOW, Y0 = T.y0 + blockIdx.y * kOH;
    if (!w.ok || X0 - L.xoff > w.hi[0] || X0 - L.xoff + kOW - 1 < w.lo[0] || Y0 > w.hi[1] || Y0 + kOH - 1 < w.lo[1])
        return;
    const int tid = threadIdx.x, tx = tid % G.tx, ty0 = tid / G.tx;
    const bool inrow = ty0 < G.ty;         // the threads beyond tx * ty rows only join the barriers
    const int ty = inrow ? ty0 : G.ty - 1;
    Cell c;
    const bool act = inrow && cell_setup(L, w, blk, c, T.x0, T.y0, TilePos{(int)blockIdx.x, (int)blockIdx.y, tx, ty, G.tx, G.ty});
    const int zs = w.zs, ze = w.ze;
    const int nv = ze - zs + 5;            // velocity planes zs-2 .. ze+2
    const int no = ze - zs + 1;            // own planes zs .. ze
    if (tid == 0) {
        *abort_flag = 0;
        for (int s = 0; s < kSV; ++s) mbar_init(&barv[s], 1);
        for (int s = 0; s < kSO; ++s) mbar_init(&baro[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue_v = [&](int t) {            // velocity plane zs-2+t into slot t % kSV
        uint64_t* b = &barv[t % kSV];
        mbar_expect_tx(b, kVBytes);
        float* d = rv + (t % kSV) * 3 * kVF;
        for (int f = 0; f < 3; ++f) tma_load_4d(d + f * kVF, &maps.v[f], X0 - 4, Y0 - 2, zs - 2 + t, blk, b);
    };
    auto issue_o = [&](int t) {            // own plane zs+t into slot t % kSO
        uint64_t* b = &baro[t % kSO];
        mbar_expect_tx(b, kOBytes);
        float* d = ro + (t % kSO) * 8 * kOF;
        for (int f = 0; f < 8; ++f) tma_load_4d(d + f * kOF, &maps.o[f], X0, Y0, zs + t, blk, b);
    };
    int issued_v = 0, issued_o = 0;
    if (tid == 0) {
        for (; issued_v < kSV && issued_v < nv; ++issued_v) issue_v(issued_v);
        for (; issued_o < kSO && issued_o < no; ++issued_o) issue_o(issued_o);
    }
    bool ok = true;
    // planes below waited_v / waited_o have landed (consumed in order)
    int waited_v = 0, waited_o = 0;
    auto wait_v = [&](int t) {
        if (ok && !mbar_wait_bounded(&barv[t % kSV], (t / kSV) & 1)) ok = false;
        if (ok) waited_v = t + 1;
    };
    auto wait_o = [&](int t) {
        if (ok && !mbar_wait_bounded(&baro[t % kSO], (t / kSO) & 1)) ok = false;
        if (ok) waited_o = t + 1;
    };
    auto vbox = [&](int t, int f) { return rv + (t % kSV) * 3 * kVF + f * kVF; };
    const int col = 4 + 4 * tx;            // box column of the thread's first cell
    // z queues: planes zs-2 .. zs+1 (slots 0..3)
    Q5v qx, qy, qz;
    for (int t = 0; t < 4 && t < nv; ++t) wait_v(t);
    {
        const int o = (ty + 2) * kVW + col;
        qx.m1 = lds4(vbox(0, 0) + o); qy.m1 = lds4(vbox(0, 1) + o); qz.m1 = lds4(vbox(0, 2) + o);
        qx.c = lds4(vbox(1, 0) + o); qy.c = lds4(vbox(1, 1) + o); qz.c = lds4(vbox(1, 2) + o);
        qx.p1 = lds4(vbox(2, 0) + o); qy.p1 = lds4(vbox(2, 1) + o); qz.p1 = lds4(vbox(2, 2) + o);
        qx.p2 = lds4(vbox(3, 0) + o); qy.p2 = lds4(vbox(3, 1) + o); qz.p2 = lds4(vbox(3, 2) + o);
    }
    // source cell of this block, in block coordinates
    const int b0 = blk % L.nb[0], b1 = (blk / L.nb[0]) % L.nb[1], b2 = blk / (L.nb[0] * L.nb[1]);
    const int sx = A.src[0] - b0 * L.B[0] + L.H, sy = A.src[1] - b1 * L.B[1] + L.H,
              sz = A.src[2] - b2 * L.B[2] + L.H;
    const bool srow = act && (c.y == sy) && sx >= c.xb && sx < c.xb + 4;
    const long long S = L.plane;
    bool aborted = false;
    for (int z = zs; z <= ze; ++z) {
        const int tv = z - zs + 2, to = z - zs;
        wait_v(tv + 2);
        wait_o(to);
        const int oc = (ty + 2) * kVW + col;
        qx.shift(lds4(vbox(tv + 2, 0) + oc));
        qy.shift(lds4(vbox(tv + 2, 1) + oc));
        qz.shift(lds4(vbox(tv + 2, 2) + oc));
        // x and y neighbours of plane z (box rows ty .. ty+4 are the rows y-2 .. y+2)
        const float* bx = vbox(tv, 0);
        const float* by = vbox(tv, 1);
        const float* bz = vbox(tv, 2);
        Row12 rx, ry, rz;
        {
            const int r = (ty + 2) * kVW + col;
            float4 a = lds4(bx + r - 4), b = lds4(bx + r), d = lds4(bx + r + 4);
            rx.v[0] = a.x; rx.v[1] = a.y; rx.v[2] = a.z; rx.v[3] = a.w;
            rx.v[4] = b.x; rx.v[5] = b.y; rx.v[6] = b.z; rx.v[7] = b.w;
            rx.v[8] = d.x; rx.v[9] = d.y; rx.v[10] = d.z; rx.v[11] = d.w;
            a = lds4(by + r - 4); b = lds4(by + r); d = lds4(by + r + 4);
            ry.v[0] = a.x; ry.v[1] = a.y; ry.v[2] = a.z; ry.v[3] = a.w;
            ry.v[4] = b.x; ry.v[5] = b.y; ry.v[6] = b.z; ry.v[7] = b.w;
            ry.v[8] = d.x; ry.v[9] = d.y; ry.v[10] = d.z; ry.v[11] = d.w;
            a = lds4(bz + r - 4); b = lds4(bz + r); d = lds4(bz + r + 4);
            rz.v[0] = a.x; rz.v[1] = a.y; rz.v[2] = a.z; rz.v[3] = a.w;
            rz.v[4] = b.x; rz.v[5] = b.y; rz.v[6] = b.z; rz.v[7] = b.w;
            rz.v[8] = d.x; rz.v[9] = d.y; rz.v[10] = d.z; rz.v[11] = d.w;
        }
        const float4 xc = make_float4(rx.v[4], rx.v[5], rx.v[6], rx.v[7]);
        const float4 yc = make_float4(ry.v[4], ry.v[5], ry.v[6], ry.v[7]);
        const float4 zcv = make_float4(rz.v[4], rz.v[5], rz.v[6], rz.v[7]);
        const float4 xm1 = lds4(bx + (ty + 1) * kVW + col), xp1 = lds4(bx + (ty + 3) * kVW + col),
                     xp2 = lds4(bx + (ty + 4) * kVW + col);
        const float4 ym2 = lds4(by + ty * kVW + col), ym1 = lds4(by + (ty + 1) * kVW + col),
                     yp1 = lds4(by + (ty + 3) * kVW + col);
        const float4 zm1 = lds4(bz + (ty + 1) * kVW + col), zp1 = lds4(bz + (ty + 3) * kVW + col),
                     zp2 = lds4(bz + (ty + 4) * kVW + col);
        float e[6][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            e[0][j] = dmx(rx, j);
            e[1][j] = dm4(ym2, ym1, yc, yp1, j);
            e[2][j] = dm4(qz.m2, qz.m1, qz.c, qz.p1, j);
            e[3][j] = __fadd_rn(dp4(xm1, xc, xp1, xp2, j), dpx(ry, j));
            e[4][j] = __fadd_rn(dp4(qx.m1, qx.c, qx.p1, qx.p2, j), dpx(rz, j));
            e[5][j] = __fadd_rn(dp4(qy.m1, qy.c, qy.p1, qy.p2, j), dp4(zm1, zcv, zp1, zp2, j));
        }
        // own cells: stresses in stress_update order (xx, yy, zz, xy, xz, yz), lambda, mu
        const float* ob = ro + (to % kSO) * 8 * kOF + ty * kOW + 4 * tx;
        float4 old[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) old[f] = lds4(ob + f * kOF);
        const float4 l4 = lds4(ob + 6 * kOF), m4 = lds4(ob + 7 * kOF);
        if (act) {
            const bool src_here = srow && z == sz;
            float ns[6][4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const StressIn in{e[0][j], e[1][j], e[2][j], e[3][j], e[4][j], e[5][j]};
                float sv[6];
#pragma unroll
                for (int f = 0; f < 6; ++f) sv[f] = cmp(old[f], j);
                stress_update(in, A.dt, A.ih, cmp(l4, j), cmp(m4, j), sv);
                if (src_here && c.xb + j == sx) {
                    sv[0] = __fadd_rn(sv[0], A.src_amp);
                    sv[1] = __fadd_rn(sv[1], A.src_amp);
                    sv[2] = __fadd_rn(sv[2], A.src_amp);
                }
#pragma unroll
                for (int f = 0; f < 6; ++f) ns[f][j] = sv[f];
            }
            const long long o = (long long)z * S;
#pragma unroll
            for (int f = 0; f < 6; ++f) st4(A.out[f] + c.base + o, c, ns[f]);
        }
        if (!ok) *abort_flag = 1;
        __syncthreads();                  // every thread is done with the planes up to tv and to
        if (*abort_flag) {
            aborted = true;
            break;
        }
        // refill the slots of planes <= tv and <= to (all used): velocity
        // planes up to tv + kSV, own planes up to to + kSO
        if (tid == 0) {
            while (issued_v < nv && issued_v <= tv + kSV) issue_v(issued_v++);
            while (issued_o < no && issued_o <= to + kSO) issue_o(issued_o++);
        }
    }
    if (aborted && tid == 0) {
        // no TMA may still write this CTA's shared memory when it exits:
        // wait (bounded) for the loads issued and not waited for
        report(A.status, DEV_TIMEOUT);
        for (int t = waited_v; t < issued_v; ++t) mbar_wait_bounded(&barv[t % kSV], (t / kSV) & 1, 100000000ull);
        for (int t = waited_o; t < issued_o; ++t) mbar_wait_bounded(&baro[t % kSO], (t / kSO) & 1, 100000000ull);
    }
    // otherwise every issued load was waited for: the last iteration waited
    // for velocity plane ze + 2 and own plane ze, the last ones issued
}

}  // namespace

void eqwp_stress_tma_shape(const BlockLayout& L, int step_i, int* tx, int* ty)
{
    const Grid g = stage_grid(L, 4 * step_i + 4);
    *tx = (int)g.b.x;
    *ty = (int)g.b.y;
}

cudaError_t launch_eqwp_stress_tma(const EqwpStressMaps& maps, int tpr, float* const* fld, const BlockLayout& L,
                                   int step_i, float src_amp, const EqwpStagParams& p, int* status,
                                   cudaStream_t st)
{
    static KernelSetup setup;
    if (cudaError_t e = kernel_setup(setup, eqwp_stress_tma_kernel, kThr, kSmemT, nullptr, nullptr)) return e;
    // the plain stage launch's tiles over the union of the blocks' windows
    const int shrink = 4 * step_i + 4;
    const Grid g = stage_grid(L, shrink);
    if ((int)g.b.x != tpr) return cudaErrorInvalidValue;   // maps built for another tile shape
    TGeo G;
    G.tx = (int)g.b.x;
    G.ty = (int)g.b.y;
    G.vw = 4 * G.tx + 8;
    G.vh = G.ty + 4;
    G.ow = 4 * G.tx;
    G.oh = G.ty;
    if (G.vw * G.vh > kVF || G.ow * G.oh > kOF || G.tx * G.ty > kThr) return cudaErrorInvalidValue;
    Tiles T = g.t;
    const long long tiles = (long long)g.g.x * g.g.y * L.nblk;
    int lo2, hi2;
    stage_region(L, edge_bits(L, 0), 2, shrink, lo2, hi2);
    int nzmax = hi2 - lo2 + 1;
    for (int b = 1; b < L.nblk; ++b) {
        stage_region(L, edge_bits(L, b), 2, shrink, lo2, hi2);
        nzmax = std::max(nzmax, hi2 - lo2 + 1);
    }
    const int nz = std::max(1, nzmax);
    // z chunks: the fewest waves of one CTA per SM, each weighted by its
    // chunk length plus the four planes of queue warm-up
    int sms = 152;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        sms = std::max(1, sms);
    }
    int nzc = 1;
    double best_cost = 1e300;
    for (int k = 1; k <= std::max(1, nz / 8); ++k) {
        const double waves = (double)((tiles * k + sms - 1) / sms);
        const double cost = waves * ((nz + k - 1) / k + 4);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            nzc = k;
        }
    }
    T.nzc = nzc;
    TmaArgs A{};
    // stress_update order: xx, yy, zz, xy, xz, yz
    A.out[0] = fld[SXX];
    A.out[1] = fld[SYY];
    A.out[2] = fld[SZZ];
    A.out[3] = fld[SXY];
    A.out[4] = fld[SXZ];
    A.out[5] = fld[SYZ];
    A.dt = p.dt;
    A.ih = p.inv_h;
    A.src_amp = src_amp;
    for (int a = 0; a < 3; ++a) A.src[a] = p.src[a];
    A.status = status;
    const dim3 grid(g.g.x, g.g.y, L.nblk * nzc);
    eqwp_stress_tma_kernel<<<grid, kThr, kSmemT, st>>>(maps, A, L, step_i, T, G);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace b2r
