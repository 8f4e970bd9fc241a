// eqwp_tile.cuh -- tile machinery shared by the elastic-wave stage kernels
// (eqwp.cu) and their adjoints (adjoint.cu): thread = 4 consecutive x cells
// (one float4) of one row, CTA = 32 x 8 threads = a 128 x 8 tile marching z
// over a chunk; x neighbours as float4 row segments through L1, z
// neighbours in 5-plane float4 register queues; the staggered and collocated
// 4th-order first differences of the 4 cells.
#pragma once
#include <algorithm>

#include "b2r_common.cuh"

namespace b2r {
namespace eqk {

// Thread = 4 consecutive x cells (one float4) of one row; CTA = 32 x 8
// threads = a 128 x 8 tile; z marched over a chunk.
constexpr int kBX = 32, kBY = 8;
#ifndef B2R_EQWP_MINB
#define B2R_EQWP_MINB 2   // resident CTAs per SM the register budget is fitted to
#endif

enum { VX, VY, VZ, SXX, SXY, SXZ, SYY, SYZ, SZZ, DISP };

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
// NC: the read-only path (fields that no thread writes during the kernel);
// otherwise a coherent load, for a persistent kernel whose other CTAs
// update the fields between its work units
template <bool NC>
__device__ __forceinline__ float4 ldf4(const float* p)
{
    if constexpr (NC) return __ldg(reinterpret_cast<const float4*>(p));
    else return *reinterpret_cast<const float4*>(p);
}
__device__ __forceinline__ float4 ldw4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float cmp(const float4& v, int j)
{
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// 12 cells x-4 .. x+7 of a row around the thread's 4 cells
struct Row12 {
    float v[12];
    template <bool NC = true>
    __device__ __forceinline__ void load(const float* p)
    {
        const float4 a = ldf4<NC>(p - 4), b = ldf4<NC>(p), c = ldf4<NC>(p + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        v[8] = c.x; v[9] = c.y; v[10] = c.z; v[11] = c.w;
    }
};
template <bool NC>
__device__ __forceinline__ Row12 row12(const float* p)
{
    Row12 r{};
    r.template load<NC>(p);
    return r;
}

// five planes z-2 .. z+2 of the thread's 4 cells
struct Q5v {
    float4 m2, m1, c, p1, p2;
    __device__ __forceinline__ void shift(float4 nv)
    {
        m2 = m1; m1 = c; c = p1; p1 = p2; p2 = nv;
    }
};

struct Win {
    int lo[3], hi[3];
    int zs, ze;
    bool ok;
};

__device__ __forceinline__ Win window(const BlockLayout& L, int blk, int zc, int nzc, int shrink)
{
    Win w;
    const int edge = edge_bits(L, blk);
#pragma unroll
    for (int a = 0; a < 3; ++a) stage_region(L, edge, a, shrink, w.lo[a], w.hi[a]);
    const int nz_out = w.hi[2] - w.lo[2] + 1;
    const int per = (nz_out + nzc - 1) / nzc;
    w.zs = w.lo[2] + zc * per;
    w.ze = min(w.hi[2], w.zs + per - 1);
    w.ok = nz_out > 0 && w.zs <= w.ze;
    return w;
}

// Common prologue: this thread's cells, their x mask, the row base pointer offset.
struct Cell {
    int blk, y, xb;             // block, row, block x of the first of the 4 cells
    bool vx[4], any, all;
    long long base;             // element offset of (xb, y, 0) in the field buffers
};

// The thread's place in a stage launch: tile (bx, by), thread (tx, ty) of a
// CTA of dx x dy threads -- the launch's own indices, or those a persistent
// kernel assigns to a work unit.
struct TilePos {
    int bx, by, tx, ty, dx, dy;
};
__device__ __forceinline__ TilePos launch_pos()
{
    return TilePos{(int)blockIdx.x, (int)blockIdx.y, (int)threadIdx.x, (int)threadIdx.y, (int)blockDim.x,
                   (int)blockDim.y};
}

__device__ __forceinline__ bool cell_setup(const BlockLayout& L, const Win& w, int blk, Cell& c, int x0, int y0,
                                           const TilePos& q)
{
    const int xs0 = x0 + q.bx * (4 * q.dx) + 4 * q.tx;
    c.blk = blk;
    c.xb = xs0 - L.xoff;
    c.y = y0 + q.by * q.dy + q.ty;
    if (!w.ok || c.y < w.lo[1] || c.y > w.hi[1]) return false;
    c.any = false;
    c.all = true;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        c.vx[j] = c.xb + j >= w.lo[0] && c.xb + j <= w.hi[0];
        c.any |= c.vx[j];
        c.all &= c.vx[j];
    }
    c.base = (long long)blk * L.bstride + (long long)c.y * L.P + xs0;
    return c.any;
}
__device__ __forceinline__ bool cell_setup(const BlockLayout& L, const Win& w, int blk, Cell& c, int x0, int y0)
{
    return cell_setup(L, w, blk, c, x0, y0, launch_pos());
}

// Read-modify-write of the thread's 4 cells, split so that every load of an
// iteration is issued before any store (the field pointers may alias as far
// as the compiler knows, so a fused load-add-store per field would serialise
// one DRAM round trip per field).
__device__ __forceinline__ float4 rd4(const float* f, const Cell& c)
{
    if (c.all) return ldw4(f);
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (c.vx[0]) o.x = f[0];
    if (c.vx[1]) o.y = f[1];
    if (c.vx[2]) o.z = f[2];
    if (c.vx[3]) o.w = f[3];
    return o;
}
// The add is an explicit round-to-nearest add, so that no kernel variant
// contracts it with the product that formed d: every variant storing the
// same update stores the same bits.  Returns the stored values.
__device__ __forceinline__ float4 wr4(float* f, const Cell& c, float4 o, const float (&d)[4])
{
    o.x = __fadd_rn(o.x, d[0]);
    o.y = __fadd_rn(o.y, d[1]);
    o.z = __fadd_rn(o.z, d[2]);
    o.w = __fadd_rn(o.w, d[3]);
    if (c.all) {
        *reinterpret_cast<float4*>(f) = o;
    } else {
        if (c.vx[0]) f[0] = o.x;
        if (c.vx[1]) f[1] = o.y;
        if (c.vx[2]) f[2] = o.z;
        if (c.vx[3]) f[3] = o.w;
    }
    return o;
}

// d/dx of the 4 cells from a 12-cell row, d/dy from rows +-1, +-2, d/dz from a queue
__device__ __forceinline__ float dcx(const Row12& r, int j, float a, float b)
{
    return a * (r.v[6 + j] - r.v[2 + j]) + b * (r.v[5 + j] - r.v[3 + j]);
}
__device__ __forceinline__ float dc4(const float4& m2, const float4& m1, const float4& p1,
                                     const float4& p2, int j, float a, float b)
{
    return a * (cmp(p2, j) - cmp(m2, j)) + b * (cmp(p1, j) - cmp(m1, j));
}

// Staggered 4th-order differences, forward Dp at i+1/2 and backward Dm at
// i-1/2: c1 (f1 - f0) + c2 (f2 - f-1), c1 = 9/8, c2 = -1/24.  Every
// operation of the staggered scheme is an explicitly rounded intrinsic, in
// the order of the FP32 oracle, so no kernel variant contracts differently
// and all of them (two stage kernels, the fused step, the replay) give the
// same bits.
constexpr float kC1 = 9.f / 8.f, kC2 = -1.f / 24.f;
__device__ __forceinline__ float sdiff(float a1, float a0, float b1, float b0)
{
    return __fadd_rn(__fmul_rn(kC1, __fsub_rn(a1, a0)), __fmul_rn(kC2, __fsub_rn(b1, b0)));
}
__device__ __forceinline__ float dpx(const Row12& r, int j)
{
    return sdiff(r.v[5 + j], r.v[4 + j], r.v[6 + j], r.v[3 + j]);
}
__device__ __forceinline__ float dmx(const Row12& r, int j)
{
    return sdiff(r.v[4 + j], r.v[3 + j], r.v[5 + j], r.v[2 + j]);
}
// rows/planes -2..+2 around the cell: Dp uses -1..+2, Dm uses -2..+1
__device__ __forceinline__ float dp4(const float4& m1, const float4& c, const float4& p1,
                                     const float4& p2, int j)
{
    return sdiff(cmp(p1, j), cmp(c, j), cmp(p2, j), cmp(m1, j));
}
__device__ __forceinline__ float dm4(const float4& m2, const float4& m1, const float4& c,
                                     const float4& p1, int j)
{
    return sdiff(cmp(c, j), cmp(m1, j), cmp(p1, j), cmp(m2, j));
}
__device__ __forceinline__ float add3(float a, float b, float c) { return __fadd_rn(__fadd_rn(a, b), c); }

// Velocity and stress updates of the staggered scheme from the raw stencil
// sums (a = D s, e = E v), dt, 1/h and the material, as the oracle rounds
// them:  v + (dt b)(a / h);  s_ii + dt (l2m e_ii + lambda (e_jj + e_kk));
// s_ij + (dt mu)(e_ij / h).
__device__ __forceinline__ float vel_update(float v, float a, float dt, float ih, float b)
{
    return __fadd_rn(v, __fmul_rn(__fmul_rn(dt, b), __fmul_rn(a, ih)));
}
struct StressIn {
    float exx, eyy, ezz, gxy, gxz, gyz;   // raw stencil sums (not yet / h)
};
__device__ __forceinline__ void stress_update(const StressIn& e, float dt, float ih, float lam, float mu,
                                              float (&s)[6])   // xx, yy, zz, xy, xz, yz; in / out
{
    const float exx = __fmul_rn(e.exx, ih), eyy = __fmul_rn(e.eyy, ih), ezz = __fmul_rn(e.ezz, ih);
    const float l2m = __fadd_rn(lam, __fmul_rn(2.f, mu));
    s[0] = __fadd_rn(s[0], __fmul_rn(dt, __fadd_rn(__fmul_rn(l2m, exx), __fmul_rn(lam, __fadd_rn(eyy, ezz)))));
    s[1] = __fadd_rn(s[1], __fmul_rn(dt, __fadd_rn(__fmul_rn(l2m, eyy), __fmul_rn(lam, __fadd_rn(exx, ezz)))));
    s[2] = __fadd_rn(s[2], __fmul_rn(dt, __fadd_rn(__fmul_rn(l2m, ezz), __fmul_rn(lam, __fadd_rn(exx, eyy)))));
    const float dm = __fmul_rn(dt, mu);
    s[3] = __fadd_rn(s[3], __fmul_rn(dm, __fmul_rn(e.gxy, ih)));
    s[4] = __fadd_rn(s[4], __fmul_rn(dm, __fmul_rn(e.gxz, ih)));
    s[5] = __fadd_rn(s[5], __fmul_rn(dm, __fmul_rn(e.gyz, ih)));
}

// Velocity-stage operator of the staggered scheme on six stress-like fields
// (xx, xy, xz, yy, yz, zz, each already offset to the thread's row):
//   ax = Dp_x xx + Dm_y xy + Dm_z xz
//   ay = Dm_x xy + Dp_y yy + Dm_z yz
//   az = Dm_x xz + Dm_y yz + Dp_z zz
// z neighbours come from register queues advanced one plane per eval().
template <bool NC>
struct VelOpT {
    const float *xx, *xy, *xz, *yy, *yz, *zz;
    Q5v qxz, qyz, qzz;
    __device__ __forceinline__ void begin(int zs, long long S)
    {
        const long long o = (long long)(zs - 2) * S;
        qxz.m1 = ldf4<NC>(xz + o); qyz.m1 = ldf4<NC>(yz + o); qzz.m1 = ldf4<NC>(zz + o);
        qxz.c = ldf4<NC>(xz + o + S); qyz.c = ldf4<NC>(yz + o + S); qzz.c = ldf4<NC>(zz + o + S);
        qxz.p1 = ldf4<NC>(xz + o + 2 * S); qyz.p1 = ldf4<NC>(yz + o + 2 * S); qzz.p1 = ldf4<NC>(zz + o + 2 * S);
        qxz.p2 = ldf4<NC>(xz + o + 3 * S); qyz.p2 = ldf4<NC>(yz + o + 3 * S); qzz.p2 = ldf4<NC>(zz + o + 3 * S);
    }
    // o: element offset of plane z; planes must be visited in increasing z
    __device__ __forceinline__ void eval(long long o, long long P, long long S, float (&ax)[4],
                                         float (&ay)[4], float (&az)[4])
    {
        qxz.shift(ldf4<NC>(xz + o + 2 * S));
        qyz.shift(ldf4<NC>(yz + o + 2 * S));
        qzz.shift(ldf4<NC>(zz + o + 2 * S));
        const Row12 rxx = row12<NC>(xx + o), rxy = row12<NC>(xy + o), rxz = row12<NC>(xz + o);
        const float4 xym2 = ldf4<NC>(xy + o - 2 * P), xym1 = ldf4<NC>(xy + o - P), xyp1 = ldf4<NC>(xy + o + P);
        const float4 yym1 = ldf4<NC>(yy + o - P), yyc = ldf4<NC>(yy + o), yyp1 = ldf4<NC>(yy + o + P), yyp2 = ldf4<NC>(yy + o + 2 * P);
        const float4 yzm2 = ldf4<NC>(yz + o - 2 * P), yzm1 = ldf4<NC>(yz + o - P), yzp1 = ldf4<NC>(yz + o + P);
        const float4 xyc = make_float4(rxy.v[4], rxy.v[5], rxy.v[6], rxy.v[7]);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            ax[j] = add3(dpx(rxx, j), dm4(xym2, xym1, xyc, xyp1, j), dm4(qxz.m2, qxz.m1, qxz.c, qxz.p1, j));
            ay[j] = add3(dmx(rxy, j), dp4(yym1, yyc, yyp1, yyp2, j), dm4(qyz.m2, qyz.m1, qyz.c, qyz.p1, j));
            az[j] = add3(dmx(rxz, j), dm4(yzm2, yzm1, qyz.c, yzp1, j), dp4(qzz.m1, qzz.c, qzz.p1, qzz.p2, j));
        }
    }
};

// Stress-stage (strain) operator of the staggered scheme on three
// velocity-like fields x, y, z:
//   e[0] = Dm_x x, e[1] = Dm_y y, e[2] = Dm_z z,
//   e[3] = Dp_y x + Dp_x y, e[4] = Dp_z x + Dp_x z, e[5] = Dp_z y + Dp_y z
template <bool NC>
struct StrOpT {
    const float *x, *y, *z;
    Q5v qx, qy, qz;
    __device__ __forceinline__ void begin(int zs, long long S)
    {
        const long long o = (long long)(zs - 2) * S;
        qx.m1 = ldf4<NC>(x + o); qy.m1 = ldf4<NC>(y + o); qz.m1 = ldf4<NC>(z + o);
        qx.c = ldf4<NC>(x + o + S); qy.c = ldf4<NC>(y + o + S); qz.c = ldf4<NC>(z + o + S);
        qx.p1 = ldf4<NC>(x + o + 2 * S); qy.p1 = ldf4<NC>(y + o + 2 * S); qz.p1 = ldf4<NC>(z + o + 2 * S);
        qx.p2 = ldf4<NC>(x + o + 3 * S); qy.p2 = ldf4<NC>(y + o + 3 * S); qz.p2 = ldf4<NC>(z + o + 3 * S);
    }
    __device__ __forceinline__ void eval(long long o, long long P, long long S, float (&e)[6][4])
    {
        qx.shift(ldf4<NC>(x + o + 2 * S));
        qy.shift(ldf4<NC>(y + o + 2 * S));
        qz.shift(ldf4<NC>(z + o + 2 * S));
        const Row12 rx = row12<NC>(x + o), ry = row12<NC>(y + o), rz = row12<NC>(z + o);
        const float4 xc = make_float4(rx.v[4], rx.v[5], rx.v[6], rx.v[7]);
        const float4 yc = make_float4(ry.v[4], ry.v[5], ry.v[6], ry.v[7]);
        const float4 zc = make_float4(rz.v[4], rz.v[5], rz.v[6], rz.v[7]);
        const float4 xm1 = ldf4<NC>(x + o - P), xp1 = ldf4<NC>(x + o + P), xp2 = ldf4<NC>(x + o + 2 * P);
        const float4 ym2 = ldf4<NC>(y + o - 2 * P), ym1 = ldf4<NC>(y + o - P), yp1 = ldf4<NC>(y + o + P);
        const float4 zm1 = ldf4<NC>(z + o - P), zp1 = ldf4<NC>(z + o + P), zp2 = ldf4<NC>(z + o + 2 * P);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            e[0][j] = dmx(rx, j);
            e[1][j] = dm4(ym2, ym1, yc, yp1, j);
            e[2][j] = dm4(qz.m2, qz.m1, qz.c, qz.p1, j);
            e[3][j] = __fadd_rn(dp4(xm1, xc, xp1, xp2, j), dpx(ry, j));
            e[4][j] = __fadd_rn(dp4(qx.m1, qx.c, qx.p1, qx.p2, j), dpx(rz, j));
            e[5][j] = __fadd_rn(dp4(qy.m1, qy.c, qy.p1, qy.p2, j), dp4(zm1, zc, zp1, zp2, j));
        }
    }
};
using VelOp = VelOpT<true>;
using StrOp = StrOpT<true>;

// L2 prefetch of the thread's 16 bytes of a plane a few iterations ahead:
// the z-marching stages are latency bound (each iteration waits on its own
// first-touch DRAM loads), and a prefetch costs no register.
#ifndef B2R_EQWP_PREFETCH
#define B2R_EQWP_PREFETCH 1
#endif
__device__ __forceinline__ void pf_l2(const float* p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
// element offset of plane z + d, clamped to the last plane the CTA itself
// reads (zlast): a prefetch past its own z chunk would fetch planes that
// another CTA reads much later, and be evicted first
__device__ __forceinline__ long long ahead(const BlockLayout& L, int z, int d, int zlast)
{
    return (long long)min(z + d, zlast) * L.plane;
}

// masked store of 4 values (the lanes of the window)
__device__ __forceinline__ void st4(float* f, const Cell& c, const float (&v)[4])
{
    if (c.all) {
        *reinterpret_cast<float4*>(f) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (c.vx[j]) f[j] = v[j];
    }
}

// Tile origin of a stage launch: the first tile starts at the lowest window
// cell of any block (x rounded down to a float4 boundary), so that no tile
// column or row lies wholly outside every window.
struct Tiles {
    int nzc;    // z chunks per block
    int x0;     // storage x of the first tile column (multiple of 4)
    int y0;     // first row
};

// A launch: grid, CTA shape (kBX * kBY threads: 32 x 8, 16 x 16 or 8 x 32,
// tiles of 128, 64 or 32 cells by 8, 16 or 32 rows) and tile origin.
struct Grid {
    dim3 g, b;
    Tiles t;
};

#ifndef B2R_EQWP_CTAS
#define B2R_EQWP_CTAS 24    // CTAs per SM a stage launch aims at (z chunks of the tiles)
#endif
#ifndef B2R_EQWP_ZMIN
#define B2R_EQWP_ZMIN 16    // planes per z chunk at least
#endif
#ifndef B2R_EQWP_YHALO
#define B2R_EQWP_YHALO 0    // cost of a re-read halo row against a computed row, percent (0 measured best)
#endif

inline Grid stage_grid(const BlockLayout& L, int shrink)
{
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-1, -1, -1};
    for (int b = 0; b < L.nblk; ++b) {
        const int e = edge_bits(L, b);
        for (int a = 0; a < 3; ++a) {
            int l, h;
            stage_region(L, e, a, shrink, l, h);
            lo[a] = std::min(lo[a], l);
            hi[a] = std::max(hi[a], h);
        }
    }
    Grid r;
    r.t.x0 = (L.xoff + lo[0]) & ~3;
    r.t.y0 = lo[1];
    // tile shape: tbx threads of 4 cells per row (8..32) by tby = 256 / tbx
    // rows, the one that computes the fewest cells over the window, a tile
    // paying for its y halo (two rows above and below are re-read) in
    // proportion; CTAs need not be a multiple of 32 threads wide
    const int W = std::max(1, L.xoff + hi[0] + 1 - r.t.x0);
    const int Hy = std::max(1, hi[1] + 1 - lo[1]);
    const int G4 = (W + 3) / 4;
    int bx = kBX, by = kBY;
    double best = 1e300;
    for (int c = 8; c <= kBX; ++c) {
        const int rws = kBX * kBY / c;
        const double cells = (double)((G4 + c - 1) / c) * c * 4 * ((Hy + rws - 1) / rws) * rws;
        const double cost = cells * (1.0 + (B2R_EQWP_YHALO / 100.0) * 4.0 / rws);
        if (cost < best - 1e-9) {
            best = cost;
            bx = c;
            by = rws;
        }
    }
    r.b = dim3(bx, by);
    const int tx = std::max(1, (G4 + bx - 1) / bx);
    const int ty = std::max(1, (Hy + by - 1) / by);
    const long long tiles = (long long)tx * ty * L.nblk;
    const long long want = 152LL * B2R_EQWP_CTAS;
    int nzc = (int)((want + tiles - 1) / tiles);
    int maxc = (hi[2] - lo[2] + 1) / B2R_EQWP_ZMIN;
    if (maxc < 1) maxc = 1;
    if (nzc > maxc) nzc = maxc;
    if (nzc < 1) nzc = 1;
    r.t.nzc = nzc;
    r.g = dim3(tx, ty, L.nblk * nzc);
    return r;
}

}  // namespace eqk
}  // namespace b2r
