// eqwp.cu -- velocity-stress elastic wave propagation on the resident blocks.
//
// Two physics modes, each a pair of 2.5-D z-marching stage kernels:
//
// REF   the reference model (eqwp.cu of the reference): collocated central
//       FD4 first derivatives (coefficients -1/12, 2/3 at +-2, +-1,
//       eqwp.cu:22-23,131-133), homogeneous constants (lame1 = 32 acting as
//       lambda, lame2 = 174.87 as mu, 1/rho = 1/1800, dt = 0.5, dx = 10,
//       eqwp.cu:9-20), stress stage first then vx, vy (+ displacement), vz
//       (eqwp.cu:679-684), body force on the y = Ngy-7-D*R plane patch while
//       ts < 50 (eqwp.cu:135,229-231,561-566).
// STAG  a new staggered-grid (Virieux) 4th-order scheme with per-cell
//       lambda, mu and buoyancy and an explosive point source: velocity stage
//       first, then stress stage.  No reference counterpart.
//
// Each stage reads the neighbours of the other field group (xy from L1/L2,
// z from a 5-plane register queue per field) and updates its own fields in
// place; a stage's inputs are never written by it, so in-place is race free.
// Both stages have radius 2, so one time step consumes 4 halo cells: stage A
// of sub-step i updates the window with shrink 4i+2, stage B shrink 4i+4.
#include "b2r_common.cuh"
#include "eqwp.h"

namespace b2r {

namespace {

// Thread = 4 consecutive x cells (one float4) of one row; CTA = 32 x 8
// threads = a 128 x 8 tile; z marched over a chunk.
constexpr int kBX = 32, kBY = 8, kTXc = 4 * kBX;
#ifndef B2R_EQWP_MINB
#define B2R_EQWP_MINB 2   // resident CTAs per SM the register budget is fitted to
#endif

enum { VX, VY, VZ, SXX, SXY, SXZ, SYY, SYZ, SZZ, DISP };

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float4 ldw4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float cmp(const float4& v, int j)
{
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// 12 cells x-4 .. x+7 of a row around the thread's 4 cells
struct Row12 {
    float v[12];
    __device__ __forceinline__ void load(const float* p)
    {
        const float4 a = ld4(p - 4), b = ld4(p), c = ld4(p + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        v[8] = c.x; v[9] = c.y; v[10] = c.z; v[11] = c.w;
    }
};

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

__device__ __forceinline__ bool cell_setup(const BlockLayout& L, const Win& w, int blk, Cell& c)
{
    const int xs0 = ((L.xoff + 2) & ~3) + blockIdx.x * kTXc + 4 * threadIdx.x;
    c.blk = blk;
    c.xb = xs0 - L.xoff;
    c.y = 2 + blockIdx.y * kBY + threadIdx.y;
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
__device__ __forceinline__ void wr4(float* f, const Cell& c, float4 o, const float (&d)[4])
{
    o.x += d[0]; o.y += d[1]; o.z += d[2]; o.w += d[3];
    if (c.all) {
        *reinterpret_cast<float4*>(f) = o;
    } else {
        if (c.vx[0]) f[0] = o.x;
        if (c.vx[1]) f[1] = o.y;
        if (c.vx[2]) f[2] = o.z;
        if (c.vx[3]) f[3] = o.w;
    }
}

// ------------------------------------------------------------ REF (collocated FD4)
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

__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
eqwp_ref_stress(FieldPtrs F, const BlockLayout L, int step_i, int nzc, EqwpRefParams p)
{
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 2);
    Cell c;
    if (!cell_setup(L, w, blk, c)) return;
    const long long P = L.P, S = L.plane;
    const float* vx = F.p[VX] + c.base;
    const float* vy = F.p[VY] + c.base;
    const float* vz = F.p[VZ] + c.base;
    Q5v qx, qy, qz;
    {
        const long long o = (long long)(w.zs - 2) * S;
        qx.m1 = ld4(vx + o); qy.m1 = ld4(vy + o); qz.m1 = ld4(vz + o);
        qx.c = ld4(vx + o + S); qy.c = ld4(vy + o + S); qz.c = ld4(vz + o + S);
        qx.p1 = ld4(vx + o + 2 * S); qy.p1 = ld4(vy + o + 2 * S); qz.p1 = ld4(vz + o + 2 * S);
        qx.p2 = ld4(vx + o + 3 * S); qy.p2 = ld4(vy + o + 3 * S); qz.p2 = ld4(vz + o + 3 * S);
    }
    const float a = p.ca, b = p.cb;
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        qx.shift(ld4(vx + o + 2 * S));
        qy.shift(ld4(vy + o + 2 * S));
        qz.shift(ld4(vz + o + 2 * S));
        Row12 rx, ry, rz;
        rx.load(vx + o);
        ry.load(vy + o);
        rz.load(vz + o);
        const float4 xm2 = ld4(vx + o - 2 * P), xm1 = ld4(vx + o - P), xp1 = ld4(vx + o + P), xp2 = ld4(vx + o + 2 * P);
        const float4 ym2 = ld4(vy + o - 2 * P), ym1 = ld4(vy + o - P), yp1 = ld4(vy + o + P), yp2 = ld4(vy + o + 2 * P);
        const float4 zm2 = ld4(vz + o - 2 * P), zm1 = ld4(vz + o - P), zp1 = ld4(vz + o + P), zp2 = ld4(vz + o + 2 * P);
        float* const dst[6] = {F.p[SXX] + c.base + o, F.p[SYY] + c.base + o, F.p[SZZ] + c.base + o,
                               F.p[SXY] + c.base + o, F.p[SXZ] + c.base + o, F.p[SYZ] + c.base + o};
        float4 old[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) old[f] = rd4(dst[f], c);
        float dxx[4], dyy[4], dzz[4], dxy[4], dxz[4], dyz[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float dvxx = dcx(rx, j, a, b);
            const float dvxy = dc4(xm2, xm1, xp1, xp2, j, a, b);
            const float dvxz = dc4(qx.m2, qx.m1, qx.p1, qx.p2, j, a, b);
            const float dvyx = dcx(ry, j, a, b);
            const float dvyy = dc4(ym2, ym1, yp1, yp2, j, a, b);
            const float dvyz = dc4(qy.m2, qy.m1, qy.p1, qy.p2, j, a, b);
            const float dvzx = dcx(rz, j, a, b);
            const float dvzy = dc4(zm2, zm1, zp1, zp2, j, a, b);
            const float dvzz = dc4(qz.m2, qz.m1, qz.p1, qz.p2, j, a, b);
            // eqwp.cu:460-473, dt folded into the Lame constants
            dxx[j] = p.l2m_dt * dvxx + p.l_dt * (dvyy + dvzz);
            dyy[j] = p.l2m_dt * dvyy + p.l_dt * (dvxx + dvzz);
            dzz[j] = p.l2m_dt * dvzz + p.l_dt * (dvxx + dvyy);
            dxy[j] = p.mu_dt * (dvxy + dvyx);
            dxz[j] = p.mu_dt * (dvxz + dvzx);
            dyz[j] = p.mu_dt * (dvyz + dvzy);
        }
        wr4(dst[0], c, old[0], dxx);
        wr4(dst[1], c, old[1], dyy);
        wr4(dst[2], c, old[2], dzz);
        wr4(dst[3], c, old[3], dxy);
        wr4(dst[4], c, old[4], dxz);
        wr4(dst[5], c, old[5], dyz);
    }
}

__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
eqwp_ref_velocity(FieldPtrs F, const BlockLayout L, int step_i, int nzc, EqwpRefParams p, int ts)
{
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 4);
    Cell c;
    if (!cell_setup(L, w, blk, c)) return;
    const long long P = L.P, S = L.plane;
    const float* sxx = F.p[SXX] + c.base;
    const float* sxy = F.p[SXY] + c.base;
    const float* sxz = F.p[SXZ] + c.base;
    const float* syy = F.p[SYY] + c.base;
    const float* syz = F.p[SYZ] + c.base;
    const float* szz = F.p[SZZ] + c.base;
    Q5v qxz, qyz, qzz;
    {
        const long long o = (long long)(w.zs - 2) * S;
        qxz.m1 = ld4(sxz + o); qyz.m1 = ld4(syz + o); qzz.m1 = ld4(szz + o);
        qxz.c = ld4(sxz + o + S); qyz.c = ld4(syz + o + S); qzz.c = ld4(szz + o + S);
        qxz.p1 = ld4(sxz + o + 2 * S); qyz.p1 = ld4(syz + o + 2 * S); qzz.p1 = ld4(szz + o + 2 * S);
        qxz.p2 = ld4(sxz + o + 3 * S); qyz.p2 = ld4(syz + o + 3 * S); qzz.p2 = ld4(szz + o + 3 * S);
    }
    const float a = p.ca, b = p.cb;
    const bool frow = (c.y == p.fy) && (ts < p.fsteps);
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        qxz.shift(ld4(sxz + o + 2 * S));
        qyz.shift(ld4(syz + o + 2 * S));
        qzz.shift(ld4(szz + o + 2 * S));
        Row12 rxx, rxy, rxz;
        rxx.load(sxx + o);
        rxy.load(sxy + o);
        rxz.load(sxz + o);
        const float4 xym2 = ld4(sxy + o - 2 * P), xym1 = ld4(sxy + o - P), xyp1 = ld4(sxy + o + P), xyp2 = ld4(sxy + o + 2 * P);
        const float4 yym2 = ld4(syy + o - 2 * P), yym1 = ld4(syy + o - P), yyp1 = ld4(syy + o + P), yyp2 = ld4(syy + o + 2 * P);
        const float4 yzm2 = ld4(syz + o - 2 * P), yzm1 = ld4(syz + o - P), yzp1 = ld4(syz + o + P), yzp2 = ld4(syz + o + 2 * P);
        const bool fz = frow && z >= p.fz0 && z < p.fz1;
        float* const dst[4] = {F.p[VX] + c.base + o, F.p[VY] + c.base + o, F.p[VZ] + c.base + o,
                               F.p[DISP] + c.base + o};
        float4 old[4];
#pragma unroll
        for (int f = 0; f < 4; ++f) old[f] = rd4(dst[f], c);
        float dvx[4], dvy[4], dvz[4], dd[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float sx = dcx(rxx, j, a, b) + dc4(xym2, xym1, xyp1, xyp2, j, a, b) +
                             dc4(qxz.m2, qxz.m1, qxz.p1, qxz.p2, j, a, b);
            float sy = dcx(rxy, j, a, b) + dc4(yym2, yym1, yyp1, yyp2, j, a, b) +
                       dc4(qyz.m2, qyz.m1, qyz.p1, qyz.p2, j, a, b);
            const float sz = dcx(rxz, j, a, b) + dc4(yzm2, yzm1, yzp1, yzp2, j, a, b) +
                             dc4(qzz.m2, qzz.m1, qzz.p1, qzz.p2, j, a, b);
            if (fz && c.xb + j >= p.fx0 && c.xb + j < p.fx1) sy += p.fval;
            dvx[j] = p.dt_rho * sx;
            dvy[j] = p.dt_rho * sy;
            dvz[j] = p.dt_rho * sz;
            dd[j] = p.dt2_rho * sy;
        }
        wr4(dst[0], c, old[0], dvx);
        wr4(dst[1], c, old[1], dvy);
        wr4(dst[2], c, old[2], dvz);
        wr4(dst[3], c, old[3], dd);
    }
}

// ------------------------------------------------------------ STAG (staggered FD4)
// forward difference at i+1/2 and backward at i-1/2, 4th order (9/8, -1/24)
__device__ __forceinline__ float dpx(const Row12& r, int j)
{
    return 1.125f * (r.v[5 + j] - r.v[4 + j]) - (1.f / 24.f) * (r.v[6 + j] - r.v[3 + j]);
}
__device__ __forceinline__ float dmx(const Row12& r, int j)
{
    return 1.125f * (r.v[4 + j] - r.v[3 + j]) - (1.f / 24.f) * (r.v[5 + j] - r.v[2 + j]);
}
// rows/planes -2..+2 around the cell: Dp uses -1..+2, Dm uses -2..+1
__device__ __forceinline__ float dp4(const float4& m1, const float4& c, const float4& p1,
                                     const float4& p2, int j)
{
    return 1.125f * (cmp(p1, j) - cmp(c, j)) - (1.f / 24.f) * (cmp(p2, j) - cmp(m1, j));
}
__device__ __forceinline__ float dm4(const float4& m2, const float4& m1, const float4& c,
                                     const float4& p1, int j)
{
    return 1.125f * (cmp(c, j) - cmp(m1, j)) - (1.f / 24.f) * (cmp(p1, j) - cmp(m2, j));
}

__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
eqwp_stag_velocity(FieldPtrs F, MatPtrs M, const BlockLayout L, int step_i, int nzc,
                   EqwpStagParams p)
{
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 2);
    Cell c;
    if (!cell_setup(L, w, blk, c)) return;
    const long long P = L.P, S = L.plane;
    const float* sxx = F.p[SXX] + c.base;
    const float* sxy = F.p[SXY] + c.base;
    const float* sxz = F.p[SXZ] + c.base;
    const float* syy = F.p[SYY] + c.base;
    const float* syz = F.p[SYZ] + c.base;
    const float* szz = F.p[SZZ] + c.base;
    const float* buoy = M.p[2] + c.base;
    Q5v qxz, qyz, qzz;
    {
        const long long o = (long long)(w.zs - 2) * S;
        qxz.m1 = ld4(sxz + o); qyz.m1 = ld4(syz + o); qzz.m1 = ld4(szz + o);
        qxz.c = ld4(sxz + o + S); qyz.c = ld4(syz + o + S); qzz.c = ld4(szz + o + S);
        qxz.p1 = ld4(sxz + o + 2 * S); qyz.p1 = ld4(syz + o + 2 * S); qzz.p1 = ld4(szz + o + 2 * S);
        qxz.p2 = ld4(sxz + o + 3 * S); qyz.p2 = ld4(syz + o + 3 * S); qzz.p2 = ld4(szz + o + 3 * S);
    }
    const float k = p.dt * p.inv_h;
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        qxz.shift(ld4(sxz + o + 2 * S));
        qyz.shift(ld4(syz + o + 2 * S));
        qzz.shift(ld4(szz + o + 2 * S));
        Row12 rxx, rxy, rxz;
        rxx.load(sxx + o);
        rxy.load(sxy + o);
        rxz.load(sxz + o);
        const float4 xym2 = ld4(sxy + o - 2 * P), xym1 = ld4(sxy + o - P), xyp1 = ld4(sxy + o + P);
        const float4 yym1 = ld4(syy + o - P), yyc = ld4(syy + o), yyp1 = ld4(syy + o + P), yyp2 = ld4(syy + o + 2 * P);
        const float4 yzm2 = ld4(syz + o - 2 * P), yzm1 = ld4(syz + o - P), yzp1 = ld4(syz + o + P);
        const float4 xyc = make_float4(rxy.v[4], rxy.v[5], rxy.v[6], rxy.v[7]);
        const float4 bb = ld4(buoy + o);
        float* const dst[3] = {F.p[VX] + c.base + o, F.p[VY] + c.base + o, F.p[VZ] + c.base + o};
        float4 old[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) old[f] = rd4(dst[f], c);
        float dvx[4], dvy[4], dvz[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float ax = dpx(rxx, j) + dm4(xym2, xym1, xyc, xyp1, j) + dm4(qxz.m2, qxz.m1, qxz.c, qxz.p1, j);
            const float ay = dmx(rxy, j) + dp4(yym1, yyc, yyp1, yyp2, j) + dm4(qyz.m2, qyz.m1, qyz.c, qyz.p1, j);
            const float az = dmx(rxz, j) + dm4(yzm2, yzm1, qyz.c, yzp1, j) + dp4(qzz.m1, qzz.c, qzz.p1, qzz.p2, j);
            const float kb = k * cmp(bb, j);
            dvx[j] = kb * ax;
            dvy[j] = kb * ay;
            dvz[j] = kb * az;
        }
        wr4(dst[0], c, old[0], dvx);
        wr4(dst[1], c, old[1], dvy);
        wr4(dst[2], c, old[2], dvz);
    }
}

__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
eqwp_stag_stress(FieldPtrs F, MatPtrs M, const BlockLayout L, int step_i, int nzc,
                 EqwpStagParams p, float src_amp)
{
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 4);
    Cell c;
    if (!cell_setup(L, w, blk, c)) return;
    const long long P = L.P, S = L.plane;
    const float* vx = F.p[VX] + c.base;
    const float* vy = F.p[VY] + c.base;
    const float* vz = F.p[VZ] + c.base;
    const float* lam = M.p[0] + c.base;
    const float* mu = M.p[1] + c.base;
    Q5v qx, qy, qz;
    {
        const long long o = (long long)(w.zs - 2) * S;
        qx.m1 = ld4(vx + o); qy.m1 = ld4(vy + o); qz.m1 = ld4(vz + o);
        qx.c = ld4(vx + o + S); qy.c = ld4(vy + o + S); qz.c = ld4(vz + o + S);
        qx.p1 = ld4(vx + o + 2 * S); qy.p1 = ld4(vy + o + 2 * S); qz.p1 = ld4(vz + o + 2 * S);
        qx.p2 = ld4(vx + o + 3 * S); qy.p2 = ld4(vy + o + 3 * S); qz.p2 = ld4(vz + o + 3 * S);
    }
    const float k = p.dt * p.inv_h;
    // source cell of this block, in block coordinates
    const int b0 = blk % L.nb[0], b1 = (blk / L.nb[0]) % L.nb[1], b2 = blk / (L.nb[0] * L.nb[1]);
    const int sx = p.src[0] - b0 * L.B[0] + L.H, sy = p.src[1] - b1 * L.B[1] + L.H,
              sz = p.src[2] - b2 * L.B[2] + L.H;
    const bool srow = (c.y == sy) && sx >= c.xb && sx < c.xb + 4;
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        qx.shift(ld4(vx + o + 2 * S));
        qy.shift(ld4(vy + o + 2 * S));
        qz.shift(ld4(vz + o + 2 * S));
        Row12 rx, ry, rz;
        rx.load(vx + o);
        ry.load(vy + o);
        rz.load(vz + o);
        const float4 xc = make_float4(rx.v[4], rx.v[5], rx.v[6], rx.v[7]);
        const float4 yc = make_float4(ry.v[4], ry.v[5], ry.v[6], ry.v[7]);
        const float4 zc4 = make_float4(rz.v[4], rz.v[5], rz.v[6], rz.v[7]);
        const float4 xm1 = ld4(vx + o - P), xp1 = ld4(vx + o + P), xp2 = ld4(vx + o + 2 * P);
        const float4 ym2 = ld4(vy + o - 2 * P), ym1 = ld4(vy + o - P), yp1 = ld4(vy + o + P);
        const float4 zm1 = ld4(vz + o - P), zp1 = ld4(vz + o + P), zp2 = ld4(vz + o + 2 * P);
        const float4 l4 = ld4(lam + o), m4 = ld4(mu + o);
        const bool src_here = srow && z == sz;
        float* const dst[6] = {F.p[SXX] + c.base + o, F.p[SYY] + c.base + o, F.p[SZZ] + c.base + o,
                               F.p[SXY] + c.base + o, F.p[SXZ] + c.base + o, F.p[SYZ] + c.base + o};
        float4 old[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) old[f] = rd4(dst[f], c);
        float dxx[4], dyy[4], dzz[4], dxy[4], dxz[4], dyz[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float exx = dmx(rx, j);
            const float eyy = dm4(ym2, ym1, yc, yp1, j);
            const float ezz = dm4(qz.m2, qz.m1, qz.c, qz.p1, j);
            const float vx_y = dp4(xm1, xc, xp1, xp2, j);
            const float vy_x = dpx(ry, j);
            const float vx_z = dp4(qx.m1, qx.c, qx.p1, qx.p2, j);
            const float vz_x = dpx(rz, j);
            const float vy_z = dp4(qy.m1, qy.c, qy.p1, qy.p2, j);
            const float vz_y = dp4(zm1, zc4, zp1, zp2, j);
            const float l = cmp(l4, j), m = cmp(m4, j);
            const float l2m = l + 2.f * m;
            float axx = k * (l2m * exx + l * (eyy + ezz));
            float ayy = k * (l2m * eyy + l * (exx + ezz));
            float azz = k * (l2m * ezz + l * (exx + eyy));
            if (src_here && c.xb + j == sx) {
                axx += src_amp;
                ayy += src_amp;
                azz += src_amp;
            }
            dxx[j] = axx;
            dyy[j] = ayy;
            dzz[j] = azz;
            dxy[j] = k * m * (vx_y + vy_x);
            dxz[j] = k * m * (vx_z + vz_x);
            dyz[j] = k * m * (vy_z + vz_y);
        }
        wr4(dst[0], c, old[0], dxx);
        wr4(dst[1], c, old[1], dyy);
        wr4(dst[2], c, old[2], dzz);
        wr4(dst[3], c, old[3], dxy);
        wr4(dst[4], c, old[4], dxz);
        wr4(dst[5], c, old[5], dyz);
    }
}

struct Grid {
    dim3 g;
    int nzc;
};

Grid stage_grid(const BlockLayout& L)
{
    Grid r;
    const int xs_begin = (L.xoff + 2) & ~3;
    const int xs_end = L.xoff + L.n[0] - 2;               // exclusive
    const int tx = (xs_end - xs_begin + kTXc - 1) / kTXc;
    const int ty = (L.n[1] - 4 + kBY - 1) / kBY;
    const long long tiles = (long long)tx * ty * L.nblk;
    const long long want = 152LL * 8 * 3;
    int nzc = (int)((want + tiles - 1) / tiles);
    int maxc = (L.n[2] - 4) / 16;
    if (maxc < 1) maxc = 1;
    if (nzc > maxc) nzc = maxc;
    if (nzc < 1) nzc = 1;
    r.nzc = nzc;
    r.g = dim3(tx, ty, L.nblk * nzc);
    return r;
}

}  // namespace

EqwpRefParams eqwp_ref_params(const BlockLayout& L)
{
    // constants of eqwp.cu:9-23 (double there), folded for FP32
    const double Dt = 0.5, Dx = 10.0, inv_rho = 0.0005555555555555556;
    const double lame1 = 32.00, lame2 = 174.87;
    EqwpRefParams p{};
    p.ca = (float)((-1.0 / 12.0) / Dx);
    p.cb = (float)((2.0 / 3.0) / Dx);
    p.l2m_dt = (float)(Dt * (lame1 + 2 * lame2));
    p.l_dt = (float)(Dt * lame1);
    p.mu_dt = (float)(Dt * lame2);
    p.dt_rho = (float)(Dt * inv_rho);
    p.dt2_rho = (float)(Dt * Dt * inv_rho);
    p.fval = -10000.f;
    p.fsteps = 50;
    // Force patch of eqwp.cu:561-566 and plane of eqwp.cu:135, as the
    // reference places them in its block of Ng = B + 4 cells (R = 1), mapped
    // to this block (interior starts at H): plane y = B - 7 of the interior,
    // x and z in [Ng/2 - 2, Ng/2 + Ng/10 - 2).
    const int ngx = L.B[0] + 4, ngz = L.B[2] + 4;
    p.fy = L.H + L.B[1] - 7;
    p.fx0 = L.H + ngx / 2 - 2;
    p.fx1 = L.H + ngx / 2 + ngx / 10 - 2;
    p.fz0 = L.H + ngz / 2 - 2;
    p.fz1 = L.H + ngz / 2 + ngz / 10 - 2;
    return p;
}

cudaError_t launch_eqwp_ref_substep(float* const* fld, const BlockLayout& L, int step_i, int ts,
                                    const EqwpRefParams& p, cudaStream_t st)
{
    FieldPtrs F{};
    for (int f = 0; f < 10; ++f) F.p[f] = fld[f];
    const Grid g = stage_grid(L);
    eqwp_ref_stress<<<g.g, dim3(kBX, kBY), 0, st>>>(F, L, step_i, g.nzc, p);
    eqwp_ref_velocity<<<g.g, dim3(kBX, kBY), 0, st>>>(F, L, step_i, g.nzc, p, ts);
    count_launches(2);
    return cudaGetLastError();
}

cudaError_t launch_eqwp_stag_substep(float* const* fld, float* const* mat, const BlockLayout& L,
                                     int step_i, int ts, const EqwpStagParams& p, cudaStream_t st)
{
    FieldPtrs F{};
    for (int f = 0; f < 9; ++f) F.p[f] = fld[f];
    MatPtrs M{};
    for (int m = 0; m < 3; ++m) M.p[m] = mat[m];
    const Grid g = stage_grid(L);
    float amp = 0.f;
    if (p.src_host && ts >= 0 && ts < p.src_len) amp = p.src_host[ts];
    eqwp_stag_velocity<<<g.g, dim3(kBX, kBY), 0, st>>>(F, M, L, step_i, g.nzc, p);
    eqwp_stag_stress<<<g.g, dim3(kBX, kBY), 0, st>>>(F, M, L, step_i, g.nzc, p, amp);
    count_launches(2);
    return cudaGetLastError();
}

}  // namespace b2r
