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

constexpr int kBX = 32, kBY = 8;

enum { VX, VY, VZ, SXX, SXY, SXZ, SYY, SYZ, SZZ, DISP };

struct Q5 {
    float m2, m1, c, p1, p2;
    __device__ __forceinline__ void shift(float nv)
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

// collocated FD4 derivative (times 1/dx folded into the coefficients)
__device__ __forceinline__ float dc(float m2, float m1, float p1, float p2, float a, float b)
{
    return a * (p2 - m2) + b * (p1 - m1);
}

// ------------------------------------------------------------ REF stress stage
__global__ void __launch_bounds__(kBX * kBY)
eqwp_ref_stress(FieldPtrs F, const BlockLayout L, int step_i, int nzc, EqwpRefParams p)
{
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 2);
    const int x = 2 + blockIdx.x * kBX + threadIdx.x;
    const int y = 2 + blockIdx.y * kBY + threadIdx.y;
    if (!w.ok || x < w.lo[0] || x > w.hi[0] || y < w.lo[1] || y > w.hi[1]) return;
    const long long base = (long long)blk * L.bstride + (long long)y * L.P + L.xoff + x;
    const long long P = L.P, S = L.plane;
    const float* vx = F.p[VX] + base;
    const float* vy = F.p[VY] + base;
    const float* vz = F.p[VZ] + base;
    Q5 qx, qy, qz;
    {
        const long long o = (long long)(w.zs - 2) * S;
        qx.m1 = __ldg(vx + o); qy.m1 = __ldg(vy + o); qz.m1 = __ldg(vz + o);
        qx.c = __ldg(vx + o + S); qy.c = __ldg(vy + o + S); qz.c = __ldg(vz + o + S);
        qx.p1 = __ldg(vx + o + 2 * S); qy.p1 = __ldg(vy + o + 2 * S); qz.p1 = __ldg(vz + o + 2 * S);
        qx.p2 = __ldg(vx + o + 3 * S); qy.p2 = __ldg(vy + o + 3 * S); qz.p2 = __ldg(vz + o + 3 * S);
    }
    const float a = p.ca, b = p.cb;
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        qx.shift(__ldg(vx + o + 2 * S));
        qy.shift(__ldg(vy + o + 2 * S));
        qz.shift(__ldg(vz + o + 2 * S));
        const float* X = vx + o;
        const float* Y = vy + o;
        const float* Z = vz + o;
        const float dvxx = dc(__ldg(X - 2), __ldg(X - 1), __ldg(X + 1), __ldg(X + 2), a, b);
        const float dvxy = dc(__ldg(X - 2 * P), __ldg(X - P), __ldg(X + P), __ldg(X + 2 * P), a, b);
        const float dvxz = dc(qx.m2, qx.m1, qx.p1, qx.p2, a, b);
        const float dvyx = dc(__ldg(Y - 2), __ldg(Y - 1), __ldg(Y + 1), __ldg(Y + 2), a, b);
        const float dvyy = dc(__ldg(Y - 2 * P), __ldg(Y - P), __ldg(Y + P), __ldg(Y + 2 * P), a, b);
        const float dvyz = dc(qy.m2, qy.m1, qy.p1, qy.p2, a, b);
        const float dvzx = dc(__ldg(Z - 2), __ldg(Z - 1), __ldg(Z + 1), __ldg(Z + 2), a, b);
        const float dvzy = dc(__ldg(Z - 2 * P), __ldg(Z - P), __ldg(Z + P), __ldg(Z + 2 * P), a, b);
        const float dvzz = dc(qz.m2, qz.m1, qz.p1, qz.p2, a, b);
        const long long id = base + o;
        // eqwp.cu:460-473, with dt folded into the Lame constants
        F.p[SXX][id] += p.l2m_dt * dvxx + p.l_dt * (dvyy + dvzz);
        F.p[SYY][id] += p.l2m_dt * dvyy + p.l_dt * (dvxx + dvzz);
        F.p[SZZ][id] += p.l2m_dt * dvzz + p.l_dt * (dvxx + dvyy);
        F.p[SXY][id] += p.mu_dt * (dvxy + dvyx);
        F.p[SXZ][id] += p.mu_dt * (dvxz + dvzx);
        F.p[SYZ][id] += p.mu_dt * (dvyz + dvzy);
    }
}

// ------------------------------------------------------------ REF velocity stage
__global__ void __launch_bounds__(kBX * kBY)
eqwp_ref_velocity(FieldPtrs F, const BlockLayout L, int step_i, int nzc, EqwpRefParams p, int ts)
{
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 4);
    const int x = 2 + blockIdx.x * kBX + threadIdx.x;
    const int y = 2 + blockIdx.y * kBY + threadIdx.y;
    if (!w.ok || x < w.lo[0] || x > w.hi[0] || y < w.lo[1] || y > w.hi[1]) return;
    const long long base = (long long)blk * L.bstride + (long long)y * L.P + L.xoff + x;
    const long long P = L.P, S = L.plane;
    const float* sxx = F.p[SXX] + base;
    const float* sxy = F.p[SXY] + base;
    const float* sxz = F.p[SXZ] + base;
    const float* syy = F.p[SYY] + base;
    const float* syz = F.p[SYZ] + base;
    const float* szz = F.p[SZZ] + base;
    Q5 qxz, qyz, qzz;
    {
        const long long o = (long long)(w.zs - 2) * S;
        qxz.m1 = __ldg(sxz + o); qyz.m1 = __ldg(syz + o); qzz.m1 = __ldg(szz + o);
        qxz.c = __ldg(sxz + o + S); qyz.c = __ldg(syz + o + S); qzz.c = __ldg(szz + o + S);
        qxz.p1 = __ldg(sxz + o + 2 * S); qyz.p1 = __ldg(syz + o + 2 * S); qzz.p1 = __ldg(szz + o + 2 * S);
        qxz.p2 = __ldg(sxz + o + 3 * S); qyz.p2 = __ldg(syz + o + 3 * S); qzz.p2 = __ldg(szz + o + 3 * S);
    }
    const float a = p.ca, b = p.cb;
    const bool frow = (y == p.fy) && (ts < p.fsteps) && x >= p.fx0 && x < p.fx1;
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        qxz.shift(__ldg(sxz + o + 2 * S));
        qyz.shift(__ldg(syz + o + 2 * S));
        qzz.shift(__ldg(szz + o + 2 * S));
        const float* XX = sxx + o;
        const float* XY = sxy + o;
        const float* XZ = sxz + o;
        const float* YY = syy + o;
        const float* YZ = syz + o;
        const float dsxx_x = dc(__ldg(XX - 2), __ldg(XX - 1), __ldg(XX + 1), __ldg(XX + 2), a, b);
        const float dsxy_y = dc(__ldg(XY - 2 * P), __ldg(XY - P), __ldg(XY + P), __ldg(XY + 2 * P), a, b);
        const float dsxz_z = dc(qxz.m2, qxz.m1, qxz.p1, qxz.p2, a, b);
        const float dsxy_x = dc(__ldg(XY - 2), __ldg(XY - 1), __ldg(XY + 1), __ldg(XY + 2), a, b);
        const float dsyy_y = dc(__ldg(YY - 2 * P), __ldg(YY - P), __ldg(YY + P), __ldg(YY + 2 * P), a, b);
        const float dsyz_z = dc(qyz.m2, qyz.m1, qyz.p1, qyz.p2, a, b);
        const float dsxz_x = dc(__ldg(XZ - 2), __ldg(XZ - 1), __ldg(XZ + 1), __ldg(XZ + 2), a, b);
        const float dsyz_y = dc(__ldg(YZ - 2 * P), __ldg(YZ - P), __ldg(YZ + P), __ldg(YZ + 2 * P), a, b);
        const float dszz_z = dc(qzz.m2, qzz.m1, qzz.p1, qzz.p2, a, b);
        const long long id = base + o;
        float sy = dsxy_x + dsyy_y + dsyz_z;
        if (frow && z >= p.fz0 && z < p.fz1) sy += p.fval;
        F.p[VX][id] += p.dt_rho * (dsxx_x + dsxy_y + dsxz_z);
        F.p[VY][id] += p.dt_rho * sy;
        F.p[DISP][id] += p.dt2_rho * sy;
        F.p[VZ][id] += p.dt_rho * (dsxz_x + dsyz_y + dszz_z);
    }
}

// ------------------------------------------------------------ STAG stages
// forward (at i+1/2) and backward (at i-1/2) staggered 4th-order differences
__device__ __forceinline__ float dp(float m1, float c, float p1, float p2)
{
    return 1.125f * (p1 - c) - (1.f / 24.f) * (p2 - m1);
}
__device__ __forceinline__ float dm(float m2, float m1, float c, float p1)
{
    return 1.125f * (c - m1) - (1.f / 24.f) * (p1 - m2);
}

__global__ void __launch_bounds__(kBX * kBY)
eqwp_stag_velocity(FieldPtrs F, MatPtrs M, const BlockLayout L, int step_i, int nzc,
                   EqwpStagParams p)
{
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 2);
    const int x = 2 + blockIdx.x * kBX + threadIdx.x;
    const int y = 2 + blockIdx.y * kBY + threadIdx.y;
    if (!w.ok || x < w.lo[0] || x > w.hi[0] || y < w.lo[1] || y > w.hi[1]) return;
    const long long base = (long long)blk * L.bstride + (long long)y * L.P + L.xoff + x;
    const long long P = L.P, S = L.plane;
    const float* sxx = F.p[SXX] + base;
    const float* sxy = F.p[SXY] + base;
    const float* sxz = F.p[SXZ] + base;
    const float* syy = F.p[SYY] + base;
    const float* syz = F.p[SYZ] + base;
    const float* szz = F.p[SZZ] + base;
    const float* buoy = M.p[2] + base;
    Q5 qxz, qyz, qzz;
    {
        const long long o = (long long)(w.zs - 2) * S;
        qxz.m1 = __ldg(sxz + o); qyz.m1 = __ldg(syz + o); qzz.m1 = __ldg(szz + o);
        qxz.c = __ldg(sxz + o + S); qyz.c = __ldg(syz + o + S); qzz.c = __ldg(szz + o + S);
        qxz.p1 = __ldg(sxz + o + 2 * S); qyz.p1 = __ldg(syz + o + 2 * S); qzz.p1 = __ldg(szz + o + 2 * S);
        qxz.p2 = __ldg(sxz + o + 3 * S); qyz.p2 = __ldg(syz + o + 3 * S); qzz.p2 = __ldg(szz + o + 3 * S);
    }
    const float k = p.dt * p.inv_h;
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        qxz.shift(__ldg(sxz + o + 2 * S));
        qyz.shift(__ldg(syz + o + 2 * S));
        qzz.shift(__ldg(szz + o + 2 * S));
        const float* XX = sxx + o;
        const float* XY = sxy + o;
        const float* XZ = sxz + o;
        const float* YY = syy + o;
        const float* YZ = syz + o;
        const float ax = dp(__ldg(XX - 1), __ldg(XX), __ldg(XX + 1), __ldg(XX + 2)) +
                         dm(__ldg(XY - 2 * P), __ldg(XY - P), __ldg(XY), __ldg(XY + P)) +
                         dm(qxz.m2, qxz.m1, qxz.c, qxz.p1);
        const float ay = dm(__ldg(XY - 2), __ldg(XY - 1), __ldg(XY), __ldg(XY + 1)) +
                         dp(__ldg(YY - P), __ldg(YY), __ldg(YY + P), __ldg(YY + 2 * P)) +
                         dm(qyz.m2, qyz.m1, qyz.c, qyz.p1);
        const float az = dm(__ldg(XZ - 2), __ldg(XZ - 1), __ldg(XZ), __ldg(XZ + 1)) +
                         dm(__ldg(YZ - 2 * P), __ldg(YZ - P), __ldg(YZ), __ldg(YZ + P)) +
                         dp(qzz.m1, qzz.c, qzz.p1, qzz.p2);
        const long long id = base + o;
        const float kb = k * __ldg(buoy + o);
        F.p[VX][id] += kb * ax;
        F.p[VY][id] += kb * ay;
        F.p[VZ][id] += kb * az;
    }
}

__global__ void __launch_bounds__(kBX * kBY)
eqwp_stag_stress(FieldPtrs F, MatPtrs M, const BlockLayout L, int step_i, int nzc,
                 EqwpStagParams p, float src_amp)
{
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 4);
    const int x = 2 + blockIdx.x * kBX + threadIdx.x;
    const int y = 2 + blockIdx.y * kBY + threadIdx.y;
    if (!w.ok || x < w.lo[0] || x > w.hi[0] || y < w.lo[1] || y > w.hi[1]) return;
    const long long base = (long long)blk * L.bstride + (long long)y * L.P + L.xoff + x;
    const long long P = L.P, S = L.plane;
    const float* vx = F.p[VX] + base;
    const float* vy = F.p[VY] + base;
    const float* vz = F.p[VZ] + base;
    const float* lam = M.p[0] + base;
    const float* mu = M.p[1] + base;
    Q5 qx, qy, qz;
    {
        const long long o = (long long)(w.zs - 2) * S;
        qx.m1 = __ldg(vx + o); qy.m1 = __ldg(vy + o); qz.m1 = __ldg(vz + o);
        qx.c = __ldg(vx + o + S); qy.c = __ldg(vy + o + S); qz.c = __ldg(vz + o + S);
        qx.p1 = __ldg(vx + o + 2 * S); qy.p1 = __ldg(vy + o + 2 * S); qz.p1 = __ldg(vz + o + 2 * S);
        qx.p2 = __ldg(vx + o + 3 * S); qy.p2 = __ldg(vy + o + 3 * S); qz.p2 = __ldg(vz + o + 3 * S);
    }
    const float k = p.dt * p.inv_h;
    // source cell of this block, in block coordinates
    const int b0 = blk % L.nb[0], b1 = (blk / L.nb[0]) % L.nb[1], b2 = blk / (L.nb[0] * L.nb[1]);
    const int sx = p.src[0] - b0 * L.B[0] + L.H, sy = p.src[1] - b1 * L.B[1] + L.H,
              sz = p.src[2] - b2 * L.B[2] + L.H;
    const bool srow = (x == sx) && (y == sy);
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        qx.shift(__ldg(vx + o + 2 * S));
        qy.shift(__ldg(vy + o + 2 * S));
        qz.shift(__ldg(vz + o + 2 * S));
        const float* X = vx + o;
        const float* Y = vy + o;
        const float* Z = vz + o;
        const float exx = dm(__ldg(X - 2), __ldg(X - 1), __ldg(X), __ldg(X + 1));
        const float eyy = dm(__ldg(Y - 2 * P), __ldg(Y - P), __ldg(Y), __ldg(Y + P));
        const float ezz = dm(qz.m2, qz.m1, qz.c, qz.p1);
        const float vx_y = dp(__ldg(X - P), __ldg(X), __ldg(X + P), __ldg(X + 2 * P));
        const float vy_x = dp(__ldg(Y - 1), __ldg(Y), __ldg(Y + 1), __ldg(Y + 2));
        const float vx_z = dp(qx.m1, qx.c, qx.p1, qx.p2);
        const float vz_x = dp(__ldg(Z - 1), __ldg(Z), __ldg(Z + 1), __ldg(Z + 2));
        const float vy_z = dp(qy.m1, qy.c, qy.p1, qy.p2);
        const float vz_y = dp(__ldg(Z - P), __ldg(Z), __ldg(Z + P), __ldg(Z + 2 * P));
        const long long id = base + o;
        const float l = __ldg(lam + o), m = __ldg(mu + o);
        const float l2m = l + 2.f * m;
        float dxx = k * (l2m * exx + l * (eyy + ezz));
        float dyy = k * (l2m * eyy + l * (exx + ezz));
        float dzz = k * (l2m * ezz + l * (exx + eyy));
        if (srow && z == sz) {
            dxx += src_amp;
            dyy += src_amp;
            dzz += src_amp;
        }
        F.p[SXX][id] += dxx;
        F.p[SYY][id] += dyy;
        F.p[SZZ][id] += dzz;
        F.p[SXY][id] += k * m * (vx_y + vy_x);
        F.p[SXZ][id] += k * m * (vx_z + vz_x);
        F.p[SYZ][id] += k * m * (vy_z + vz_y);
    }
}

struct Grid {
    dim3 g;
    int nzc;
};

Grid stage_grid(const BlockLayout& L)
{
    Grid r;
    const int nx = L.n[0] - 4, ny = L.n[1] - 4;
    const int tx = (nx + kBX - 1) / kBX, ty = (ny + kBY - 1) / kBY;
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
