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
#include "eqwp_tile.cuh"
#include "eqwp_stag.cuh"

namespace b2r {

namespace {

using namespace eqk;

// ------------------------------------------------------------ REF (collocated FD4)
__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
eqwp_ref_stress(FieldPtrs F, const BlockLayout L, int step_i, Tiles T, EqwpRefParams p)
{
    const int nzc = T.nzc;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 2);
    Cell c;
    if (!cell_setup(L, w, blk, c, T.x0, T.y0)) return;
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
        if (B2R_EQWP_PREFETCH > 0) {
            const long long oa = ahead(L, z, B2R_EQWP_PREFETCH, w.ze),
                            oq = ahead(L, z, 2 + B2R_EQWP_PREFETCH, w.ze + 2);
            pf_l2(vx + oq);
            pf_l2(vy + oq);
            pf_l2(vz + oq);
#pragma unroll
            for (int f = SXX; f <= SZZ; ++f) pf_l2(F.p[f] + c.base + oa);
        }
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
eqwp_ref_velocity(FieldPtrs F, const BlockLayout L, int step_i, Tiles T, EqwpRefParams p, int ts)
{
    const int nzc = T.nzc;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 4);
    Cell c;
    if (!cell_setup(L, w, blk, c, T.x0, T.y0)) return;
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
        if (B2R_EQWP_PREFETCH > 0) {
            const long long oa = ahead(L, z, B2R_EQWP_PREFETCH, w.ze),
                            oq = ahead(L, z, 2 + B2R_EQWP_PREFETCH, w.ze + 2);
            pf_l2(sxz + oq);
            pf_l2(syz + oq);
            pf_l2(szz + oq);
            pf_l2(sxx + oa);
            pf_l2(sxy + oa);
            pf_l2(syy + oa);
#pragma unroll
            for (int f = VX; f <= VZ; ++f) pf_l2(F.p[f] + c.base + oa);
            pf_l2(F.p[DISP] + c.base + oa);
        }
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
// The stage bodies are in eqwp_stag.cuh (shared with the batched kernel).
template <bool ACC>
__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
eqwp_stag_velocity(FieldPtrs F, FieldPtrs O, MatPtrs M, const BlockLayout L, int step_i, Tiles T,
                   EqwpStagParams p, AccPtrs A)
{
    const int blk = blockIdx.z / T.nzc, zc = blockIdx.z % T.nzc;
    stag_velocity_unit<ACC>(F, O, M, L, step_i, T, p, A, blk, zc, launch_pos());
}

// Tiles of a stress-stage launch that hold a cell the halo exchange reads:
// an owned cell within H of a face that has a neighbour block (H = the halo
// width; the owned cells of an axis are [H, H + B)).
__device__ __forceinline__ bool band_tile(const BlockLayout& L, int blk, const Tiles& T, const TilePos& q, int zs,
                                          int ze)
{
    const int e = edge_bits(L, blk), H = L.H;
    const int x0 = T.x0 - L.xoff + q.bx * 4 * q.dx, x1 = x0 + 4 * q.dx - 1;
    const int y0 = T.y0 + q.by * q.dy, y1 = y0 + q.dy - 1;
    const int lo[3] = {x0, y0, zs}, hi[3] = {x1, y1, ze};
    bool band = false;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        band |= (!(e & (1 << (2 * a))) && lo[a] < 2 * H) || (!(e & (2 << (2 * a))) && hi[a] >= L.B[a]);
    return band;
}

// split: 0 every tile; 1 the tiles of band_tile only; 2 the others only
__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
eqwp_stag_stress(FieldPtrs F, FieldPtrs O, MatPtrs M, const BlockLayout L, int step_i, Tiles T,
                 EqwpStagParams p, float src_amp, int split)
{
    const int blk = blockIdx.z / T.nzc, zc = blockIdx.z % T.nzc;
    const TilePos q = launch_pos();
    if (split) {
        const Win w = window(L, blk, zc, T.nzc, 4 * step_i + 4);
        if (band_tile(L, blk, T, q, w.zs, w.ze) != (split == 1)) return;
    }
    stag_stress_unit(F, O, M, L, step_i, T, p, src_amp, blk, zc, q);
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
    const Grid ga = stage_grid(L, 4 * step_i + 2), gb = stage_grid(L, 4 * step_i + 4);
    eqwp_ref_stress<<<ga.g, ga.b, 0, st>>>(F, L, step_i, ga.t, p);
    eqwp_ref_velocity<<<gb.g, gb.b, 0, st>>>(F, L, step_i, gb.t, p, ts);
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
    const Grid ga = stage_grid(L, 4 * step_i + 2), gb = stage_grid(L, 4 * step_i + 4);
    float amp = 0.f;
    if (p.src_host && ts >= 0 && ts < p.src_len) amp = p.src_host[ts];
    eqwp_stag_velocity<false><<<ga.g, ga.b, 0, st>>>(F, F, M, L, step_i, ga.t, p, AccPtrs{});
    eqwp_stag_stress<<<gb.g, gb.b, 0, st>>>(F, F, M, L, step_i, gb.t, p, amp, 0);
    count_launches(2);
    return cudaGetLastError();
}

cudaError_t launch_eqwp_stag_stress(float* const* fld, float* const* mat, const BlockLayout& L, int step_i, int ts,
                                    const EqwpStagParams& p, int split, cudaStream_t st)
{
    FieldPtrs F{};
    for (int f = 0; f < 9; ++f) F.p[f] = fld[f];
    MatPtrs M{};
    for (int m = 0; m < 3; ++m) M.p[m] = mat[m];
    const Grid gb = stage_grid(L, 4 * step_i + 4);
    float amp = 0.f;
    if (p.src_host && ts >= 0 && ts < p.src_len) amp = p.src_host[ts];
    eqwp_stag_stress<<<gb.g, gb.b, 0, st>>>(F, F, M, L, step_i, gb.t, p, amp, split);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_eqwp_stag_velocity(float* const* fld, float* const* mat, const BlockLayout& L, int step_i,
                                      const EqwpStagParams& p, cudaStream_t st)
{
    FieldPtrs F{};
    for (int f = 0; f < 9; ++f) F.p[f] = fld[f];
    MatPtrs M{};
    for (int m = 0; m < 3; ++m) M.p[m] = mat[m];
    const Grid ga = stage_grid(L, 4 * step_i + 2);
    eqwp_stag_velocity<false><<<ga.g, ga.b, 0, st>>>(F, F, M, L, step_i, ga.t, p, AccPtrs{});
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_eqwp_stag_step_replay(const float* const* v_in, float* const* s, float* const* v_out,
                                         float* const* acc, float* const* mat, const BlockLayout& L,
                                         int ts, const EqwpStagParams& p, cudaStream_t st)
{
    FieldPtrs F{}, O{};
    for (int f = 0; f < 3; ++f) {
        F.p[VX + f] = const_cast<float*>(v_in[f]);
        O.p[VX + f] = v_out[f];
    }
    for (int f = 0; f < 6; ++f) F.p[SXX + f] = O.p[SXX + f] = s[f];
    MatPtrs M{};
    for (int m = 0; m < 3; ++m) M.p[m] = mat[m];
    AccPtrs A{};
    for (int a = 0; a < 3; ++a) A.p[a] = acc[a];
    const Grid ga = stage_grid(L, 2), gb = stage_grid(L, 4);
    float amp = 0.f;
    if (p.src_host && ts >= 0 && ts < p.src_len) amp = p.src_host[ts];
    eqwp_stag_velocity<true><<<ga.g, ga.b, 0, st>>>(F, O, M, L, 0, ga.t, p, A);
    // the stress stage reads the new velocities and updates the stresses in place
    eqwp_stag_stress<<<gb.g, gb.b, 0, st>>>(O, O, M, L, 0, gb.t, p, amp, 0);
    count_launches(2);
    return cudaGetLastError();
}

}  // namespace b2r
