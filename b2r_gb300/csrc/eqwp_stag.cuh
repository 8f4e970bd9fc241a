// eqwp_stag.cuh -- the two stage bodies of the staggered elastic-wave step
// (velocity, then stress), one work unit each: a tile of the stage launch's
// grid over one z chunk of one block.  Used by the stage kernels (eqwp.cu,
// one unit per CTA) and the batched persistent kernel (eqwp_batch.cu, units
// claimed from a work queue).
#pragma once
#include "eqwp.h"
#include "eqwp_tile.cuh"

namespace b2r {
namespace eqk {

// Both stages read every input (neighbourhoods and the old values of the
// updated fields) through F and write the updated fields through O; in place
// when O == F.  With ACC the velocity stage also stores the unscaled stencil
// sums (ax, ay, az) into A (the acceleration times rho*h), which the adjoint
// uses for the buoyancy gradient.
// NC: fields read through the read-only path (false in the persistent batch
// kernel, whose other CTAs update them between units)
template <bool ACC, bool NC = true>
__device__ __forceinline__ void stag_velocity_unit(const FieldPtrs& F, const FieldPtrs& O, const MatPtrs& M,
                                                   const BlockLayout& L, int step_i, const Tiles& T,
                                                   const EqwpStagParams& p, const AccPtrs& A, int blk, int zc,
                                                   const TilePos& q)
{
    const int nzc = T.nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 2);
    Cell c;
    if (!cell_setup(L, w, blk, c, T.x0, T.y0, q)) return;
    const long long P = L.P, S = L.plane;
    VelOpT<NC> op;
    op.xx = F.p[SXX] + c.base;
    op.xy = F.p[SXY] + c.base;
    op.xz = F.p[SXZ] + c.base;
    op.yy = F.p[SYY] + c.base;
    op.yz = F.p[SYZ] + c.base;
    op.zz = F.p[SZZ] + c.base;
    op.begin(w.zs, S);
    const float* buoy = M.p[2] + c.base;
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        if (B2R_EQWP_PREFETCH > 0) {
            const long long oa = ahead(L, z, B2R_EQWP_PREFETCH, w.ze),
                            oq = ahead(L, z, 2 + B2R_EQWP_PREFETCH, w.ze + 2);
            pf_l2(op.xz + oq);
            pf_l2(op.yz + oq);
            pf_l2(op.zz + oq);
            pf_l2(op.xx + oa);
            pf_l2(op.xy + oa);
            pf_l2(op.yy + oa);
            pf_l2(buoy + oa);
#pragma unroll
            for (int f = 0; f < 3; ++f) pf_l2(F.p[VX + f] + c.base + oa);
        }
        float a[3][4];
        op.eval(o, P, S, a[0], a[1], a[2]);
        const float4 bb = ld4(buoy + o);
        float4 old[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) old[f] = rd4(F.p[VX + f] + c.base + o, c);
        float nv[3][4];
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int j = 0; j < 4; ++j) nv[f][j] = vel_update(cmp(old[f], j), a[f][j], p.dt, p.inv_h, cmp(bb, j));
#pragma unroll
        for (int f = 0; f < 3; ++f) st4(O.p[VX + f] + c.base + o, c, nv[f]);
        if (ACC) {
#pragma unroll
            for (int f = 0; f < 3; ++f) st4(A.p[f] + c.base + o, c, a[f]);
        }
    }
}

template <bool NC = true>
__device__ __forceinline__ void stag_stress_unit(const FieldPtrs& F, const FieldPtrs& O, const MatPtrs& M,
                                                 const BlockLayout& L, int step_i, const Tiles& T,
                                                 const EqwpStagParams& p, float src_amp, int blk, int zc,
                                                 const TilePos& q)
{
    const int nzc = T.nzc;
    const Win w = window(L, blk, zc, nzc, 4 * step_i + 4);
    Cell c;
    if (!cell_setup(L, w, blk, c, T.x0, T.y0, q)) return;
    const long long P = L.P, S = L.plane;
    StrOpT<NC> op;
    op.x = F.p[VX] + c.base;
    op.y = F.p[VY] + c.base;
    op.z = F.p[VZ] + c.base;
    op.begin(w.zs, S);
    const float* lam = M.p[0] + c.base;
    const float* mu = M.p[1] + c.base;
    // source cell of this block, in block coordinates
    const int b0 = blk % L.nb[0], b1 = (blk / L.nb[0]) % L.nb[1], b2 = blk / (L.nb[0] * L.nb[1]);
    const int sx = p.src[0] - b0 * L.B[0] + L.H, sy = p.src[1] - b1 * L.B[1] + L.H,
              sz = p.src[2] - b2 * L.B[2] + L.H;
    const bool srow = (c.y == sy) && sx >= c.xb && sx < c.xb + 4;
    // updated fields in the order of stress_update: xx, yy, zz, xy, xz, yz
    static constexpr int kOut[6] = {SXX, SYY, SZZ, SXY, SXZ, SYZ};
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S;
        if (B2R_EQWP_PREFETCH > 0) {
            const long long oa = ahead(L, z, B2R_EQWP_PREFETCH, w.ze),
                            oq = ahead(L, z, 2 + B2R_EQWP_PREFETCH, w.ze + 2);
            pf_l2(op.x + oq);
            pf_l2(op.y + oq);
            pf_l2(op.z + oq);
            pf_l2(lam + oa);
            pf_l2(mu + oa);
#pragma unroll
            for (int f = 0; f < 6; ++f) pf_l2(F.p[kOut[f]] + c.base + oa);
        }
        float e[6][4];
        op.eval(o, P, S, e);
        const float4 l4 = ld4(lam + o), m4 = ld4(mu + o);
        const bool src_here = srow && z == sz;
        float4 old[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) old[f] = rd4(F.p[kOut[f]] + c.base + o, c);
        float ns[6][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const StressIn in{e[0][j], e[1][j], e[2][j], e[3][j], e[4][j], e[5][j]};
            float sv[6];
#pragma unroll
            for (int f = 0; f < 6; ++f) sv[f] = cmp(old[f], j);
            stress_update(in, p.dt, p.inv_h, cmp(l4, j), cmp(m4, j), sv);
            if (src_here && c.xb + j == sx) {
                sv[0] = __fadd_rn(sv[0], src_amp);
                sv[1] = __fadd_rn(sv[1], src_amp);
                sv[2] = __fadd_rn(sv[2], src_amp);
            }
#pragma unroll
            for (int f = 0; f < 6; ++f) ns[f][j] = sv[f];
        }
#pragma unroll
        for (int f = 0; f < 6; ++f) st4(O.p[kOut[f]] + c.base + o, c, ns[f]);
    }
}

}  // namespace eqk
}  // namespace b2r
