// heat_upd.cuh -- the folded radius-1 heat update of 4 consecutive cells,
//     u' = a0*u + ax*(u[x-1]+u[x+1]) + ay*(u[y-1]+u[y+1]) + az*(u[z-1]+u[z+1])
// (heat-3D.cu:228-231 folded as in heat.cu), in this order for every cell:
// one multiply, then three fused multiply-adds on the neighbour-pair sums.
// Cells (x, y) and (z, w) of the float4 go through the packed two-lane FP32
// instructions of sm_100 and later (__fmul2_rn, __fadd2_rn, __ffma2_rn):
// every lane is the IEEE round-to-nearest operation of the scalar form, so
// the results are bit-identical to it while the FP instructions per update
// halve, except the x-neighbour sums, whose operand pairs straddle the
// float4's register pairs (scalar adds).
#pragma once
#include "heat.h"

namespace b2r {

// c centre, l / r = the cells left of x and right of x+3, ym / yp / zm / zp
// neighbour float4s
__device__ __forceinline__ float4 heat_upd4(const HeatCoef& C, float4 c, float l, float r, float4 ym,
                                            float4 yp, float4 zm, float4 zp)
{
    const float2 a0 = make_float2(C.a0, C.a0), ax = make_float2(C.ax[0], C.ax[0]),
                 ay = make_float2(C.ay[0], C.ay[0]), az = make_float2(C.az[0], C.az[0]);
    float2 lo = __fmul2_rn(a0, make_float2(c.x, c.y));
    float2 hi = __fmul2_rn(a0, make_float2(c.z, c.w));
    lo = __ffma2_rn(ax, make_float2(l + c.y, c.x + c.z), lo);
    hi = __ffma2_rn(ax, make_float2(c.y + c.w, c.z + r), hi);
    lo = __ffma2_rn(ay, __fadd2_rn(make_float2(ym.x, ym.y), make_float2(yp.x, yp.y)), lo);
    hi = __ffma2_rn(ay, __fadd2_rn(make_float2(ym.z, ym.w), make_float2(yp.z, yp.w)), hi);
    lo = __ffma2_rn(az, __fadd2_rn(make_float2(zm.x, zm.y), make_float2(zp.x, zp.y)), lo);
    hi = __ffma2_rn(az, __fadd2_rn(make_float2(zm.z, zm.w), make_float2(zp.z, zp.w)), hi);
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

}  // namespace b2r
