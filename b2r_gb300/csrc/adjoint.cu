// adjoint.cu -- hand-written discrete adjoint of the staggered elastic-wave
// time stepping (no reference counterpart) and the receiver misfit gradient
// with respect to lambda, mu and rho, with wavefield checkpointing.
//
// Forward step n (eqwp.cu STAG stage kernels), on the interior window W:
//   v'  = v + dt*b*(Dsigma)          velocity stage (Dp/Dm staggered FD4)
//   s'  = s + dt*C(lambda,mu)*E(v') + src_n   stress stage
//   d_n = vy'(receivers)
// Misfit J = 1/2 sum_n sum_r (d_n,r - obs_n,r)^2.  Reverse step n, with
// (vb, sb) the adjoints of (v', s'):
//   1. vb_y(rec) += d_n - obs_n
//   2. stress stage: q = C*sb on W (0 elsewhere);  vb += dt*E^T q;
//      g_lambda += dt*tr(E v')*tr(sb), g_mu += dt*(2 e_ii sb_ii + gamma_ij sb_ij)
//   3. velocity stage: w = b*vb on W (0 elsewhere);  sb += dt*D^T w;
//      g_b += dt*(D s)*vb on W
// with Dp^T = -Dm and Dm^T = -Dp for the 4th-order staggered differences.
// The per-step gradient increments are formed in FP32 and summed in FP32
// partial sums, which adjoint_fold adds into the FP64 gradients every
// kFoldSteps reverse steps on a fixed schedule of step numbers (so the bits
// do not depend on the checkpoint interval); a partial sum holds at most
// kFoldSteps increments.  This GPU's FP64 rate is a small fraction of its
// FP32 rate, so the products stay in FP32, and the per-step read-modify-write
// of the sums moves 4 B per gradient instead of 8.  g_rho = -g_b / rho^2 at
// the end.
#include <cstdio>
#include <vector>

#include "b2r_common.cuh"
#include "eqwp.h"
#include "eqwp_tile.cuh"

namespace b2r {
namespace {

using namespace eqk;

// L2 prefetch distance of the reverse kernels (planes; 0 = none)
#ifndef B2R_ADJ_PREFETCH
#define B2R_ADJ_PREFETCH 1
#endif

// FP32 partial gradient sums of a thread's 4 cells, loaded before and stored
// after the field stores of an iteration (16-byte aligned: the first cell of
// a thread is a multiple of 4 elements from the buffer base)
struct G4 {
    float v[4];
    __device__ __forceinline__ void load(const float* g, const Cell& c)
    {
        if (c.all) {
            const float4 a = ldw4(g);
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) v[j] = c.vx[j] ? g[j] : 0.f;
        }
    }
    __device__ __forceinline__ void store(float* g, const Cell& c) const
    {
        if (c.all) {
            *reinterpret_cast<float4*>(g) = make_float4(v[0], v[1], v[2], v[3]);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (c.vx[j]) g[j] = v[j];
        }
    }
};

// sb component (xx, xy, xz, yy, yz, zz numbering) of each strain row of StrOp
__device__ constexpr int kStrainS[6] = {0, 3, 5, 1, 2, 4};

// lambda / mu gradient increments of one cell (lane j of the thread's 4),
// explicitly rounded so that every kernel forming them gets the same bits:
//   g_lambda += k tr(e) tr(sb),  g_mu += k (2 e_ii sb_ii + gamma_ij sb_ij)
// (sb in strain-row order xx, yy, zz, xy, xz, yz; e = E v^n, raw sums)
__device__ __forceinline__ void lm_increment(float k, const float4 (&sb)[6], const float (&ev)[6][4], int j,
                                             float& gl, float& gm)
{
    const float sxx = cmp(sb[0], j), syy = cmp(sb[1], j), szz = cmp(sb[2], j);
    const float sxy = cmp(sb[3], j), sxz = cmp(sb[4], j), syz = cmp(sb[5], j);
    const float exx = ev[0][j], eyy = ev[1][j], ezz = ev[2][j];
    const float tr = add3(sxx, syy, szz);
    gl = __fadd_rn(gl, __fmul_rn(k, __fmul_rn(add3(exx, eyy, ezz), tr)));
    const float nrm = add3(__fmul_rn(exx, sxx), __fmul_rn(eyy, syy), __fmul_rn(ezz, szz));
    const float shr = add3(__fmul_rn(ev[3][j], sxy), __fmul_rn(ev[4][j], sxz), __fmul_rn(ev[5][j], syz));
    gm = __fadd_rn(gm, __fmul_rn(k, __fadd_rn(__fmul_rn(2.f, nrm), shr)));
}

struct AdjV {
    const float* q[6];     // C*sb of the later step (xx, xy, xz, yy, yz, zz)
    float* vb[3];          // adjoint velocity, updated
    float* w[3];           // b*vb on the window (out)
    const float* acc[3];   // forward stencil sums (D s^n) of this step
    const float* buoy;
    float* g_b;            // FP32 partial sums
    float k;               // dt / h
};

struct AdjS {
    const float* w[3];     // b*vb of this step
    float* sb[6];          // adjoint stress, updated (xx, xy, xz, yy, yz, zz)
    float* q[6];           // C*sb for the earlier step (out)
    const float* v[3];     // forward velocity v^n
    const float* lam;
    const float* mu;
    float* g_lam;          // FP32 partial sums
    float* g_mu;
    float k;
};

// Adjoint of the stress stage of step n followed by the velocity-stage
// weighting:  vb -= k * D q  (D^T E = -D: the transpose of the strain
// operator is minus the velocity-stage operator), then w = b * vb and
// g_b += k * (D s^n) . vb on the window.
__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
adj_velocity_kernel(AdjV A, const BlockLayout L, Tiles T)
{
    const int nzc = T.nzc;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 2);
    Cell c;
    if (!cell_setup(L, w, blk, c, T.x0, T.y0)) return;
    const long long P = L.P, S = L.plane;
    VelOp op;
    op.xx = A.q[0] + c.base;
    op.xy = A.q[1] + c.base;
    op.xz = A.q[2] + c.base;
    op.yy = A.q[3] + c.base;
    op.yz = A.q[4] + c.base;
    op.zz = A.q[5] + c.base;
    op.begin(w.zs, S);
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S + c.base;
        if (B2R_ADJ_PREFETCH > 0) {
            const long long oa = ahead(L, z, B2R_ADJ_PREFETCH, w.ze) + c.base,
                            oq = ahead(L, z, 2 + B2R_ADJ_PREFETCH, w.ze + 2);
            pf_l2(op.xz + oq);
            pf_l2(op.yz + oq);
            pf_l2(op.zz + oq);
            pf_l2(op.xx + oq - 2 * S);
            pf_l2(op.xy + oq - 2 * S);
            pf_l2(op.yy + oq - 2 * S);
            pf_l2(A.buoy + oa);
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                pf_l2(A.vb[f] + oa);
                pf_l2(A.acc[f] + oa);
            }
            pf_l2(A.g_b + oa);
        }
        float a[3][4];
        op.eval(o - c.base, P, S, a[0], a[1], a[2]);
        const float4 bb = ld4(A.buoy + o);
        float4 vb[3], ac[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            vb[f] = rd4(A.vb[f] + o, c);
            ac[f] = ld4(A.acc[f] + o);
        }
        G4 gb;
        gb.load(A.g_b + o, c);
        float d[3][4];
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int j = 0; j < 4; ++j) d[f][j] = -(A.k * a[f][j]);
#pragma unroll
        for (int f = 0; f < 3; ++f) vb[f] = wr4(A.vb[f] + o, c, vb[f], d[f]);
        float wv[3][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float b = cmp(bb, j);
            const float x = cmp(vb[0], j), y = cmp(vb[1], j), zz = cmp(vb[2], j);
            wv[0][j] = b * x;
            wv[1][j] = b * y;
            wv[2][j] = b * zz;
            gb.v[j] = __fadd_rn(gb.v[j], A.k * (cmp(ac[0], j) * x + cmp(ac[1], j) * y + cmp(ac[2], j) * zz));
        }
#pragma unroll
        for (int f = 0; f < 3; ++f) st4(A.w[f] + o, c, wv[f]);
        gb.store(A.g_b + o, c);
    }
}

// Adjoint of the velocity stage of step n followed by the stress weighting
// of step n-1:  sb -= k * E w  (D^T = -E), then q = C(lambda, mu) * sb on
// the window.
__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
adj_stress_kernel(AdjS A, const BlockLayout L, Tiles T)
{
    const int nzc = T.nzc;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4);
    Cell c;
    if (!cell_setup(L, w, blk, c, T.x0, T.y0)) return;
    const long long P = L.P, S = L.plane;
    StrOp ow;
    ow.x = A.w[0] + c.base;
    ow.y = A.w[1] + c.base;
    ow.z = A.w[2] + c.base;
    ow.begin(w.zs, S);
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S + c.base;
        if (B2R_ADJ_PREFETCH > 0) {
            const long long oa = ahead(L, z, B2R_ADJ_PREFETCH, w.ze) + c.base,
                            oq = ahead(L, z, 2 + B2R_ADJ_PREFETCH, w.ze + 2);
            pf_l2(ow.x + oq);
            pf_l2(ow.y + oq);
            pf_l2(ow.z + oq);
            pf_l2(A.lam + oa);
            pf_l2(A.mu + oa);
#pragma unroll
            for (int f = 0; f < 6; ++f) pf_l2(A.sb[f] + oa);
        }
        float ew[6][4];
        ow.eval(o - c.base, P, S, ew);
        const float4 l4 = ld4(A.lam + o), m4 = ld4(A.mu + o);
        float4 sb[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) sb[f] = rd4(A.sb[kStrainS[f]] + o, c);
        float d[6][4];
#pragma unroll
        for (int f = 0; f < 6; ++f)
#pragma unroll
            for (int j = 0; j < 4; ++j) d[f][j] = -(A.k * ew[f][j]);
#pragma unroll
        for (int f = 0; f < 6; ++f) sb[f] = wr4(A.sb[kStrainS[f]] + o, c, sb[f], d[f]);
        float qv[6][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float l = cmp(l4, j), m = cmp(m4, j);
            const float sxx = cmp(sb[0], j), syy = cmp(sb[1], j), szz = cmp(sb[2], j);
            const float tr = sxx + syy + szz;
            qv[0][j] = 2.f * m * sxx + l * tr;
            qv[1][j] = 2.f * m * syy + l * tr;
            qv[2][j] = 2.f * m * szz + l * tr;
            qv[3][j] = m * cmp(sb[3], j);
            qv[4][j] = m * cmp(sb[4], j);
            qv[5][j] = m * cmp(sb[5], j);
        }
#pragma unroll
        for (int f = 0; f < 6; ++f) st4(A.q[kStrainS[f]] + o, c, qv[f]);
    }
}

// lambda / mu gradients of the stress stage of step n-1 on the window:
// g_lambda += k * tr(E v^n) tr(sb),  g_mu += k * (2 e_ii sb_ii + gamma_ij sb_ij)
__global__ void __launch_bounds__(kBX * kBY, B2R_EQWP_MINB)
adj_grad_lm_kernel(AdjS A, const BlockLayout L, Tiles T)
{
    const int nzc = T.nzc;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4);
    Cell c;
    if (!cell_setup(L, w, blk, c, T.x0, T.y0)) return;
    const long long P = L.P, S = L.plane;
    StrOp ov;
    ov.x = A.v[0] + c.base;
    ov.y = A.v[1] + c.base;
    ov.z = A.v[2] + c.base;
    ov.begin(w.zs, S);
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S + c.base;
        if (B2R_ADJ_PREFETCH > 0) {
            const long long oa = ahead(L, z, B2R_ADJ_PREFETCH, w.ze) + c.base,
                            oq = ahead(L, z, 2 + B2R_ADJ_PREFETCH, w.ze + 2);
            pf_l2(ov.x + oq);
            pf_l2(ov.y + oq);
            pf_l2(ov.z + oq);
#pragma unroll
            for (int f = 0; f < 6; ++f) pf_l2(A.sb[f] + oa);
            pf_l2(A.g_lam + oa);
            pf_l2(A.g_mu + oa);
        }
        float ev[6][4];
        ov.eval(o - c.base, P, S, ev);
        float4 sb[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) sb[f] = ld4(A.sb[kStrainS[f]] + o);
        G4 gl, gm;
        gl.load(A.g_lam + o, c);
        gm.load(A.g_mu + o, c);
#pragma unroll
        for (int j = 0; j < 4; ++j) lm_increment(A.k, sb, ev, j, gl.v[j], gm.v[j]);
        gl.store(A.g_lam + o, c);
        gm.store(A.g_mu + o, c);
    }
}

// adj_stress_kernel and adj_grad_lm_kernel in one sweep: the updated sb
// stays in registers for the lambda / mu gradients instead of being re-read
// (68 + 92 -> 136 B per cell).  Two strain operators (w and v^n) are live,
// so the register budget is fitted to one CTA per SM unless
// B2R_ADJ_FUSED_MINB says otherwise.
#ifndef B2R_ADJ_FUSED_MINB
#define B2R_ADJ_FUSED_MINB 1
#endif
__global__ void __launch_bounds__(kBX * kBY, B2R_ADJ_FUSED_MINB)
adj_stress_lm_kernel(AdjS A, const BlockLayout L, Tiles T)
{
    const int nzc = T.nzc;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const Win w = window(L, blk, zc, nzc, 4);
    Cell c;
    if (!cell_setup(L, w, blk, c, T.x0, T.y0)) return;
    const long long P = L.P, S = L.plane;
    StrOp ow, ov;
    ow.x = A.w[0] + c.base;
    ow.y = A.w[1] + c.base;
    ow.z = A.w[2] + c.base;
    ov.x = A.v[0] + c.base;
    ov.y = A.v[1] + c.base;
    ov.z = A.v[2] + c.base;
    ow.begin(w.zs, S);
    ov.begin(w.zs, S);
    for (int z = w.zs; z <= w.ze; ++z) {
        const long long o = (long long)z * S + c.base;
        if (B2R_ADJ_PREFETCH > 0) {
            const long long oa = ahead(L, z, B2R_ADJ_PREFETCH, w.ze) + c.base,
                            oq = ahead(L, z, 2 + B2R_ADJ_PREFETCH, w.ze + 2);
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                pf_l2(A.w[f] + c.base + oq);
                pf_l2(A.v[f] + c.base + oq);
            }
            pf_l2(A.lam + oa);
            pf_l2(A.mu + oa);
#pragma unroll
            for (int f = 0; f < 6; ++f) pf_l2(A.sb[f] + oa);
            pf_l2(A.g_lam + oa);
            pf_l2(A.g_mu + oa);
        }
        float ew[6][4];
        ow.eval(o - c.base, P, S, ew);
        const float4 l4 = ld4(A.lam + o), m4 = ld4(A.mu + o);
        float4 sb[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) sb[f] = rd4(A.sb[kStrainS[f]] + o, c);
        float d[6][4];
#pragma unroll
        for (int f = 0; f < 6; ++f)
#pragma unroll
            for (int j = 0; j < 4; ++j) d[f][j] = -(A.k * ew[f][j]);
#pragma unroll
        for (int f = 0; f < 6; ++f) sb[f] = wr4(A.sb[kStrainS[f]] + o, c, sb[f], d[f]);
        float qv[6][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float l = cmp(l4, j), m = cmp(m4, j);
            const float sxx = cmp(sb[0], j), syy = cmp(sb[1], j), szz = cmp(sb[2], j);
            const float tr = sxx + syy + szz;
            qv[0][j] = 2.f * m * sxx + l * tr;
            qv[1][j] = 2.f * m * syy + l * tr;
            qv[2][j] = 2.f * m * szz + l * tr;
            qv[3][j] = m * cmp(sb[3], j);
            qv[4][j] = m * cmp(sb[4], j);
            qv[5][j] = m * cmp(sb[5], j);
        }
#pragma unroll
        for (int f = 0; f < 6; ++f) st4(A.q[kStrainS[f]] + o, c, qv[f]);
        // lambda / mu gradients of the stress stage of step n-1 from the sb
        // just stored, exactly as adj_grad_lm_kernel forms them
        float ev[6][4];
        ov.eval(o - c.base, P, S, ev);
        G4 gl, gm;
        gl.load(A.g_lam + o, c);
        gm.load(A.g_mu + o, c);
#pragma unroll
        for (int j = 0; j < 4; ++j) lm_increment(A.k, sb, ev, j, gl.v[j], gm.v[j]);
        gl.store(A.g_lam + o, c);
        gm.store(A.g_mu + o, c);
    }
}

__global__ void rec_sample_kernel(const float* vy, const long long* idx, int nrec, float* out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrec) out[r] = vy[idx[r]];
}

__global__ void rec_inject_kernel(float* vby, const long long* idx, int nrec, const float* res)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrec) atomicAdd(&vby[idx[r]], res[r]);
}

// g_rho = -g_b * b^2 ; copy interior gradients out (x fastest, env cells)
__global__ void grad_out_kernel(const double* g, const float* buoy, int rho, const BlockLayout L,
                                double* out)
{
    const long long total = (long long)L.B[0] * L.B[1] * L.B[2];
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(e % L.B[0]);
        const long long r = e / L.B[0];
        const int y = (int)(r % L.B[1]);
        const int z = (int)(r / L.B[1]);
        const long long id = (long long)(z + L.H) * L.plane + (long long)(y + L.H) * L.P + L.xoff + x + L.H;
        double v = g[id];
        if (rho) {
            const double b = buoy[id];
            v = -v * b * b;
        }
        out[e] = v;
    }
}

inline int grid_for(long long work)
{
    long long g = (work + 255) / 256;
    if (g > 152LL * 16) g = 152LL * 16;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

// ---------------------------------------------------------------- driver

cudaError_t adjoint_sample(const float* vy, const long long* d_idx, int nrec, float* out, cudaStream_t st)
{
    rec_sample_kernel<<<(nrec + 127) / 128, 128, 0, st>>>(vy, d_idx, nrec, out);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t adjoint_inject(float* vby, const long long* d_idx, int nrec, const float* res, cudaStream_t st)
{
    rec_inject_kernel<<<(nrec + 127) / 128, 128, 0, st>>>(vby, d_idx, nrec, res);
    count_launches(1);
    return cudaGetLastError();
}

// Reverse step n: q (from the later step) -> vb, w, g_b; then, unless n is
// the first step, w -> sb, q for step n-1, g_lambda, g_mu (one sweep when
// fused, else the stress kernel and the gradient kernel).  tmp = vb[3],
// sb[6], q[6], w[3]; v_n = forward v^n, acc_n = forward D s^n.
cudaError_t adjoint_step(float* const* tmp, const float* const* v_n, const float* const* acc_n,
                         const float* const* mat, float* const* g, const BlockLayout& L, float dt_h,
                         bool last, bool fused, cudaStream_t st)
{
    AdjV V;
    AdjS T;
    for (int k = 0; k < 3; ++k) {
        V.vb[k] = tmp[k];
        V.w[k] = tmp[15 + k];
        V.acc[k] = acc_n[k];
        T.w[k] = tmp[15 + k];
        T.v[k] = v_n[k];
    }
    for (int k = 0; k < 6; ++k) {
        V.q[k] = tmp[9 + k];
        T.sb[k] = tmp[3 + k];
        T.q[k] = tmp[9 + k];
    }
    V.buoy = mat[2];
    V.g_b = g[2];
    V.k = dt_h;
    T.lam = mat[0];
    T.mu = mat[1];
    T.g_lam = g[0];
    T.g_mu = g[1];
    T.k = dt_h;
    const Grid ga = stage_grid(L, 2), gb = stage_grid(L, 4);
    adj_velocity_kernel<<<ga.g, ga.b, 0, st>>>(V, L, ga.t);
    count_launches(1);
    if (!last) {
        if (fused) {
            adj_stress_lm_kernel<<<gb.g, gb.b, 0, st>>>(T, L, gb.t);
            count_launches(1);
        } else {
            adj_stress_kernel<<<gb.g, gb.b, 0, st>>>(T, L, gb.t);
            adj_grad_lm_kernel<<<gb.g, gb.b, 0, st>>>(T, L, gb.t);
            count_launches(2);
        }
    }
    return cudaGetLastError();
}

namespace {
constexpr int kFoldSteps = 32;    // reverse steps per FP32 partial sum

__global__ void adjoint_fold_kernel(float* g0, float* g1, float* g2, double* h0, double* h1, double* h2,
                                    long long n4)
{
    float* g[3] = {g0, g1, g2};
    double* h[3] = {h0, h1, h2};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            float4* gp = reinterpret_cast<float4*>(g[m]) + i;
            double2* hp = reinterpret_cast<double2*>(h[m]) + 2 * i;
            const float4 a = *gp;
            const double2 b0 = hp[0], b1 = hp[1];
            hp[0] = make_double2(b0.x + (double)a.x, b0.y + (double)a.y);
            hp[1] = make_double2(b1.x + (double)a.z, b1.y + (double)a.w);
            *gp = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}
}  // namespace

int adjoint_fold_steps() { return kFoldSteps; }

cudaError_t adjoint_fold(float* const* g, double* const* g64, const BlockLayout& L, cudaStream_t st)
{
    const long long n4 = L.bstride * L.nblk / 4;   // bstride is a multiple of 4 cells (rows of 32)
    const long long blocks = std::min<long long>((n4 + 255) / 256, 152LL * 16);
    adjoint_fold_kernel<<<(unsigned)std::max(1LL, blocks), 256, 0, st>>>(g[0], g[1], g[2], g64[0], g64[1], g64[2], n4);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t adjoint_grad_out(const double* g, const float* buoy, int rho, const BlockLayout& L,
                             double* out, cudaStream_t st)
{
    grad_out_kernel<<<grid_for((long long)L.B[0] * L.B[1] * L.B[2]), 256, 0, st>>>(g, buoy, rho, L, out);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace b2r
