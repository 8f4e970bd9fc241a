// eqwp_fused.cu -- the staggered elastic-wave time step in one HBM pass.
//
// The two-stage form (eqwp.cu) streams the fields twice per step: the
// velocity stage reads the stresses and rewrites the velocities, then the
// stress stage reads the new velocities and rewrites the stresses (120 B per
// cell).  Here one CTA does both stages for its tile while marching z, so a
// step moves each field once: 9 fields read + 9 written + 3 material fields
// read = 84 B per cell.
//
// CTA = 32 x 16 threads; thread (c, r) owns the columns (c, r) and
// (c, r + 16) of a 32 x 32 velocity region: the 28 x 28 tile it owns plus a
// 2-cell ring, whose new velocities are recomputed here (the neighbouring
// tiles compute them too, from the same inputs, so they agree bit for bit).
//   * stresses s^n: TMA boxes of 36 x 36 cells (tile + 4-cell ring) per
//     field and plane into a ring of kSlots planes in shared memory, issued
//     one plane ahead of use; x / y neighbours and z neighbours of the
//     thread's own column are all read from that ring;
//   * new velocities v^{n+1}: each thread keeps its own columns' last five
//     planes in registers (z neighbours) and publishes plane q to a double
//     buffer in shared memory for the x / y neighbours of the stress stage;
//   * iteration j computes the velocity at plane p = zs - 2 + j and the
//     stresses at plane q = p - 2, whose velocity z neighbours (q-2 .. q+2)
//     are then complete.
// The step is out of place (v^n, s^n -> v^{n+1}, s^{n+1}): a tile reads its
// neighbours' old values, which an in-place update would overwrite.  Every
// operation is the explicitly rounded one of the two-stage kernels, so both
// forms and the FP32 oracle agree bit for bit.
#include "b2r_common.cuh"
#include "eqwp.h"
#include "eqwp_tile.cuh"

namespace b2r {

namespace {

using namespace eqk;

constexpr int kOwn = 28;                    // owned tile edge (cells)
constexpr int kVR = kOwn + 4;               // velocity region edge = 32
constexpr int kSB = kOwn + 8;               // staged stress box edge = 36
constexpr int kSlots = 6;                   // stress planes resident
constexpr int kPlanePad = 1312;             // 36*36 = 1296 floats padded to 128-byte multiples
constexpr int kRows = 16;                   // thread rows; each thread has rows r and r + 16
constexpr int kFThreads = 32 * kRows;
constexpr uint32_t kSlotBytes = 6u * kSB * kSB * 4u;   // TMA bytes per staged plane
constexpr size_t kSmemS = (size_t)kSlots * 6 * kPlanePad * 4;
constexpr size_t kSmemV = (size_t)2 * 3 * kVR * kVR * 4;
constexpr size_t kFusedSmem = 128 + kSmemS + kSmemV + kSlots * 8;

// shared-memory field order of a staged plane: xx, xy, xz, yy, yz, zz
enum { QXX, QXY, QXZ, QYY, QYZ, QZZ };

struct FusedArgs {
    const float* vin[3];
    float* vout[3];
    float* sout[6];        // xx, xy, xz, yy, yz, zz
    const float* lam;
    const float* mu;
    const float* buoy;
    float dt, ih, src_amp;
    int src[3];            // source cell, global interior coordinates
    int* status;
};

__device__ __forceinline__ const float* splane(const float* sS, int t, int f)
{
    return sS + ((t % kSlots) * 6 + f) * kPlanePad;
}

__global__ void __launch_bounds__(kFThreads, 1)
eqwp_stag_fused(const __grid_constant__ StressMaps maps, FusedArgs A, const BlockLayout L, int step_i,
                Tiles T)
{
    extern __shared__ unsigned char smem_raw[];
    float* sS = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float* sV = sS + kSlots * 6 * kPlanePad;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sV + 2 * 3 * kVR * kVR);
    __shared__ int s_abort;

    const int nzc = T.nzc;
    const int blk = blockIdx.z / nzc, zc = blockIdx.z % nzc;
    const int edge = edge_bits(L, blk);
    int vlo[3], vhi[3], slo[3], shi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        stage_region(L, edge, a, 4 * step_i + 2, vlo[a], vhi[a]);
        stage_region(L, edge, a, 4 * step_i + 4, slo[a], shi[a]);
    }
    const int nzv = vhi[2] - vlo[2] + 1;
    const int per = (nzv + nzc - 1) / nzc;
    const int zs = vlo[2] + zc * per, ze = min(vhi[2], zs + per - 1);
    const int x0 = T.x0 - L.xoff + blockIdx.x * kOwn;    // block x of the tile's first cell
    const int y0 = T.y0 + blockIdx.y * kOwn;
    // uniform per CTA: nothing of this tile lies in the velocity window
    if (nzv <= 0 || zs > ze || x0 > vhi[0] || x0 + kOwn - 1 < vlo[0] || y0 > vhi[1] ||
        y0 + kOwn - 1 < vlo[1])
        return;

    const int tid = threadIdx.x, c = tid & 31, r0 = tid >> 5;
    const long long P = L.P, S = L.plane;
    const long long bbase = (long long)blk * L.bstride + L.xoff;

    // per-column state: column k has velocity-region row r0 + 16 k
    int cy[2];
    bool ok[2], inV[2], own[2], inS[2];
    long long cidx[2];    // element offset of (x, y, 0)
    const int x = x0 - 2 + c;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int r = r0 + kRows * k;
        cy[k] = y0 - 2 + r;
        ok[k] = x >= 0 && x < L.n[0] && cy[k] >= 0 && cy[k] < L.n[1];
        inV[k] = ok[k] && x >= vlo[0] && x <= vhi[0] && cy[k] >= vlo[1] && cy[k] <= vhi[1];
        own[k] = c >= 2 && c < kVR - 2 && r >= 2 && r < kVR - 2;
        inS[k] = own[k] && ok[k] && x >= slo[0] && x <= shi[0] && cy[k] >= slo[1] && cy[k] <= shi[1];
        cidx[k] = bbase + (long long)cy[k] * P + x;
    }
    // source cell in block coordinates
    const int b0 = blk % L.nb[0], b1 = (blk / L.nb[0]) % L.nb[1], b2 = blk / (L.nb[0] * L.nb[1]);
    const int sxs = A.src[0] - b0 * L.B[0] + L.H, sys = A.src[1] - b1 * L.B[1] + L.H,
              szs = A.src[2] - b2 * L.B[2] + L.H;

    // staged planes t = 0 .. tlast are the planes zs - 4 + t
    const int tlast = ze - zs + 8;
    const int bx_tma = L.xoff + x0 - 4, by_tma = y0 - 4;
    if (tid == 0) {
        s_abort = 0;
        for (int i = 0; i < kSlots; ++i) mbar_init(&bar[i], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0)
        for (int t = 0; t <= 4; ++t) {
            mbar_expect_tx(&bar[t % kSlots], kSlotBytes);
            for (int f = 0; f < 6; ++f)
                tma_load_4d(const_cast<float*>(splane(sS, t, f)), &maps.m[f], bx_tma, by_tma, zs - 4 + t, blk,
                            &bar[t % kSlots]);
        }
    int issued = 5;       // staged planes issued so far (thread 0)

    float qx[2][5], qy[2][5], qz[2][5];   // new velocity of planes p-4 .. p (index 4 = p)
    float pv[2][3], pb[2], pl[2], pm[2];  // prefetched v^n, b of plane p; lambda, mu of plane q
#pragma unroll
    for (int k = 0; k < 2; ++k) {
#pragma unroll
        for (int i = 0; i < 5; ++i) qx[k][i] = qy[k][i] = qz[k][i] = 0.f;
        const long long o = cidx[k] + (long long)(zs - 2) * S;
#pragma unroll
        for (int f = 0; f < 3; ++f) pv[k][f] = ok[k] ? __ldg(A.vin[f] + o) : 0.f;
        pb[k] = ok[k] ? __ldg(A.buoy + o) : 0.f;
        pl[k] = pm[k] = 0.f;
    }

    const int njt = ze - zs + 5;    // iterations: p = zs - 2 .. ze + 2
    bool aborted = false;
    for (int j = 0; j < njt; ++j) {
        const int p = zs - 2 + j, q = p - 2;
        __syncthreads();
        if (s_abort) {
            aborted = true;
            break;
        }
        // refill the slot of plane t = j - 1, which iteration j - 1 was the last to read
        if (tid == 0 && issued <= tlast) {
            const int t = issued++;
            mbar_expect_tx(&bar[t % kSlots], kSlotBytes);
            for (int f = 0; f < 6; ++f)
                tma_load_4d(const_cast<float*>(splane(sS, t, f)), &maps.m[f], bx_tma, by_tma, zs - 4 + t, blk,
                            &bar[t % kSlots]);
        }
        // planes j .. j + 4 (p - 2 .. p + 2) must have landed
        {
            const int t0 = j == 0 ? 0 : j + 4;
            for (int t = t0; t <= j + 4; ++t)
                if (!mbar_wait_bounded(&bar[t % kSlots], (t / kSlots) & 1)) {
                    s_abort = 1;
                    report(A.status, DEV_TIMEOUT);
                }
        }
        // ---- velocity at plane p on the 32 x 32 region
        const bool pin = p >= vlo[2] && p <= vhi[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int bxs = c + 2, bys = r0 + kRows * k + 2;     // staged-box coordinates
            float nv[3] = {pv[k][0], pv[k][1], pv[k][2]};
            if (pin && inV[k]) {
                const float* xx = splane(sS, j + 2, QXX) + bys * kSB + bxs;
                const float* xy = splane(sS, j + 2, QXY) + bys * kSB + bxs;
                const float* xz = splane(sS, j + 2, QXZ) + bys * kSB + bxs;
                const float* yy = splane(sS, j + 2, QYY) + bys * kSB + bxs;
                const float* yz = splane(sS, j + 2, QYZ) + bys * kSB + bxs;
                const int o = bys * kSB + bxs;
                // own column, planes p-2 .. p+2 (t = j .. j+4)
                const float xzm2 = splane(sS, j, QXZ)[o], xzm1 = splane(sS, j + 1, QXZ)[o],
                            xzp1 = splane(sS, j + 3, QXZ)[o];
                const float yzm2 = splane(sS, j, QYZ)[o], yzm1 = splane(sS, j + 1, QYZ)[o],
                            yzp1 = splane(sS, j + 3, QYZ)[o];
                const float zzm1 = splane(sS, j + 1, QZZ)[o], zzc = splane(sS, j + 2, QZZ)[o],
                            zzp1 = splane(sS, j + 3, QZZ)[o], zzp2 = splane(sS, j + 4, QZZ)[o];
                const float ax = add3(sdiff(xx[1], xx[0], xx[2], xx[-1]),
                                      sdiff(xy[0], xy[-kSB], xy[kSB], xy[-2 * kSB]),
                                      sdiff(xz[0], xzm1, xzp1, xzm2));
                const float ay = add3(sdiff(xy[0], xy[-1], xy[1], xy[-2]),
                                      sdiff(yy[kSB], yy[0], yy[2 * kSB], yy[-kSB]),
                                      sdiff(yz[0], yzm1, yzp1, yzm2));
                const float az = add3(sdiff(xz[0], xz[-1], xz[1], xz[-2]),
                                      sdiff(yz[0], yz[-kSB], yz[kSB], yz[-2 * kSB]),
                                      sdiff(zzp1, zzc, zzp2, zzm1));
                nv[0] = vel_update(nv[0], ax, A.dt, A.ih, pb[k]);
                nv[1] = vel_update(nv[1], ay, A.dt, A.ih, pb[k]);
                nv[2] = vel_update(nv[2], az, A.dt, A.ih, pb[k]);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                qx[k][i] = qx[k][i + 1];
                qy[k][i] = qy[k][i + 1];
                qz[k][i] = qz[k][i + 1];
            }
            qx[k][4] = nv[0];
            qy[k][4] = nv[1];
            qz[k][4] = nv[2];
            if (pin && own[k] && inV[k] && p >= zs && p <= ze) {
                const long long o = cidx[k] + (long long)p * S;
                A.vout[0][o] = nv[0];
                A.vout[1][o] = nv[1];
                A.vout[2][o] = nv[2];
            }
        }
        // ---- stresses at plane q = p - 2 on the owned tile
        if (j >= 4 && q >= slo[2] && q <= shi[2]) {
            const float* vb = sV + (j & 1) * 3 * kVR * kVR;
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (!inS[k]) continue;
                const int r = r0 + kRows * k;
                const float* vx = vb + r * kVR + c;
                const float* vy = vx + kVR * kVR;
                const float* vz = vy + kVR * kVR;
                // queue index i holds plane p - 4 + i: q = index 2
                StressIn e;
                e.exx = sdiff(vx[0], vx[-1], vx[1], vx[-2]);
                e.eyy = sdiff(vy[0], vy[-kVR], vy[kVR], vy[-2 * kVR]);
                e.ezz = sdiff(qz[k][2], qz[k][1], qz[k][3], qz[k][0]);
                e.gxy = __fadd_rn(sdiff(vx[kVR], vx[0], vx[2 * kVR], vx[-kVR]), sdiff(vy[1], vy[0], vy[2], vy[-1]));
                e.gxz = __fadd_rn(sdiff(qx[k][3], qx[k][2], qx[k][4], qx[k][1]), sdiff(vz[1], vz[0], vz[2], vz[-1]));
                e.gyz = __fadd_rn(sdiff(qy[k][3], qy[k][2], qy[k][4], qy[k][1]),
                                  sdiff(vz[kVR], vz[0], vz[2 * kVR], vz[-kVR]));
                const int o = (r + 2) * kSB + c + 2;
                float sv[6] = {splane(sS, j, QXX)[o], splane(sS, j, QYY)[o], splane(sS, j, QZZ)[o],
                               splane(sS, j, QXY)[o], splane(sS, j, QXZ)[o], splane(sS, j, QYZ)[o]};
                stress_update(e, A.dt, A.ih, pl[k], pm[k], sv);
                if (x == sxs && cy[k] == sys && q == szs) {
                    sv[0] = __fadd_rn(sv[0], A.src_amp);
                    sv[1] = __fadd_rn(sv[1], A.src_amp);
                    sv[2] = __fadd_rn(sv[2], A.src_amp);
                }
                const long long g = cidx[k] + (long long)q * S;
                A.sout[QXX][g] = sv[0];
                A.sout[QYY][g] = sv[1];
                A.sout[QZZ][g] = sv[2];
                A.sout[QXY][g] = sv[3];
                A.sout[QXZ][g] = sv[4];
                A.sout[QYZ][g] = sv[5];
            }
        }
        // ---- publish v(p - 1) for the next iteration's stresses (plane q + 1)
        {
            float* vn = sV + ((j + 1) & 1) * 3 * kVR * kVR;
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int i = (r0 + kRows * k) * kVR + c;
                vn[i] = qx[k][3];
                vn[kVR * kVR + i] = qy[k][3];
                vn[2 * kVR * kVR + i] = qz[k][3];
            }
        }
        // ---- prefetch v^n, b of plane p + 1 and lambda, mu of plane q + 1
        if (j + 1 < njt) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (ok[k]) {
                    const long long o = cidx[k] + (long long)(p + 1) * S;
#pragma unroll
                    for (int f = 0; f < 3; ++f) pv[k][f] = __ldg(A.vin[f] + o);
                    pb[k] = __ldg(A.buoy + o);
                }
                if (inS[k] && q + 1 >= zs) {
                    const long long o = cidx[k] + (long long)(q + 1) * S;
                    pl[k] = __ldg(A.lam + o);
                    pm[k] = __ldg(A.mu + o);
                }
            }
        }
    }
    // no TMA may still be writing this CTA's shared memory when it exits
    __syncthreads();
    if ((aborted || s_abort) && tid == 0)
        for (int t = 0; t < issued; ++t) mbar_wait_bounded(&bar[t % kSlots], (t / kSlots) & 1, 100000000ull);
}

}  // namespace

size_t eqwp_fused_smem() { return kFusedSmem; }
int eqwp_fused_box() { return kSB; }

cudaError_t launch_eqwp_stag_fused(const StressMaps& maps, const float* const* vin, float* const* vout,
                                   float* const* sout, float* const* mat, const BlockLayout& L, int step_i,
                                   int ts, const EqwpStagParams& p, int* status, cudaStream_t st)
{
    static KernelSetup setup;
    if (cudaError_t e = kernel_setup(setup, eqwp_stag_fused, kFThreads, kFusedSmem, nullptr, nullptr)) return e;
    FusedArgs A{};
    for (int f = 0; f < 3; ++f) {
        A.vin[f] = vin[f];
        A.vout[f] = vout[f];
    }
    for (int f = 0; f < 6; ++f) A.sout[f] = sout[f];
    A.lam = mat[0];
    A.mu = mat[1];
    A.buoy = mat[2];
    A.dt = p.dt;
    A.ih = p.inv_h;
    A.src_amp = (p.src_host && ts >= 0 && ts < p.src_len) ? p.src_host[ts] : 0.f;
    for (int a = 0; a < 3; ++a) A.src[a] = p.src[a];
    A.status = status;
    // tiles over the union of the blocks' velocity windows; the first tile's
    // staged box starts on a 16-byte boundary
    const int shrink = 4 * step_i + 2;
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
    Tiles T{};
    T.x0 = (L.xoff + lo[0]) & ~3;
    T.y0 = lo[1];
    const int tx = std::max(1, (L.xoff + hi[0] + 1 - T.x0 + kOwn - 1) / kOwn);
    const int ty = std::max(1, (hi[1] + 1 - lo[1] + kOwn - 1) / kOwn);
    const long long tiles = (long long)tx * ty * L.nblk;
    const int nz = std::max(1, hi[2] - lo[2] + 1);
    // z chunks: fewest waves of one CTA per SM, each weighted by its chunk
    // length plus the four planes of warm-up
    int best = 1;
    double best_cost = 1e300;
    for (int nzc = 1; nzc <= std::max(1, nz / 16); ++nzc) {
        const long long ctas = tiles * nzc;
        const double waves = (double)((ctas + 151) / 152);
        const double cost = waves * ((nz + nzc - 1) / nzc + 4);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = nzc;
        }
    }
    T.nzc = best;
    const dim3 grid(tx, ty, L.nblk * best);
    eqwp_stag_fused<<<grid, kFThreads, kFusedSmem, st>>>(maps, A, L, step_i, T);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace b2r
