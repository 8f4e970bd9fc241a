// heat.cu -- explicit 3-D heat diffusion, stencil radius D = 1..4.
//
// Replaces fdm_heat_diffuse_delta1..4 (heat-3D.cu:173-521) and the
// edge-freezing fdm_heat_diffuse_delta1_verify (heat-3D.cu:57-158).  Scheme
// (heat-3D.cu:228-231, 315-318, 410-413, 514-517):
//     u' = u + alpha_dt * (Lx/dx^2 + Ly/dy^2 + Lz/dz^2)
// with the order-2D central second differences L of heat-3D.cu:15-28, folded
// here into   u' = a0*u + sum_k [ax_k (u[x-k]+u[x+k]) + ay_k (..y..) + az_k (..z..)].
//
// Kernel shape: 2.5-D sweep.  A CTA owns a 128 x TY tile of one block in xy
// (lane = 4 consecutive x cells, warp = RY rows) and a chunk of z planes.
// Every input plane of the tile plus a D-row / 4-column skirt arrives in
// shared memory by one TMA load into an S-deep ring (mbarrier completion);
// each thread keeps its 2D+1 planes of float4 in a register queue along z
// and reads the xy neighbours of the current plane from shared memory.
// One HBM read and one write per cell and sub-step; the skirt re-reads hit L2.
#include <cstdio>

#include "heat_unit.cuh"

namespace b2r {

namespace {

using heatk::kThreads;
using heatk::kTX;
using heatk::kWarps;

// Work schedule of one launch: units = (block, z-chunk of Lz output planes,
// tile row, tile column) numbered with the tile column fastest, dealt
// round-robin to gridDim.x CTAs.  Units that run at the same time are
// neighbouring tiles of the same planes, so whole DRAM rows are fetched
// together and the tile skirts hit L2.  gridDim.x = number of units gives one
// unit per CTA; a smaller grid makes the CTAs persistent.
struct HeatSched {
    int ntx, nty;            // tile columns / rows per block
    int NZ, Lz, nzc;         // output planes per column, planes per chunk, chunks
    long long U;             // units
};

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }

// rows per warp of the delta-4 sweep (2 for the other radii)
#ifndef B2R_HEAT4_RY
#define B2R_HEAT4_RY 2
#endif

// resident CTAs per SM the register budget is fitted to, by stencil radius
#ifndef B2R_HEAT4_MINB
#define B2R_HEAT4_MINB 2
#endif
template <int D>
struct MinBlocks {
    static constexpr int value = D == 1 ? 5 : (D == 2 ? 3 : (D == 3 ? 2 : B2R_HEAT4_MINB));
};

template <int D, int RY, int S>
__global__ void __launch_bounds__(kThreads, MinBlocks<D>::value)
heat_sweep_kernel(const __grid_constant__ CUtensorMap tin, float* __restrict__ out,
                  const BlockLayout L, const int step_i, const HeatCoef C, const HeatSched sch,
                  int* __restrict__ status)
{
    using Cfg = heatk::Cfg<D, RY, S>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    heatk::Ring rg;
    heatk::ring_init<S, Cfg::SLOT>(rg, smem_raw);
    // the input was written by the previous launch on this stream
    pdl_wait();
    pdl_trigger();
    for (long long u = blockIdx.x; u < sch.U; u += gridDim.x) {
        const int tx = (int)(u % sch.ntx);
        long long r = u / sch.ntx;
        const int ty = (int)(r % sch.nty);
        r /= sch.nty;
        const int zc = (int)(r % sch.nzc);
        const int blk = (int)(r / sch.nzc);
        const int zi0 = zc * sch.Lz;
        const int zi1 = min(sch.NZ, zi0 + sch.Lz);
        if (!heatk::sweep_unit<D, RY, S, Cfg::SLOT>(&tin, out, L, step_i, C, blk, tx, ty, zi0, zi1, rg)) {
            if (threadIdx.x == 0) report(status, DEV_TIMEOUT);
            heatk::ring_drain<S>(rg);
            return;
        }
    }
}

template <int D, int RY, int S>
cudaError_t launch_t(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                     const HeatCoef& c, int* status, cudaStream_t st, const HeatTune& tune)
{
    using Cfg = heatk::Cfg<D, RY, S>;
    auto kern = heat_sweep_kernel<D, RY, S>;
    static KernelSetup setup;
    int resident = 0, resident_per_sm = 0;    // CTAs resident per SM / on the whole GPU
    if (cudaError_t e = kernel_setup(setup, kern, kThreads, Cfg::SMEM, &resident_per_sm, &resident))
        return e;
    HeatSched sch;
    const int xs_begin = (L.xoff + D) & ~3;
    const int xs_end = L.xoff + L.n[0] - D;              // exclusive
    sch.ntx = (xs_end - xs_begin + kTX - 1) / kTX;
    sch.nty = (L.n[1] - 2 * D + Cfg::TY - 1) / Cfg::TY;
    sch.NZ = L.n[2] - 2 * D;
    const long long tiles = (long long)sch.ntx * sch.nty * L.nblk;
    int Lz = tune.zchunk;
    if (Lz <= 0) {
        // default: chunks of 16 planes (the fastest on 512^3 D=1 of every
        // schedule the autotuner tries), fewer when the grid would be small
        Lz = 16;
        if (tiles * ((sch.NZ + 15) / 16) < 2LL * resident) {
            long long nzc = (2LL * resident + tiles - 1) / tiles;
            if (nzc > sch.NZ / 4) nzc = sch.NZ / 4 > 0 ? sch.NZ / 4 : 1;
            Lz = (int)((sch.NZ + nzc - 1) / nzc);
        }
    }
    if (Lz > sch.NZ) Lz = sch.NZ;
    if (Lz < 1) Lz = 1;
    sch.Lz = Lz;
    sch.nzc = (sch.NZ + Lz - 1) / Lz;
    sch.U = tiles * sch.nzc;
    long long G = sch.U;                                 // one unit per CTA
    if (tune.ctas_per_sm > 0) {                          // persistent
        const long long cap = (long long)resident / (resident_per_sm > 0 ? resident_per_sm : 1) *
                              (tune.ctas_per_sm < resident_per_sm ? tune.ctas_per_sm : resident_per_sm);
        if (G > cap) G = cap;
    }
    if (G < 1) G = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)G);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = tune.pdl ? 1 : 0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, *tin, out, L, step_i, c, sch, status);
    count_launches(1);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace

int heat_box_h(int D) { return kWarps * (D == 4 ? B2R_HEAT4_RY : 2) + 2 * D; }
int heat_box_w() { return kTX + 8; }

HeatCoef heat_coef(int D, double alpha_dt, double dx, double dy, double dz)
{
    // central second-difference weights c0..c4 of heat-3D.cu:15-28 (exact)
    static const double cw[5][5] = {
        {0, 0, 0, 0, 0},
        {-2.0, 1.0, 0, 0, 0},
        {-5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0, 0, 0},
        {-49.0 / 18.0, 3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0, 0},
        {-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0}};
    const double wx = alpha_dt / (dx * dx), wy = alpha_dt / (dy * dy), wz = alpha_dt / (dz * dz);
    HeatCoef c{};
    c.a0 = (float)(1.0 + cw[D][0] * (wx + wy + wz));
    for (int k = 1; k <= D; ++k) {
        c.ax[k - 1] = (float)(wx * cw[D][k]);
        c.ay[k - 1] = (float)(wy * cw[D][k]);
        c.az[k - 1] = (float)(wz * cw[D][k]);
    }
    return c;
}

cudaError_t launch_heat_substep(const CUtensorMap* tin, float* out, const BlockLayout& L, int D,
                                int step_i, const HeatCoef& c, int* status, cudaStream_t st,
                                const HeatTune& tune)
{
    switch (D) {
    case 1: return launch_t<1, 2, 4>(tin, out, L, step_i, c, status, st, tune);
    case 2: return launch_t<2, 2, 5>(tin, out, L, step_i, c, status, st, tune);
    case 3: return launch_t<3, 2, 6>(tin, out, L, step_i, c, status, st, tune);
    case 4: return launch_t<4, B2R_HEAT4_RY, 7>(tin, out, L, step_i, c, status, st, tune);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace b2r
