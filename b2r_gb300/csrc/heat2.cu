// heat2.cu -- two heat time steps per HBM pass (temporal blocking), radius 1:
// the launch of heat2_unit.cuh's units over every tile of every block.
#include "heat2_unit.cuh"

namespace b2r {
namespace {

using namespace h2k;

constexpr int kS2 = 4;                // input ring slots
constexpr size_t kSmem2 = size_t(kS2) * kPlane * 4 + 2 * size_t(kP1) * 4 + kS2 * 8 + 16 + 128;

__device__ __forceinline__ void pdl_wait2() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger2() { asm volatile("griddepcontrol.launch_dependents;"); }

struct H2Sched {
    int ntx, nty, NZ, Lz, nzc;
    long long U;
};

__global__ void __launch_bounds__(kT2, 2)
heat2_kernel(const __grid_constant__ CUtensorMap tin, float* __restrict__ out, const BlockLayout L,
             const int step_i, const HeatCoef C, const H2Sched sch, int* __restrict__ status)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    H2Ctx c;
    float* ring = reinterpret_cast<float*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    c.ring = ring;
    c.s1 = ring + kS2 * kPlane;                          // 2 stage-1 planes
    c.bar = reinterpret_cast<uint64_t*>(c.s1 + 2 * kP1);
    c.abort_flag = reinterpret_cast<int*>(c.bar + kS2);
    c.tid = threadIdx.x;
    c.lane = c.tid & 31;
    c.warp = c.tid >> 5;
    c.tmap = &tin;
    c.C = C;
    c.plane = L.plane;
    c.P = L.P;
    if (c.tid == 0) {
        *c.abort_flag = 0;
        for (int s = 0; s < kS2; ++s) mbar_init(&c.bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    pdl_wait2();
    pdl_trigger2();

    c.gp = 0;
    c.issued_hi = 0;
    c.stop = 0;
    c.aborted = false;
    for (long long u = blockIdx.x; u < sch.U && !c.aborted; u += gridDim.x) {
        const int tx = (int)(u % sch.ntx);
        long long r = u / sch.ntx;
        const int ty = (int)(r % sch.nty);
        r /= sch.nty;
        const int zc = (int)(r % sch.nzc);
        const int blk = (int)(r / sch.nzc);
        if (!h2_unit<kS2, kPlane>(c, &tin, out, L, step_i, blk, tx, ty, zc * sch.Lz, sch.Lz, false)) break;
    }
    if (c.aborted && c.tid == 0) {
        report(status, DEV_TIMEOUT);
        for (unsigned g = c.stop; g < c.issued_hi; ++g)
            mbar_wait_bounded(&c.bar[g % kS2], (g / kS2) & 1, 100000000ull);
    }
}

}  // namespace

int heat2_box_w() { return kBoxW; }
int heat2_box_h() { return kBoxH; }

cudaError_t launch_heat_substep2(const CUtensorMap* tin, float* out, const BlockLayout& L, int step_i,
                                 const HeatCoef& c, int* status, cudaStream_t st, int zchunk)
{
    static KernelSetup setup;
    int resident = 0;                          // CTAs resident on the whole GPU
    if (cudaError_t e = kernel_setup(setup, heat2_kernel, kT2, kSmem2, nullptr, &resident)) return e;
    H2Sched sch;
    sch.ntx = h2_ntx(L);
    sch.nty = h2_nty(L);
    sch.NZ = L.n[2] - 2;
    const long long tiles = (long long)sch.ntx * sch.nty * L.nblk;
    int Lz = zchunk > 0 ? zchunk : 16;
    if (zchunk <= 0 && tiles * ((sch.NZ + 15) / 16) < 2LL * resident) {
        long long nzc = (2LL * resident + tiles - 1) / tiles;
        if (nzc > sch.NZ / 4) nzc = sch.NZ / 4 > 0 ? sch.NZ / 4 : 1;
        Lz = (int)((sch.NZ + nzc - 1) / nzc);
    }
    if (Lz > sch.NZ) Lz = sch.NZ;
    sch.Lz = Lz;
    sch.nzc = (sch.NZ + Lz - 1) / Lz;
    sch.U = tiles * sch.nzc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(sch.U < 1 ? 1 : sch.U));
    cfg.blockDim = dim3(kT2);
    cfg.dynamicSmemBytes = kSmem2;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, heat2_kernel, *tin, out, L, step_i, c, sch, status);
    count_launches(1);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace b2r
