// noalloc.cu -- the heat block entry for callers that cannot allocate.
//
// b2r_heat_3D_gpu_main allocates its two ping-pong blocks and a status word
// with cudaMalloc on every call, as the reference's heat_3D_gpu_main does.
// Some callers cannot do that: a host framework that owns all device memory
// through its own pool and forbids raw cudaMalloc/cudaFree (whose implicit
// device-wide synchronisation would stall the framework's other streams), or
// a control loop that cannot afford an allocation's latency.  This file gives
// them the same computation with its scratch in a fixed device array that is
// part of the library image: the caller passes device input and output, and
// nothing is allocated.
//
// Limits and sharing:
// * each of the two ping-pong buffers holds at most kNoAllocCells cells in
//   the library's padded layout (the same layout as b2r_heat_3D_gpu_main:
//   rows padded to a multiple of 32 cells with at least 4 cells before the
//   block and 8 after it), i.e. P * Ngy * Ngz <= 4,194,304 with P the padded
//   row pitch -- cubes up to 147^3 at R*D = 1; larger blocks are rejected
//   with B2R_ERR_ARG;
// * the array (2 x 16 MiB + 256 B) is resident on every GPU that loads the
//   library, until the process exits;
// * every call on a device uses the same array and leaves its contents
//   behind; the call clears the status word and overwrites both buffers
//   before reading them.  Calls that overlap on the GPU (other streams,
//   other host threads) race on the array and must be serialised by the
//   caller;
// * every call looks up the array's device address on the current device
//   (cudaGetSymbolAddress; cheap, and never stale after a context is torn
//   down and re-created); the first call on a device also loads the
//   library's device code there, so make that first call before any stream
//   capture.
#include <cstdio>

#include "api_internal.h"

namespace b2r {
namespace {

constexpr size_t kNoAllocCells = size_t(4) << 20;            // per ping-pong buffer
constexpr size_t kStatusFloats = 64;                          // 256 B for the status word

// [buffer A | buffer B | status word]
static __device__ __align__(256) float g_noalloc_scratch[2 * kNoAllocCells + kStatusFloats];

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in: kernels must be given this address.
cudaError_t scratch_address(void** out)
{
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *out = p;
    return cudaSuccess;
}

// Errors are reported on stderr and by the returned status.
b2r_status nfail(b2r_status s, const char* what, cudaError_t e = cudaSuccess)
{
    if (e != cudaSuccess)
        fprintf(stderr, "b2r_heat_3D_gpu_main_noalloc: %s: %s\n", what, cudaGetErrorString(e));
    else
        fprintf(stderr, "b2r_heat_3D_gpu_main_noalloc: %s\n", what);
    return s;
}

}  // namespace
}  // namespace b2r

using namespace b2r;

extern "C" b2r_status b2r_heat_3D_gpu_main_noalloc(const float* d_in, float* d_out, int R, int D,
                                                  const char* edge_flag, int Ngx, int Ngy, int Ngz,
                                                  double alpha_dt, double dx, double dy, double dz,
                                                  void* cuda_stream)
{
    if (!d_in || !d_out) return nfail(B2R_ERR_ARG, "null device pointer");
    if (D < 1 || D > 4) return nfail(B2R_ERR_ARG, "stencil radius D must be 1..4");
    if (R < 1) return nfail(B2R_ERR_ARG, "R must be >= 1");
    const int H = R * D;
    const int n[3] = {Ngx, Ngy, Ngz};
    int B[3];
    for (int a = 0; a < 3; ++a) {
        B[a] = n[a] - 2 * H;
        if (B[a] < 1) return nfail(B2R_ERR_ARG, "block too small for R*D");
    }
    int edge = 0;
    if (edge_flag)
        for (int a = 0; a < 3; ++a) {
            const signed char v = static_cast<signed char>(edge_flag[a]);
            if (v < 0) edge |= 1 << (2 * a);
            if (v > 0) edge |= 1 << (2 * a + 1);
        }
    // the allocating entry's padded float layout (b2r_heat_3D_gpu_main)
    const int nb[3] = {1, 1, 1};
    BlockLayout L{};
    b2r_api::fill_layout(L, n, B, nb, H, 4, 0, edge);
    if ((size_t)L.bstride > kNoAllocCells) {
        fprintf(stderr,
                "b2r_heat_3D_gpu_main_noalloc: block %dx%dx%d needs %lld padded cells per buffer;"
                " the no-allocation scratch holds %zu\n",
                Ngx, Ngy, Ngz, L.bstride, kNoAllocCells);
        return B2R_ERR_ARG;
    }

    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return nfail(B2R_ERR_CUDA, "cudaGetSymbolAddress(scratch)", e);
    float* buf[2] = {static_cast<float*>(base), static_cast<float*>(base) + kNoAllocCells};
    int* status = reinterpret_cast<int*>(static_cast<float*>(base) + 2 * kNoAllocCells);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);

    // the array keeps the previous call's contents: clear the status word,
    // and fill both buffers from the input (heat-3D.cu:590-592)
    if ((e = cudaMemsetAsync(status, 0, sizeof(int), st)) != cudaSuccess)
        return nfail(B2R_ERR_CUDA, "clear status", e);
    for (int b = 0; b < 2; ++b)
        if ((e = cudaMemcpy2DAsync(buf[b] + L.xoff, L.P * sizeof(float), d_in, Ngx * sizeof(float),
                                   Ngx * sizeof(float), (size_t)Ngy * Ngz, cudaMemcpyDeviceToDevice,
                                   st)) != cudaSuccess)
            return nfail(B2R_ERR_CUDA, "copy input", e);
    CUtensorMap tm[2];
    for (int b = 0; b < 2; ++b)
        if (!make_block_tmap(&tm[b], buf[b], L, 4, heat_box_w(), heat_box_h(D), 1))
            return nfail(B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    const HeatCoef hc = heat_coef(D, alpha_dt, dx, dy, dz);
    int cur = 0;
    for (int i = 0; i < R; ++i) {   // heat-3D.cu:602-628
        if ((e = launch_heat_substep(&tm[cur], buf[1 - cur], L, D, i, hc, status, st)) != cudaSuccess)
            return nfail(B2R_ERR_CUDA, "heat launch", e);
        cur = 1 - cur;
    }
    // output = input with planes [R*D, Ngz-R*D) replaced (heat-3D.cu:633-635)
    const size_t plane_bytes = (size_t)Ngx * Ngy * sizeof(float);
    if (d_out != d_in) {
        if ((e = cudaMemcpyAsync(d_out, d_in, plane_bytes * H, cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d_out + (size_t)(Ngz - H) * Ngx * Ngy, d_in + (size_t)(Ngz - H) * Ngx * Ngy,
                                 plane_bytes * H, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
            return nfail(B2R_ERR_CUDA, "copy untouched planes", e);
    }
    if ((e = cudaMemcpy2DAsync(d_out + (size_t)H * Ngx * Ngy, Ngx * sizeof(float),
                               buf[cur] + L.xoff + (size_t)H * L.plane, L.P * sizeof(float),
                               Ngx * sizeof(float), (size_t)Ngy * (Ngz - 2 * H),
                               cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return nfail(B2R_ERR_CUDA, "copy result", e);
    int dev_status = 0;
    if ((e = cudaMemcpyAsync(&dev_status, status, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return nfail(B2R_ERR_CUDA, "synchronise", e);
    if (dev_status != DEV_OK) return nfail(B2R_ERR_TIMEOUT, "a device-side bounded wait gave up");
    return B2R_OK;
}
