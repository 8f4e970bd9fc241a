// selfcheck.cu -- exercise of the device-side failure path (no reference
// counterpart).
//
// Every wait in the library's kernels (TMA ring mbarriers, the batch queue's
// dependency counters) gives up after a time limit, sets the device status
// word to DEV_TIMEOUT and returns, so a stalled pipeline becomes an error
// status on the host instead of a hung GPU.  This entry point runs that path
// on purpose: one CTA initialises an mbarrier, waits (with the library's
// bounded wait) for a phase that nothing will complete, gives up after
// limit_ms, reports, and exits; no copy is in flight, nothing else waits on
// it, and the context stays usable.
#include "b2r_common.cuh"
#include "b2r.h"

namespace b2r {
namespace {

__global__ void bounded_wait_kernel(int* status, unsigned long long limit_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, limit_ns)) report(status, DEV_TIMEOUT);
}

}  // namespace
}  // namespace b2r

extern "C" b2r_status b2r_selfcheck_bounded_wait(double limit_ms, void* cuda_stream)
{
    using namespace b2r;
    if (!(limit_ms > 0.0) || limit_ms > 10000.0) return B2R_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    int* d_status = nullptr;
    if (cudaMalloc(&d_status, sizeof(int)) != cudaSuccess) return B2R_ERR_OOM;
    int s = -1;
    cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(int), st);
    if (e == cudaSuccess) {
        bounded_wait_kernel<<<1, 32, 0, st>>>(d_status, (unsigned long long)(limit_ms * 1e6));
        count_launches(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&s, d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_status);
    if (e != cudaSuccess) return B2R_ERR_CUDA;
    return s == DEV_TIMEOUT ? B2R_ERR_TIMEOUT : (s == 0 ? B2R_OK : B2R_ERR_STATE);
}
