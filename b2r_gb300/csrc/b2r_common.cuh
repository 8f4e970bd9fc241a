// b2r_common.cuh -- shared device helpers of libb2r (sm_103a only).
//
// * BlockLayout: how the Bx*By*Bz padded subdomain blocks live in HBM.
// * Bounded mbarrier waits and TMA tile loads in inline PTX.
// * Region of a B2R sub-step (the shrinking update window, heat-3D.cu:191,
//   with the fixed-shell mask of heat-3D.cu:81-114).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "../../include/b2r.h"

namespace b2r {

// Device status word codes (written by kernels, read by the host).
enum : int { DEV_OK = 0, DEV_TIMEOUT = 1, DEV_BOUNDS = 2 };

// Padded blocks in HBM.  Block b (x fastest over the block grid) starts at
// element b*bstride; cell (x,y,z) of a block (0 <= x < n[0] ...) is at
// z*plane + y*P + xoff + x.  xoff puts the first interior cell (x = H) on a
// 128-byte boundary and leaves >= 16 bytes of pad before x = 0 and after
// x = n[0]-1, so every tile load starts on a 16-byte boundary at a
// non-negative x and word loads one past the row stay inside it.  P is a
// multiple of 128 bytes, so rows, planes and blocks stay aligned.
struct BlockLayout {
    int n[3];           // padded block cells per axis (B + 2H)
    int B[3];           // interior cells per axis
    int nb[3];          // blocks per axis
    int nblk;           // total blocks
    int H;              // halo depth
    int xoff;           // storage x of cell x = 0
    int P;              // row pitch (cells)
    int periodic;       // 1: halos wrap around the domain
    int fixed_edge;     // >= 0: edge mask of every block (single-block entries)
    long long plane;    // P * n[1]
    long long bstride;  // plane * n[2]
};

__host__ __device__ inline int edge_bits(const BlockLayout& L, int blk)
{
    if (L.fixed_edge >= 0) return L.fixed_edge;
    if (L.periodic) return 0;
    int bx = blk % L.nb[0];
    int by = (blk / L.nb[0]) % L.nb[1];
    int bz = blk / (L.nb[0] * L.nb[1]);
    int e = 0;
    if (bx == 0) e |= 1;
    if (bx == L.nb[0] - 1) e |= 2;
    if (by == 0) e |= 4;
    if (by == L.nb[1] - 1) e |= 8;
    if (bz == 0) e |= 16;
    if (bz == L.nb[2] - 1) e |= 32;
    return e;
}

// Update window of a stage with shrink s along axis a (inclusive bounds).
__host__ __device__ inline void stage_region(const BlockLayout& L, int edge, int a, int s,
                                             int& lo, int& hi)
{
    int n = L.n[a];
    lo = s;
    hi = n - 1 - s;
    // the fixed shell never goes stale: on a boundary face the window is the
    // whole interior side, whatever the shrink
    if ((edge >> (2 * a)) & 1) lo = L.H;
    if ((edge >> (2 * a + 1)) & 1) hi = n - 1 - L.H;
}

#if defined(__CUDACC__)

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for phase `parity` of an mbarrier, giving up after ~limit_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint64_t limit_ns = 2000000000ull)
{
    if (mbar_try_wait(bar, parity)) return true;
    uint64_t t0 = global_ns();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 255u && global_ns() - t0 > limit_ns) return false;
    }
}

// 4-D TMA tile load (x, y, z, block) into shared memory, completion on bar.
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int x, int y,
                                            int z, int w, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void report(int* status, int code)
{
    if (status) atomicCAS(status, 0, code);
}

#endif  // __CUDACC__

// ---------------------------------------------------------------- host side
// Process-wide count of kernels launched by the library.
void count_launches(long long n);

// Encode a 4-D tiled tensor map over all padded blocks of one field.
// elem_bytes 4 (float) or 1 (uint8).  Returns false on failure.
bool make_block_tmap(CUtensorMap* map, const void* base, const BlockLayout& L, int elem_bytes,
                     int box_x, int box_y, int box_z);

// One-time launch setup of a kernel on each device: raise its dynamic
// shared-memory limit and read how many CTAs of `threads` threads fit per SM.
// The function attribute belongs to the device that is current when it is
// set, so the setup is kept per device (device ordinals below
// kSetupDevices).  Host threads may launch concurrently: the first caller on
// a device does the setup under the lock and publishes the result with a
// release store; a failed setup is not published, so the next call tries
// again.
constexpr int kSetupDevices = 64;
struct KernelSetup {
    std::mutex mu;
    std::atomic<int> per_sm[kSetupDevices] = {};   // 0 until the setup on that device succeeded
    int sms[kSetupDevices] = {};                   // written before per_sm[dev] is published
};

template <class Kernel>
cudaError_t kernel_setup(KernelSetup& ks, Kernel kern, int threads, size_t smem, int* per_sm, int* total)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kSetupDevices) return cudaErrorInvalidDevice;
    int v = ks.per_sm[dev].load(std::memory_order_acquire);
    if (v == 0) {
        std::lock_guard<std::mutex> lock(ks.mu);
        v = ks.per_sm[dev].load(std::memory_order_relaxed);
        if (v == 0) {
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            int sms = 0, occ = 0;
            if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem)) != cudaSuccess)
                return e;
            ks.sms[dev] = sms > 0 ? sms : 1;
            v = occ > 0 ? occ : 1;
            ks.per_sm[dev].store(v, std::memory_order_release);
        }
    }
    if (per_sm) *per_sm = v;
    if (total) *total = v * ks.sms[dev];
    return cudaSuccess;
}

// A dynamic shared-memory limit that several launch shapes of one kernel
// share: only ever raised, per device (the attribute belongs to the device
// that is current when it is set), under a lock (handles on several host
// threads).
struct SmemLimit {
    std::mutex mu;
    size_t bytes[kSetupDevices] = {};
};

inline cudaError_t raise_smem_limit(SmemLimit& s, const void* kern, size_t bytes)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kSetupDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(s.mu);
    if (bytes > s.bytes[dev]) {
        if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes)) != cudaSuccess)
            return e;
        s.bytes[dev] = bytes;
    }
    return cudaSuccess;
}

}  // namespace b2r
