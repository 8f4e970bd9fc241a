// work_queue.cuh -- the device work queue of the batched persistent kernels
// (batch.cu: heat instances; eqwp_batch.cu: elastic-wave instances).
//
// Work items (round t, instance k, unit u) are listed round-major by the
// host; instances are sorted by round count (descending), so the instances
// still active at round t are a prefix of the list.  A CTA claims the next
// item with one atomicAdd on a head counter.  Before reading round t of instance
// k it waits until done[k] >= t * units[k] (every unit of round t-1 of that
// instance has finished), runs the unit and bumps done[k] with a release
// reduction.  Items are claimed in increasing order and an item only waits
// on smaller items, which are held by running CTAs, so the queue cannot
// deadlock; every wait is bounded (2 s) and reports B2R_ERR_TIMEOUT.
#pragma once
#include <vector>

#include "b2r_common.cuh"

namespace b2r {
namespace wq {

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// A work item packed into 64 bits: round t (bits 40..63), instance k in the
// queue's instance order (bits 24..39), unit u (bits 0..23).
constexpr int kItemKBits = 16, kItemUBits = 24;
__host__ __device__ inline unsigned long long pack_item(int t, int k, int u)
{
    return ((unsigned long long)t << (kItemKBits + kItemUBits)) | ((unsigned long long)k << kItemUBits) |
           (unsigned long long)u;
}
__device__ __forceinline__ void unpack_item(unsigned long long x, int& t, int& k, int& u)
{
    t = (int)(x >> (kItemKBits + kItemUBits));
    k = (int)((x >> kItemUBits) & ((1u << kItemKBits) - 1));
    u = (int)(x & ((1u << kItemUBits) - 1));
}

// The queue, written out by the host in claim order: round-major over
// instances sorted by their round count (descending), so that those still
// stepping at round t are a prefix; each instance's units in order.  Returns
// false if an instance has more units or rounds than an item can name, or
// the queue would hold more than 2^28 items.
inline bool round_major_items(const int* rounds, const int* units, int n, std::vector<unsigned long long>& items)
{
    long long total = 0;
    int maxr = 0;
    for (int j = 0; j < n; ++j) {
        if (n >= (1 << kItemKBits) || units[j] >= (1 << kItemUBits) ||
            rounds[j] >= (1 << (64 - kItemKBits - kItemUBits)))
            return false;
        total += (long long)units[j] * rounds[j];
        maxr = rounds[j] > maxr ? rounds[j] : maxr;
    }
    if (total > (1ll << 28)) return false;
    items.clear();
    items.reserve((size_t)total);
    for (int t = 0; t < maxr; ++t)
        for (int j = 0; j < n && rounds[j] > t; ++j)
            for (int u = 0; u < units[j]; ++u) items.push_back(pack_item(t, j, u));
    return true;
}

// Bounded wait (2 s) until *done >= need; false if it gave up.  Afterwards
// the data that other CTAs stored with generic stores may be read through
// TMA as well.
__device__ __forceinline__ bool wait_done(const unsigned* done, unsigned need)
{
    bool ok = true;
    if (ld_acquire(done) < need) {
        const uint64_t t0 = global_ns();
        while (ld_acquire(done) < need) {
            if (global_ns() - t0 > 2000000000ull) {
                ok = false;
                break;
            }
            __nanosleep(100);
        }
    }
    asm volatile("fence.proxy.async.global;" ::: "memory");
    return ok;
}

// One unit done, after a __syncthreads that follows all of the CTA's stores:
// release at gpu scope; PTX fences are cumulative, so this orders the whole
// CTA's stores (ordered before it by the barrier) before the count that the
// next round's readers acquire.  Thread 0 only.
__device__ __forceinline__ void release_done(unsigned* done)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(done) : "memory");
}

}  // namespace wq
}  // namespace b2r
