// work_queue.cuh -- the device work queue of the batched persistent kernels
// (batch.cu: heat instances; eqwp_batch.cu: elastic-wave instances).
//
// Work items (round t, instance k, unit u) are numbered round-major;
// instances are sorted by round count (descending), so the instances still
// active at round t are a prefix of the list.  A CTA claims the next item
// with one atomicAdd on a head counter.  Before reading round t of instance
// k it waits until done[k] >= t * units[k] (every unit of round t-1 of that
// instance has finished), runs the unit and bumps done[k] with a release
// reduction.  Items are claimed in increasing order and an item only waits
// on smaller items, which are held by running CTAs, so the queue cannot
// deadlock; every wait is bounded (2 s) and reports B2R_ERR_TIMEOUT.
#pragma once
#include "b2r_common.cuh"

namespace b2r {
namespace wq {

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Item -> (round, instance, unit) by binary searches in the schedule tables
// (step_off: items before round t; active: instances still active at round
// t; prefix: units of instances [0, k)) -- the elastic-wave batch; the heat
// batch reads its items from an array the host writes in claim order.
__device__ __forceinline__ void decode(long long item, const long long* step_off, const int* active,
                                       const long long* prefix, int maxrounds, int& t, int& k, int& u)
{
    int lo = 0, hi = maxrounds;                     // last t with step_off[t] <= item
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (step_off[mid] <= item) lo = mid; else hi = mid;
    }
    t = lo;
    const long long r = item - step_off[t];
    int kl = 0, kh = active[t];                     // last k with prefix[k] <= r
    while (kh - kl > 1) {
        const int mid = (kl + kh) >> 1;
        if (prefix[mid] <= r) kl = mid; else kh = mid;
    }
    k = kl;
    u = (int)(r - prefix[k]);
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
