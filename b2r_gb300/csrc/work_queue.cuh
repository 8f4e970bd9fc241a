// work_queue.cuh -- the device work queue of the batched persistent kernels
// (batch.cu: heat instances; eqwp_batch.cu: elastic-wave instances).
//
// Work items (round t, instance k, unit u) are numbered round-major;
// instances are sorted by round count (descending), so the instances still
// active at round t are a prefix of the list.  A CTA claims the next item
// with one atomicAdd on a head counter.  Before round t of unit u it waits
// until u and the units next to it have finished round t-1 (a counter per
// unit), runs the unit and bumps u's counter with a release reduction.
// Items are claimed in increasing order and an item only waits on smaller
// items, which are held by running CTAs, so the queue cannot deadlock; every
// wait is bounded (2 s) and reports B2R_ERR_TIMEOUT.  Units must be at least
// as large as the stencil's reach in every direction (tiles of >= 32 x 8
// cells, z chunks of >= 8 planes), so that only adjacent units share cells.
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
// t; prefix: units of instances [0, k)).
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

// Bounded wait (2 s for all of them together) until unit u of an instance's
// nx x ny x nz grid of units and its neighbours -- the six that share a face,
// or all 26 around it when diag -- have each finished `need` rounds
// (done[v]: rounds finished by unit v); false if it gave up.  A unit reads
// and overwrites only cells of its own tile and of the tiles next to it, so
// these are the only units whose previous round it depends on.
__device__ __forceinline__ bool wait_neighbours(const unsigned* done, int u, int nx, int ny, int nz, unsigned need,
                                                bool diag)
{
    const int x = u % nx, r = u / nx, y = r % ny, z = r / ny;
    const uint64_t t0 = global_ns();
    bool ok = true;
    for (int dz = -1; dz <= 1 && ok; ++dz)
        for (int dy = -1; dy <= 1 && ok; ++dy)
            for (int dx = -1; dx <= 1 && ok; ++dx) {
                if (!diag && (dx != 0) + (dy != 0) + (dz != 0) > 1) continue;
                const int xx = x + dx, yy = y + dy, zz = z + dz;
                if (xx < 0 || xx >= nx || yy < 0 || yy >= ny || zz < 0 || zz >= nz) continue;
                const unsigned* d = done + (xx + nx * (yy + ny * zz));
                while (ld_acquire(d) < need) {
                    if (global_ns() - t0 > 2000000000ull) {
                        ok = false;
                        break;
                    }
                    __nanosleep(64);
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
