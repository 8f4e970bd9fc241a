// gol.h -- internal interface of the Game of Life kernel (gol.cu).
#pragma once
#include "b2r_common.cuh"

namespace b2r {

// One generation (shrink step_i+1) of every block, in -> out.  Cells of a
// word outside the window are copied from `in`.
cudaError_t launch_gol_substep(const uint8_t* in, uint8_t* out, const BlockLayout& L, int step_i,
                               cudaStream_t st);

// ng (1 .. gol_max_generations_per_pass()) generations of sub-steps i0 ..
// i0 + ng - 1 in one pass, in -> out.  Only the window of the last of them
// is written to `out`.
cudaError_t launch_gol_period(const uint8_t* in, uint8_t* out, const BlockLayout& L, int i0, int ng,
                              cudaStream_t st);
int gol_max_generations_per_pass();

// gol_bits.cu: the same generation as launch_gol_substep with bit-sliced
// cells (32 per word), identical results.
cudaError_t launch_gol_bits_substep(const uint8_t* in, uint8_t* out, const BlockLayout& L, int step_i,
                                   cudaStream_t st);
// ng generations (sub-steps i0 .. i0+ng-1) in one pass on bit-sliced cells;
// only the window of the last one is written to `out`.  push_halos (a pass
// that ends a period; block rows of a multiple of 32 cells) also copies the
// new band cells into the neighbour blocks' halos of `out`, as the next
// period's halo gather would.  rows: output rows per band of a CTA at most
// (0 = 32; any value at least the block height: one band per block).
cudaError_t launch_gol_bits_period(const uint8_t* in, uint8_t* out, const BlockLayout& L, int i0, int ng,
                                   bool push_halos, cudaStream_t st, int rows = 0);
int gol_bits_max_generations_per_pass();

// z chunks per block of the several-generation pass (host side): the CTAs
// (tiles x chunks) are dealt over `sms` SMs, the busiest SM holding
// ceil(CTAs / sms) of them, each computing its chunk of nz planes plus about
// ng - 1 planes of z skirt per generation; the count that makes the busiest
// SM's planes fewest, with every CTA resident at once (cap per SM) and, where
// the block allows, at least minper CTAs per SM on average.
inline int gol_period_chunks(long long tiles, int nz, int ng, int sms, int cap, int minper)
{
    sms = sms > 0 ? sms : 1;
    cap = cap > 0 ? cap : 1;
    int nzc = 1;
    long long best = -1;
    bool best_full = false;
    for (int c = 1; c <= nz; ++c) {
        const long long ctas = tiles * c;
        if (c > 1 && ctas > (long long)sms * cap) break;
        const bool full = ctas >= (long long)minper * sms;
        const long long busiest = (ctas + sms - 1) / sms;
        const long long cost = busiest * ((nz + c - 1) / c + ng - 1);
        if (best < 0 || (full && !best_full) || (full == best_full && cost < best)) {
            best = cost;
            best_full = full;
            nzc = c;
        }
    }
    return nzc;
}

}  // namespace b2r
