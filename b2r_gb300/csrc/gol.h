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

}  // namespace b2r
