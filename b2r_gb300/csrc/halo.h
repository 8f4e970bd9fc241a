// halo.h -- internal interface of halo.cu (B2R boundary update, scatter/gather).
#pragma once
#include "b2r_common.cuh"

namespace b2r {

constexpr int kMaxFields = 10;

template <typename T>
struct FieldSet {
    T* p[kMaxFields];
};

// X->Y->Z halo exchange of nfields fields among all blocks.  bounce == null:
// direct neighbour copies; else staged through `bounce`, which must hold
// nfields * halo_bounce_elems(L) elements.
template <typename T>
cudaError_t launch_halo_exchange(const FieldSet<T>& fs, int nfields, const BlockLayout& L,
                                 T* bounce, cudaStream_t st);
size_t halo_bounce_elems(const BlockLayout& L);
// The same boundary update in one launch: every halo cell copied from the
// block owning it (26 face / edge / corner regions per block).
template <typename T>
cudaError_t launch_halo_gather(const FieldSet<T>& fs, int nfields, const BlockLayout& L, cudaStream_t st);

// Dense domain array (shell > 0: with a fixed shell of that depth; periodic
// layouts: bare torus) -> every padded block, halos included; blocks2, when
// not null, is a second set of blocks written with the same cells.
template <typename T>
cudaError_t launch_scatter(const T* dom, T* blocks, T* blocks2, const BlockLayout& L, int shell,
                           cudaStream_t st);
// Blocks -> dense domain array (interiors from their owners, shell from the
// edge blocks' halos, which are never updated).
template <typename T>
cudaError_t launch_gather(T* dom, const T* blocks, const BlockLayout& L, int shell,
                          cudaStream_t st);

}  // namespace b2r
