// halo.cu -- device-side B2R boundary update between subdomains resident on
// one GPU, and the domain <-> blocks scatter/gather.
//
// The reference moves R*D-deep face slabs between MPI ranks dimension by
// dimension, X then Y then Z, with growing slab extents so that edges and
// corners arrive without diagonal messages (b2r_halo_sync.cu:195-379,
// 389-508; transport b2r_comm.hpp).  Here every block lives in the same HBM,
// so "send + receive" is one device copy:
//   * direct:  one launch per axis copies each neighbour's interior slab
//              straight into the halo (boundary_updating_direct);
//   * staged:  pack every slab of an axis into a device bounce buffer, then
//              unpack it (sub_matrix_pack/unpack + boundary_updating).
// Slab extents per axis follow the reference: x slabs span interior y,z; y
// slabs full padded x and interior z; z slabs full padded x and y.  One
// launch covers all blocks, both sides and up to kMaxFields fields.
#include <algorithm>
#include <type_traits>

#include "b2r_common.cuh"
#include "halo.h"

namespace b2r {

namespace {

// Slab geometry of an axis: extent e[3] (cells), with the halo axis extent H.
struct Slab {
    int e[3];
    long long cells;  // e0*e1*e2
};

__host__ __device__ inline Slab slab_of(const BlockLayout& L, int axis)
{
    Slab s;
    for (int a = 0; a < 3; ++a) {
        if (a == axis) s.e[a] = L.H;
        else if (a < axis) s.e[a] = L.n[a];     // axes already exchanged: full extent
        else s.e[a] = L.B[a];                   // later axes: interior only
    }
    s.cells = (long long)s.e[0] * s.e[1] * s.e[2];
    return s;
}

// Map slab cell (c0,c1,c2) on `side` (0 = low halo, 1 = high halo) of block
// `blk` to destination / source element offsets.  Returns false when the
// neighbour does not exist (domain boundary, not periodic).
__device__ inline bool slab_map(const BlockLayout& L, int axis, int blk, int side, int c0, int c1,
                                int c2, long long& dst, long long& src)
{
    int b[3] = {blk % L.nb[0], (blk / L.nb[0]) % L.nb[1], blk / (L.nb[0] * L.nb[1])};
    int c[3] = {c0, c1, c2};
    int d[3], s[3];
    for (int a = 0; a < 3; ++a) {
        if (a == axis) continue;
        int base = (a < axis) ? 0 : L.H;
        d[a] = s[a] = base + c[a];
    }
    int nbk[3] = {b[0], b[1], b[2]};
    if (side == 0) {
        nbk[axis] -= 1;
        d[axis] = c[axis];                       // my low halo [0, H)
        s[axis] = L.B[axis] + c[axis];           // neighbour's high interior slab [B, B+H)
    } else {
        nbk[axis] += 1;
        d[axis] = L.B[axis] + L.H + c[axis];     // my high halo [B+H, B+2H)
        s[axis] = L.H + c[axis];                 // neighbour's low interior slab [H, 2H)
    }
    if (nbk[axis] < 0 || nbk[axis] >= L.nb[axis]) {
        if (!L.periodic) return false;
        nbk[axis] = (nbk[axis] + L.nb[axis]) % L.nb[axis];
    }
    const int nblk = nbk[0] + L.nb[0] * (nbk[1] + L.nb[1] * nbk[2]);
    dst = (long long)blk * L.bstride + (long long)d[2] * L.plane + (long long)d[1] * L.P + L.xoff + d[0];
    src = (long long)nblk * L.bstride + (long long)s[2] * L.plane + (long long)s[1] * L.P + L.xoff + s[0];
    return true;
}

// One (field, block, side) per blockIdx.y; slab cells (x fastest) over
// blockIdx.x/threadIdx.x with 32-bit index arithmetic.
template <typename T>
__global__ void halo_direct_kernel(FieldSet<T> fs, const BlockLayout L, int axis, Slab sl)
{
    const int side = blockIdx.y & 1;
    const int blk = (blockIdx.y >> 1) % L.nblk;
    const int fld = (blockIdx.y >> 1) / L.nblk;
    T* f = fs.p[fld];
    const int cells = (int)sl.cells;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cells; e += gridDim.x * blockDim.x) {
        const int c0 = e % sl.e[0];
        const int r1 = e / sl.e[0];
        const int c1 = r1 % sl.e[1];
        const int c2 = r1 / sl.e[1];
        long long dst, src;
        if (slab_map(L, axis, blk, side, c0, c1, c2, dst, src)) f[dst] = f[src];
    }
}

// staged form: bounce[slab] <- neighbour slab, then halo <- bounce[slab]
template <typename T>
__global__ void halo_pack_kernel(FieldSet<T> fs, T* bounce, const BlockLayout L, int axis,
                                 Slab sl, int unpack)
{
    const int side = blockIdx.y & 1;
    const int blk = (blockIdx.y >> 1) % L.nblk;
    const int fld = (blockIdx.y >> 1) / L.nblk;
    T* f = fs.p[fld];
    const int cells = (int)sl.cells;
    T* buf = bounce + ((long long)fld * L.nblk * 2 + blk * 2 + side) * sl.cells;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cells; e += gridDim.x * blockDim.x) {
        const int c0 = e % sl.e[0];
        const int r1 = e / sl.e[0];
        const int c1 = r1 % sl.e[1];
        const int c2 = r1 / sl.e[1];
        long long dst, src;
        if (!slab_map(L, axis, blk, side, c0, c1, c2, dst, src)) continue;
        if (unpack) f[dst] = buf[e];
        else buf[e] = f[src];
    }
}

// domain array <-> blocks.  shell > 0: non-periodic domain with a `shell`
// deep fixed shell; periodic: bare torus.  One warp per row of cells: the
// row's source (scatter) or owner blocks (gather) are found once per row,
// and the lanes walk x with kRowUnroll loads in flight before their stores,
// so the copy runs at HBM speed without per-cell index divisions.
constexpr int kRowWarps = 8;
constexpr int kRowUnroll = 4;

// a global coordinate at most one period outside [0, e) (the halo depth
// never exceeds a block), wrapped onto the torus
__device__ __forceinline__ int wrap_once(int g, int e)
{
    return g < 0 ? g + e : (g >= e ? g - e : g);
}

// blocks2 (may be null): a second set of blocks that gets the same cells
template <typename T>
__global__ void __launch_bounds__(kRowWarps * 32)
scatter_kernel(const T* __restrict__ dom, T* __restrict__ blocks, T* __restrict__ blocks2,
               const BlockLayout L, int shell)
{
    const int lane = threadIdx.x & 31;
    const int e0 = L.nb[0] * L.B[0], e1 = L.nb[1] * L.B[1], e2 = L.nb[2] * L.B[2];
    const int dn0 = e0 + 2 * shell, dn1 = e1 + 2 * shell;
    const long long nrows = (long long)L.n[1] * L.n[2] * L.nblk;
    for (long long r = (long long)blockIdx.x * kRowWarps + (threadIdx.x >> 5); r < nrows;
         r += (long long)gridDim.x * kRowWarps) {
        const int y = (int)(r % L.n[1]);
        const long long rz = r / L.n[1];
        const int z = (int)(rz % L.n[2]);
        const int blk = (int)(rz / L.n[2]);
        const int b0 = blk % L.nb[0], b1 = (blk / L.nb[0]) % L.nb[1], b2 = blk / (L.nb[0] * L.nb[1]);
        const int gx0 = b0 * L.B[0] - L.H;          // global x of block cell x = 0
        int g1 = b1 * L.B[1] + y - L.H, g2 = b2 * L.B[2] + z - L.H;
        // domain row, indexed by the global x (from -shell with a shell);
        // no row: the block row lies outside the domain and its shell (zeros)
        long long row = -1;
        if (L.periodic) {
            g1 = wrap_once(g1, e1);
            g2 = wrap_once(g2, e2);
            if ((unsigned)g1 < (unsigned)e1 && (unsigned)g2 < (unsigned)e2)
                row = ((long long)g2 * e1 + g1) * e0;
        } else if (g1 >= -shell && g1 < e1 + shell && g2 >= -shell && g2 < e2 + shell) {
            row = ((long long)(g2 + shell) * dn1 + (g1 + shell)) * dn0 + shell;
        }
        const long long o = blk * L.bstride + (long long)z * L.plane + (long long)y * L.P + L.xoff;
        for (int xb = 0; xb < L.n[0]; xb += 32 * kRowUnroll) {
            T v[kRowUnroll];
#pragma unroll
            for (int u = 0; u < kRowUnroll; ++u) {
                const int x = xb + u * 32 + lane;
                int g0 = gx0 + x;
                bool in;
                if (L.periodic) {
                    g0 = wrap_once(g0, e0);
                    in = (unsigned)g0 < (unsigned)e0;
                } else {
                    in = g0 >= -shell && g0 < e0 + shell;
                }
                v[u] = (row >= 0 && x < L.n[0] && in) ? dom[row + g0] : T(0);
            }
#pragma unroll
            for (int u = 0; u < kRowUnroll; ++u) {
                const int x = xb + u * 32 + lane;
                if (x < L.n[0]) {
                    blocks[o + x] = v[u];
                    if (blocks2) blocks2[o + x] = v[u];
                }
            }
        }
    }
}

// owner block of global coordinate g along an axis (the shell belongs to
// the edge blocks' halos)
__device__ __forceinline__ int owner_of(int g, int B, int nb)
{
    int b = g >= 0 ? g / B : 0;
    return b >= nb ? nb - 1 : b;
}

template <typename T>
__global__ void __launch_bounds__(kRowWarps * 32)
gather_kernel(T* __restrict__ dom, const T* __restrict__ blocks, const BlockLayout L, int shell)
{
    const int lane = threadIdx.x & 31;
    const int dn0 = L.nb[0] * L.B[0] + 2 * shell, dn1 = L.nb[1] * L.B[1] + 2 * shell;
    const int dn2 = L.nb[2] * L.B[2] + 2 * shell;
    const long long nrows = (long long)dn1 * dn2;
    for (long long r = (long long)blockIdx.x * kRowWarps + (threadIdx.x >> 5); r < nrows;
         r += (long long)gridDim.x * kRowWarps) {
        const int g1 = (int)(r % dn1) - shell, g2 = (int)(r / dn1) - shell;
        const int bb1 = owner_of(g1, L.B[1], L.nb[1]), bb2 = owner_of(g2, L.B[2], L.nb[2]);
        const int l1 = g1 - bb1 * L.B[1] + L.H, l2 = g2 - bb2 * L.B[2] + L.H;
        const long long drow = r * dn0;
        const long long o = (long long)l2 * L.plane + (long long)l1 * L.P + L.xoff;
        const int blk_yz = L.nb[0] * (bb1 + L.nb[1] * bb2);
        // the row's cells [lo, hi) are owned by x-block bb0 (block cell x = d0 - shell - bb0*B + H)
        for (int bb0 = 0; bb0 < L.nb[0]; ++bb0) {
            const int lo = bb0 == 0 ? 0 : shell + bb0 * L.B[0];
            const int hi = bb0 == L.nb[0] - 1 ? dn0 : shell + (bb0 + 1) * L.B[0];
            const long long srow = (long long)(blk_yz + bb0) * L.bstride + o + (L.H - shell - bb0 * L.B[0]);
            for (int xb = lo; xb < hi; xb += 32 * kRowUnroll) {
                T v[kRowUnroll];
#pragma unroll
                for (int u = 0; u < kRowUnroll; ++u) {
                    const int d0 = xb + u * 32 + lane;
                    v[u] = d0 < hi ? blocks[srow + d0] : T(0);
                }
#pragma unroll
                for (int u = 0; u < kRowUnroll; ++u) {
                    const int d0 = xb + u * 32 + lane;
                    if (d0 < hi) dom[drow + d0] = v[u];
                }
            }
        }
    }
}

// ---------------------------------------------------------------- one-launch exchange
// On one GPU every block can read every other block, so each halo cell can
// be copied straight from the block that owns it: the halo shell of a block
// splits into 26 regions (faces, edges, corners), region (dx, dy, dz) being
// the interior slab of neighbour (bx+dx, by+dy, bz+dz) that borders it.  The
// X -> Y -> Z sequence of the reference delivers exactly these values
// (edges and corners arrive in two or three hops from the same owners), so
// one launch replaces three, with no ordering between the regions.  Halo
// cells without an owner (domain boundary, not periodic) keep their values.
// Each region's rows move in the widest vectors (16 down to the cell size)
// that its row length and row starts allow.
#ifndef B2R_HALO_VPT
#define B2R_HALO_VPT 4   // vectors per thread of the one-launch exchange
#endif
struct HaloDirs {
    int n;                  // regions with a possible owner
    int cta0[27];           // first CTA of region k (cta0[n] = total CTAs)
    int d[26][3];           // direction
    int ex[26], ey[26], ez[26];   // extent: x in vectors, y, z in cells
    int dst[26][3], src[26][3];   // origins (cells) in the block and in the owner
    int vb[26];                   // vector bytes of region k's rows
};

// copy ex x ey x ez vectors of VB bytes (rows of ex vectors), grid-stride,
// four vectors per thread and round: their loads are issued before their
// stores (a region's cells are never another region's sources, so the
// source and destination do not alias)
template <int VB>
__device__ __forceinline__ void copy_box(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src, unsigned ex,
                                         unsigned ey, unsigned total, long long rowb, long long planeb,
                                         unsigned e0, unsigned stride)
{
    typedef typename std::conditional<VB == 16, uint4,
            typename std::conditional<VB == 8, uint2,
            typename std::conditional<VB == 4, uint32_t,
            typename std::conditional<VB == 2, uint16_t, uint8_t>::type>::type>::type>::type V;
    constexpr int U = 4;
    for (unsigned e = e0; e < total; e += U * stride) {
        V v[U];
        long long off[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned ee = e + u * stride;
            off[u] = -1;
            if (ee < total) {
                const unsigned vx = ee % ex, r = ee / ex;
                const unsigned y = r % ey, z = r / ey;
                off[u] = (long long)vx * VB + y * rowb + z * planeb;
                v[u] = *reinterpret_cast<const V*>(src + off[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (off[u] >= 0) *reinterpret_cast<V*>(dst + off[u]) = v[u];
    }
}

__global__ void __launch_bounds__(256)
halo_gather_kernel(FieldSet<uint8_t> fs, const BlockLayout L, int cb, const HaloDirs hd)
{
    const int blk = blockIdx.y % L.nblk;
    uint8_t* base = fs.p[blockIdx.y / L.nblk];
    int k = 0;
    while (k + 1 < hd.n && (int)blockIdx.x >= hd.cta0[k + 1]) ++k;
    const int b[3] = {blk % L.nb[0], (blk / L.nb[0]) % L.nb[1], blk / (L.nb[0] * L.nb[1])};
    int o[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        o[a] = b[a] + hd.d[k][a];
        if (o[a] < 0 || o[a] >= L.nb[a]) {
            if (!L.periodic) return;
            o[a] = (o[a] + L.nb[a]) % L.nb[a];
        }
    }
    const int oblk = o[0] + L.nb[0] * (o[1] + L.nb[1] * o[2]);
    const long long rowb = (long long)L.P * cb, planeb = (long long)L.plane * cb;
    uint8_t* dst = base + ((long long)blk * L.bstride + L.xoff + hd.dst[k][0]) * cb +
                   hd.dst[k][1] * rowb + hd.dst[k][2] * planeb;
    const uint8_t* src = base + ((long long)oblk * L.bstride + L.xoff + hd.src[k][0]) * cb +
                         hd.src[k][1] * rowb + hd.src[k][2] * planeb;
    const unsigned ex = hd.ex[k], ey = hd.ey[k];
    const unsigned total = ex * ey * (unsigned)hd.ez[k];
    const unsigned nct = hd.cta0[k + 1] - hd.cta0[k];
    const unsigned e0 = (blockIdx.x - hd.cta0[k]) * blockDim.x + threadIdx.x, stride = nct * blockDim.x;
    switch (hd.vb[k]) {   // uniform per CTA
    case 16: copy_box<16>(dst, src, ex, ey, total, rowb, planeb, e0, stride); break;
    case 8: copy_box<8>(dst, src, ex, ey, total, rowb, planeb, e0, stride); break;
    case 4: copy_box<4>(dst, src, ex, ey, total, rowb, planeb, e0, stride); break;
    case 2: copy_box<2>(dst, src, ex, ey, total, rowb, planeb, e0, stride); break;
    default: copy_box<1>(dst, src, ex, ey, total, rowb, planeb, e0, stride); break;
    }
}

inline int grid_for(long long work, int threads)
{
    long long g = (work + threads - 1) / threads;
    if (g > 152LL * 32) g = 152LL * 32;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

template <typename T>
cudaError_t launch_halo_exchange(const FieldSet<T>& fs, int nfields, const BlockLayout& L,
                                 T* bounce, cudaStream_t st)
{
    if (L.nblk == 1 && !L.periodic) return cudaSuccess;   // all halos are shell
    for (int axis = 0; axis < 3; ++axis) {
        const Slab sl = slab_of(L, axis);
        long long gx = (sl.cells + 255) / 256;
        const long long per_y = 2LL * L.nblk * nfields;
        const long long cap = (152LL * 32 + per_y - 1) / per_y;   // ~32 CTAs per SM overall
        if (gx > cap) gx = cap;
        if (gx < 1) gx = 1;
        dim3 grid((unsigned)gx, (unsigned)per_y);
        if (bounce == nullptr) {
            halo_direct_kernel<T><<<grid, 256, 0, st>>>(fs, L, axis, sl);
            count_launches(1);
        } else {
            halo_pack_kernel<T><<<grid, 256, 0, st>>>(fs, bounce, L, axis, sl, 0);
            halo_pack_kernel<T><<<grid, 256, 0, st>>>(fs, bounce, L, axis, sl, 1);
            count_launches(2);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename T>
cudaError_t launch_halo_gather(const FieldSet<T>& fs, int nfields, const BlockLayout& L, cudaStream_t st)
{
    if (L.nblk == 1 && !L.periodic) return cudaSuccess;   // all halos are shell
    const int cb = (int)sizeof(T);
    HaloDirs hd{};
    const long long per_cta = 256LL * B2R_HALO_VPT;    // vectors per CTA
    int ctas = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int d[3] = {dx, dy, dz};
                if (!dx && !dy && !dz) continue;
                bool any = true;
                for (int a = 0; a < 3; ++a)
                    if (d[a] && L.nb[a] == 1 && !L.periodic) any = false;
                if (!any) continue;
                const int k = hd.n++;
                int ext[3];
                for (int a = 0; a < 3; ++a) {
                    hd.d[k][a] = d[a];
                    ext[a] = d[a] ? L.H : L.B[a];
                    hd.dst[k][a] = d[a] < 0 ? 0 : (d[a] == 0 ? L.H : L.H + L.B[a]);
                    hd.src[k][a] = d[a] < 0 ? L.B[a] : L.H;
                }
                // widest vector that the region's row length and both row starts are multiples of
                int vb = 16;
                while (vb > cb && ((ext[0] * cb) % vb || ((L.xoff + hd.dst[k][0]) * cb) % vb ||
                                   ((L.xoff + hd.src[k][0]) * cb) % vb))
                    vb >>= 1;
                if (vb < cb) vb = cb;
                hd.vb[k] = vb;
                hd.ex[k] = ext[0] * cb / vb;
                hd.ey[k] = ext[1];
                hd.ez[k] = ext[2];
                const long long nv = (long long)hd.ex[k] * ext[1] * ext[2];
                hd.cta0[k] = ctas;
                ctas += (int)std::max(1LL, std::min<long long>((nv + per_cta - 1) / per_cta, 4096));
            }
    hd.cta0[hd.n] = ctas;
    if (hd.n == 0) return cudaSuccess;
    FieldSet<uint8_t> fb{};
    for (int f = 0; f < nfields; ++f) fb.p[f] = reinterpret_cast<uint8_t*>(fs.p[f]);
    const dim3 grid((unsigned)ctas, (unsigned)(nfields * L.nblk));
    halo_gather_kernel<<<grid, 256, 0, st>>>(fb, L, cb, hd);
    count_launches(1);
    return cudaGetLastError();
}

size_t halo_bounce_elems(const BlockLayout& L)
{
    size_t m = 0;
    for (int axis = 0; axis < 3; ++axis) {
        const Slab sl = slab_of(L, axis);
        size_t w = (size_t)(2 * sl.cells * L.nblk);
        if (w > m) m = w;
    }
    return m;
}

template <typename T>
cudaError_t launch_scatter(const T* dom, T* blocks, T* blocks2, const BlockLayout& L, int shell,
                           cudaStream_t st)
{
    const long long rows = (long long)L.n[1] * L.n[2] * L.nblk;
    scatter_kernel<T><<<grid_for(rows * 32, kRowWarps * 32), kRowWarps * 32, 0, st>>>(dom, blocks, blocks2, L,
                                                                                      shell);
    count_launches(1);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gather(T* dom, const T* blocks, const BlockLayout& L, int shell, cudaStream_t st)
{
    const long long rows = (long long)(L.nb[1] * L.B[1] + 2 * shell) * (L.nb[2] * L.B[2] + 2 * shell);
    gather_kernel<T><<<grid_for(rows * 32, kRowWarps * 32), kRowWarps * 32, 0, st>>>(dom, blocks, L, shell);
    count_launches(1);
    return cudaGetLastError();
}

template cudaError_t launch_halo_exchange<float>(const FieldSet<float>&, int, const BlockLayout&,
                                                 float*, cudaStream_t);
template cudaError_t launch_halo_exchange<uint8_t>(const FieldSet<uint8_t>&, int,
                                                   const BlockLayout&, uint8_t*, cudaStream_t);
template cudaError_t launch_halo_gather<float>(const FieldSet<float>&, int, const BlockLayout&, cudaStream_t);
template cudaError_t launch_halo_gather<uint8_t>(const FieldSet<uint8_t>&, int, const BlockLayout&,
                                                 cudaStream_t);
template cudaError_t launch_scatter<float>(const float*, float*, float*, const BlockLayout&, int, cudaStream_t);
template cudaError_t launch_scatter<uint8_t>(const uint8_t*, uint8_t*, uint8_t*, const BlockLayout&, int,
                                             cudaStream_t);
template cudaError_t launch_gather<float>(float*, const float*, const BlockLayout&, int, cudaStream_t);
template cudaError_t launch_gather<uint8_t>(uint8_t*, const uint8_t*, const BlockLayout&, int,
                                            cudaStream_t);

}  // namespace b2r
