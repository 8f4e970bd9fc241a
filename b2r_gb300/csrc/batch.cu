// batch.cu -- many independent heat instances of uneven sizes and stencil
// orders advanced in ONE persistent launch driven by a device work queue.
//
// No reference counterpart (the reference runs one model per MPI rank); each
// instance is a single-block heat domain with a fixed shell, stepped with the
// scheme of heat-3D.cu:228-231/315-318/410-413/514-517 exactly as the plain
// sweep does, so results are bit-identical to per-instance plain runs.
//
// Work items (step t, instance k, unit u) are numbered step-major; instances
// are sorted by step count (descending), so the instances still active at
// step t are a prefix of the list.  A CTA claims the next item with one
// atomicAdd on a head counter.  Before reading step t of instance k it waits
// until done[k] >= t * units[k] (every unit of step t-1 of that instance has
// finished), then streams the unit exactly as the plain sweep does and bumps
// done[k].  Items are claimed in increasing order and an item only waits on
// smaller items, which are held by running CTAs, so the queue cannot
// deadlock; every wait is bounded (2 s) and reports B2R_ERR_TIMEOUT.
#include <algorithm>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "heat_unit.cuh"

namespace b2r {
namespace {

using heatk::kThreads;
// One ring for every stencil order: 5 slots (D = 4 needs D+1), each as large
// as the biggest plane.  D <= 2 tiles have 2 rows per warp, D >= 3 tiles one
// (their register queues are 2D+1 planes deep); 2 CTAs/SM without spills.
constexpr int kS = 5;
template <int D>
struct RowsPerWarp {
    static constexpr int value = D <= 2 ? 2 : 1;
};
constexpr int cmax(int a, int b) { return a > b ? a : b; }
// tile shapes: LPR lanes per row = 32, 16, 8 -> 128, 64, 32 cells wide
template <int D, int LPR>
using BCfg = heatk::Cfg<D, RowsPerWarp<D>::value, kS, 0, LPR>;
template <int LPR>
constexpr int slot_max()
{
    return cmax(cmax(BCfg<1, LPR>::SLOT, BCfg<2, LPR>::SLOT), cmax(BCfg<3, LPR>::SLOT, BCfg<4, LPR>::SLOT));
}
constexpr int kSlot = cmax(cmax(slot_max<32>(), slot_max<16>()), slot_max<8>());
constexpr size_t kSmem = size_t(kS) * kSlot * sizeof(float) + kS * sizeof(uint64_t) + 16 + 128;
constexpr int kLpr[3] = {32, 16, 8};
constexpr int kBoxH[5][3] = {{0, 0, 0},
                             {BCfg<1, 32>::BH, BCfg<1, 16>::BH, BCfg<1, 8>::BH},
                             {BCfg<2, 32>::BH, BCfg<2, 16>::BH, BCfg<2, 8>::BH},
                             {BCfg<3, 32>::BH, BCfg<3, 16>::BH, BCfg<3, 8>::BH},
                             {BCfg<4, 32>::BH, BCfg<4, 16>::BH, BCfg<4, 8>::BH}};
constexpr int kTileY[5][3] = {{0, 0, 0},
                              {BCfg<1, 32>::TY, BCfg<1, 16>::TY, BCfg<1, 8>::TY},
                              {BCfg<2, 32>::TY, BCfg<2, 16>::TY, BCfg<2, 8>::TY},
                              {BCfg<3, 32>::TY, BCfg<3, 16>::TY, BCfg<3, 8>::TY},
                              {BCfg<4, 32>::TY, BCfg<4, 16>::TY, BCfg<4, 8>::TY}};

struct InstDev {
    BlockLayout L;
    float* buf[2];
    HeatCoef C;
    int D, nsteps, ntx, nty, NZ, Lz, nzc, units;
};

struct BatchArgs {
    const InstDev* inst;                 // sorted by nsteps, descending
    const CUtensorMap* maps;             // 2 per instance: buffer 0, buffer 1
    const long long* step_off;           // items before step t (size maxsteps+1)
    const int* active;                   // instances still stepping at step t
    const long long* unit_prefix;        // units of instances [0, k) (size n+1)
    unsigned long long* head;            // next item (zeroed per run)
    unsigned* done;                      // finished units per instance (zeroed per run)
    int* status;
    int maxsteps, ninst;
    long long total;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// the four unit bodies are inlined into the kernel (measured faster than
// separate calls, whose calling convention spills the register queues)
#ifdef B2R_BATCH_NOINLINE
#define B2R_UNIT_INLINE __noinline__
#else
#define B2R_UNIT_INLINE __forceinline__
#endif
template <int D, int LPR>
__device__ B2R_UNIT_INLINE bool run_unit(const BatchArgs& a, const InstDev& in, int k, int t, int u,
                                         heatk::Ring& rg)
{
    const int tx = u % in.ntx;
    const int r = u / in.ntx;
    const int ty = r % in.nty;
    const int zc = r / in.nty;
    const int zi0 = zc * in.Lz;
    const int zi1 = min(in.NZ, zi0 + in.Lz);
    return heatk::sweep_unit<D, RowsPerWarp<D>::value, kS, kSlot, LPR>(
        &a.maps[2 * k + (t & 1)], in.buf[(t + 1) & 1], in.L, 0, in.C, 0, tx, ty, zi0, zi1, rg);
}

// Item -> (step, instance, unit) by binary searches in the shared-memory
// copies of the schedule tables.
__device__ __forceinline__ void decode(long long item, const long long* step_off, const int* active,
                                       const long long* prefix, int maxsteps, int& t, int& k, int& u)
{
    int lo = 0, hi = maxsteps;                      // last t with step_off[t] <= item
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

#ifndef B2R_BATCH_MINB
#define B2R_BATCH_MINB 2   // resident CTAs per SM the register budget is fitted to (no spills)
#endif
// LPR: tile shape of every instance of the launch (lanes per tile row)
template <int LPR>
__global__ void __launch_bounds__(kThreads, B2R_BATCH_MINB) batch_kernel(const BatchArgs a)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    heatk::Ring rg;
    heatk::ring_init<kS, kSlot>(rg, smem_raw);
    // schedule tables after the ring (the ring ends 16 bytes after its barriers)
    long long* s_step_off = reinterpret_cast<long long*>(
        reinterpret_cast<unsigned char*>(rg.abort_flag) + 16);
    long long* s_prefix = s_step_off + (a.maxsteps + 1);
    int* s_active = reinterpret_cast<int*>(s_prefix + (a.ninst + 1));
    for (int i = threadIdx.x; i <= a.maxsteps; i += blockDim.x) {
        s_step_off[i] = a.step_off[i];
        s_active[i] = a.active[i];
    }
    for (int i = threadIdx.x; i <= a.ninst; i += blockDim.x) s_prefix[i] = a.unit_prefix[i];
    __shared__ long long s_next, s_cur;
    __shared__ int s_t, s_k, s_u, s_ok;
    if (threadIdx.x == 0) s_next = (long long)atomicAdd(a.head, 1ull);
    for (;;) {
        __syncthreads();                     // every thread is done with the last item's values
        if (threadIdx.x == 0) {
            const long long item = s_next;
            s_cur = item;
            if (item < a.total) {
            int t, k, u;
            decode(item, s_step_off, s_active, s_prefix, a.maxsteps, t, k, u);
            int ok = 1;
            if (t > 0) {        // wait for step t-1 of this instance (bounded)
                const unsigned need = (unsigned)t * (unsigned)a.inst[k].units;
                if (ld_acquire(&a.done[k]) < need) {
                    const uint64_t t0 = global_ns();
                    while (ld_acquire(&a.done[k]) < need) {
                        if (global_ns() - t0 > 2000000000ull) {
                            ok = 0;
                            break;
                        }
                        __nanosleep(100);
                    }
                }
                // data written by other CTAs' generic stores is read by TMA
                asm volatile("fence.proxy.async.global;" ::: "memory");
            }
            s_t = t;
            s_k = k;
            s_u = u;
            s_ok = ok;
            // claim the next item now, so it is ready when this one is done
            s_next = (long long)atomicAdd(a.head, 1ull);
            }
        }
        __syncthreads();
        if (s_cur >= a.total) break;
        if (!s_ok) {
            if (threadIdx.x == 0) report(a.status, DEV_TIMEOUT);
            return;                          // no load of this CTA is in flight here
        }
        const int t = s_t, k = s_k, u = s_u;
        const InstDev& in = a.inst[k];
        bool ok;
        switch (in.D) {
        case 1: ok = run_unit<1, LPR>(a, in, k, t, u, rg); break;
        case 2: ok = run_unit<2, LPR>(a, in, k, t, u, rg); break;
        case 3: ok = run_unit<3, LPR>(a, in, k, t, u, rg); break;
        default: ok = run_unit<4, LPR>(a, in, k, t, u, rg); break;
        }
        if (!ok) {
            if (threadIdx.x == 0) report(a.status, DEV_TIMEOUT);
            heatk::ring_drain<kS>(rg);
            return;
        }
        __syncthreads();                     // every store of this unit is issued
        if (threadIdx.x == 0) {
            // release at gpu scope; PTX fences are cumulative, so this orders
            // the whole CTA's stores (ordered before it by the barrier) before
            // the count that the next step's readers acquire
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&a.done[k]) : "memory");
        }
    }
}

}  // namespace
}  // namespace b2r

using namespace b2r;

struct b2r_batch {
    int n = 0;
    std::vector<b2r_batch_item> items;
    std::vector<int> order;          // sorted position -> caller index
    std::vector<int> pos;            // caller index -> sorted position
    std::vector<InstDev> host;       // sorted
    std::vector<CUtensorMap> maps;   // sorted, 2 per instance
    InstDev* d_inst = nullptr;
    CUtensorMap* d_maps = nullptr;
    long long* d_step_off = nullptr;
    int* d_active = nullptr;
    long long* d_prefix = nullptr;
    unsigned long long* d_head = nullptr;
    unsigned* d_done = nullptr;
    int* d_status = nullptr;
    float* staging = nullptr;
    size_t staging_bytes = 0;
    int maxsteps = 0;
    long long total = 0;
    int lz_policy = 16;              // z chunk cap per unit (autotuned)
    int shape = 0;                   // tile shape of every instance: index into kLpr (autotuned)
    int grid[3] = {0, 0, 0};         // persistent grid per tile shape
    size_t smem = 0;                 // ring + schedule tables
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t gstream = nullptr;
    long long launches = 0;
};

namespace {

thread_local char g_berr[512];

b2r_status bfail(b2r_status s, const char* msg, cudaError_t e = cudaSuccess)
{
    if (e != cudaSuccess) snprintf(g_berr, sizeof g_berr, "%s: %s", msg, cudaGetErrorString(e));
    else snprintf(g_berr, sizeof g_berr, "%s", msg);
    return s;
}

#define BCK(call, msg)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            cudaGetLastError(); /* a non-sticky error must not resurface in a later check */ \
            return bfail(e_ == cudaErrorMemoryAllocation ? B2R_ERR_OOM : B2R_ERR_CUDA, msg, e_); \
        }                                                                                    \
    } while (0)

inline int roundup(int v, int m) { return (v + m - 1) / m * m; }

// cells one plane of an instance computes with tile shape s
long long plane_cells(const b2r_batch* b, int k, int s)
{
    const InstDev& in = b->host[k];
    const BlockLayout& L = in.L;
    const int D = in.D;
    const int X = L.xoff + L.n[0] - D - ((L.xoff + D) & ~3), Y = L.n[1] - 2 * D;
    const int tw = 4 * kLpr[s], th = kTileY[D][s];
    return (long long)((X + tw - 1) / tw) * tw * ((Y + th - 1) / th) * th;
}

// The tile shape for the whole mix: the fewest cells computed over every
// instance's steps, narrow tiles paying a little for their wider skirt.
int default_shape(const b2r_batch* b)
{
    static const double penalty[3] = {1.0, 1.03, 1.08};
    int best = 0;
    double bc = 1e300;
    for (int s = 0; s < 3; ++s) {
        double c = 0;
        for (int k = 0; k < b->n; ++k)
            c += (double)plane_cells(b, k, s) * b->host[k].NZ * b->host[k].nsteps;
        c *= penalty[s];
        if (c < bc - 1e-9) {
            bc = c;
            best = s;
        }
    }
    return best;
}

b2r_status build_schedule(b2r_batch* b);

// tile counts and tensor-map boxes of every instance for shape s
b2r_status apply_shape(b2r_batch* b, int s)
{
    b->shape = s;
    for (int k = 0; k < b->n; ++k) {
        InstDev& in = b->host[k];
        const BlockLayout& L = in.L;
        const int D = in.D;
        const int X = L.xoff + L.n[0] - D - ((L.xoff + D) & ~3), Y = L.n[1] - 2 * D;
        const int tw = 4 * kLpr[s], th = kTileY[D][s];
        in.ntx = (X + tw - 1) / tw;
        in.nty = (Y + th - 1) / th;
        for (int f = 0; f < 2; ++f)
            if (!make_block_tmap(&b->maps[2 * k + f], in.buf[f], L, 4, tw + 8, kBoxH[D][s], 1))
                return bfail(B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    }
    BCK(cudaMemcpy(b->d_maps, b->maps.data(), sizeof(CUtensorMap) * 2 * b->n, cudaMemcpyHostToDevice),
        "copy tensor maps");
    return build_schedule(b);
}

// schedule tables for the current Lz policy
b2r_status build_schedule(b2r_batch* b)
{
    std::vector<long long> prefix(b->n + 1, 0);
    for (int k = 0; k < b->n; ++k) {
        InstDev& in = b->host[k];
        in.Lz = std::min(in.NZ, b->lz_policy > 0 ? b->lz_policy : in.NZ);
        in.nzc = (in.NZ + in.Lz - 1) / in.Lz;
        in.units = in.ntx * in.nty * in.nzc;
        prefix[k + 1] = prefix[k] + in.units;
    }
    std::vector<long long> step_off(b->maxsteps + 1, 0);
    std::vector<int> active(b->maxsteps + 1, 0);
    for (int t = 0; t < b->maxsteps; ++t) {
        int A = 0;
        while (A < b->n && b->host[A].nsteps > t) ++A;
        active[t] = A;
        step_off[t + 1] = step_off[t] + prefix[A];
    }
    b->total = step_off[b->maxsteps];
    BCK(cudaMemcpy(b->d_inst, b->host.data(), sizeof(InstDev) * b->n, cudaMemcpyHostToDevice), "copy descriptors");
    BCK(cudaMemcpy(b->d_step_off, step_off.data(), sizeof(long long) * (b->maxsteps + 1), cudaMemcpyHostToDevice), "copy step table");
    BCK(cudaMemcpy(b->d_active, active.data(), sizeof(int) * (b->maxsteps + 1), cudaMemcpyHostToDevice), "copy active table");
    BCK(cudaMemcpy(b->d_prefix, prefix.data(), sizeof(long long) * (b->n + 1), cudaMemcpyHostToDevice), "copy prefix table");
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    return B2R_OK;
}

b2r_status enqueue_run(b2r_batch* b, cudaStream_t st)
{
    BCK(cudaMemsetAsync(b->d_head, 0, sizeof(unsigned long long), st), "reset queue");
    BCK(cudaMemsetAsync(b->d_done, 0, sizeof(unsigned) * b->n, st), "reset counters");
    BatchArgs a;
    a.inst = b->d_inst;
    a.maps = b->d_maps;
    a.step_off = b->d_step_off;
    a.active = b->d_active;
    a.unit_prefix = b->d_prefix;
    a.head = b->d_head;
    a.done = b->d_done;
    a.status = b->d_status;
    a.maxsteps = b->maxsteps;
    a.ninst = b->n;
    a.total = b->total;
    switch (b->shape) {
    case 0: batch_kernel<32><<<b->grid[0], kThreads, b->smem, st>>>(a); break;
    case 1: batch_kernel<16><<<b->grid[1], kThreads, b->smem, st>>>(a); break;
    default: batch_kernel<8><<<b->grid[2], kThreads, b->smem, st>>>(a); break;
    }
    BCK(cudaGetLastError(), "batch launch");
    return B2R_OK;
}

}  // namespace

extern "C" {

const char* b2r_batch_last_error(void) { return g_berr; }

b2r_status b2r_batch_create(const b2r_batch_item* items, int n, b2r_batch** out)
{
    if (!items || n <= 0 || !out) return bfail(B2R_ERR_ARG, "invalid batch description");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        const b2r_batch_item& it = items[i];
        if (it.D < 1 || it.D > 4) return bfail(B2R_ERR_ARG, "stencil radius D must be 1..4");
        if (it.nsteps < 0) return bfail(B2R_ERR_ARG, "nsteps must be >= 0");
        for (int a = 0; a < 3; ++a)
            if (it.env[a] < 1) return bfail(B2R_ERR_ARG, "instance sizes must be positive");
    }
    b2r_batch* b = new (std::nothrow) b2r_batch();
    if (!b) return bfail(B2R_ERR_OOM, "host allocation failed");
    b->n = n;
    b->items.assign(items, items + n);
    b->order.resize(n);
    for (int i = 0; i < n; ++i) b->order[i] = i;
    std::stable_sort(b->order.begin(), b->order.end(),
                     [&](int x, int y) { return items[x].nsteps > items[y].nsteps; });
    b->pos.resize(n);
    for (int k = 0; k < n; ++k) b->pos[b->order[k]] = k;
    b->host.resize(n);
    b->maps.resize(2 * n);
    auto bail = [&](b2r_status s) {
        b2r_batch_destroy(b);
        return s;
    };
    for (int k = 0; k < n; ++k) {
        const b2r_batch_item& it = items[b->order[k]];
        InstDev& in = b->host[k];
        const int D = it.D;
        BlockLayout& L = in.L;
        L = BlockLayout{};
        for (int a = 0; a < 3; ++a) {
            L.n[a] = it.env[a] + 2 * D;
            L.B[a] = it.env[a];
            L.nb[a] = 1;
        }
        L.nblk = 1;
        L.H = D;
        L.xoff = roundup(D + 4, 32) - D;
        L.P = roundup(L.xoff + L.n[0] + 8, 32);
        L.periodic = 0;
        L.fixed_edge = 63;
        L.plane = (long long)L.P * L.n[1];
        L.bstride = L.plane * L.n[2];
        in.D = D;
        in.nsteps = it.nsteps;
        in.C = heat_coef(D, it.alpha_dt, it.dx, it.dy, it.dz);
        in.NZ = L.n[2] - 2 * D;
        const size_t fb = (size_t)L.bstride * sizeof(float);
        for (int s = 0; s < 2; ++s) {
            if (cudaMalloc(&in.buf[s], fb) != cudaSuccess)
                return bail(bfail(B2R_ERR_OOM, "instance allocation failed"));
            cudaMemset(in.buf[s], 0, fb);
        }
        b->maxsteps = std::max(b->maxsteps, it.nsteps);
    }
    if (cudaMalloc(&b->d_inst, sizeof(InstDev) * n) != cudaSuccess ||
        cudaMalloc(&b->d_maps, sizeof(CUtensorMap) * 2 * n) != cudaSuccess ||
        cudaMalloc(&b->d_step_off, sizeof(long long) * (b->maxsteps + 1)) != cudaSuccess ||
        cudaMalloc(&b->d_active, sizeof(int) * (b->maxsteps + 1)) != cudaSuccess ||
        cudaMalloc(&b->d_prefix, sizeof(long long) * (n + 1)) != cudaSuccess ||
        cudaMalloc(&b->d_head, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&b->d_done, sizeof(unsigned) * n) != cudaSuccess ||
        cudaMalloc(&b->d_status, sizeof(int)) != cudaSuccess)
        return bail(bfail(B2R_ERR_OOM, "batch table allocation failed"));
    cudaMemset(b->d_status, 0, sizeof(int));
    // persistent grid: every resident slot
    b->smem = kSmem + sizeof(long long) * (b->maxsteps + 1 + n + 1) + sizeof(int) * (b->maxsteps + 1) + 16;
    if (b->smem > 200 * 1024) return bail(bfail(B2R_ERR_ARG, "too many time steps for the batch schedule"));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    {
        const void* fns[3] = {(const void*)batch_kernel<32>, (const void*)batch_kernel<16>,
                              (const void*)batch_kernel<8>};
        // the limit is per function and device: only ever raised, so that a
        // batch with a smaller schedule does not lower it under one created
        // before it
        static SmemLimit limit[3];
        for (int s = 0; s < 3; ++s) {
            int occ = 0;
            if (raise_smem_limit(limit[s], fns[s], b->smem) != cudaSuccess)
                return bail(bfail(B2R_ERR_CUDA, "smem attribute"));
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fns[s], kThreads, b->smem);
            b->grid[s] = std::max(1, occ) * std::max(1, sms);
        }
    }
    b2r_status st = apply_shape(b, default_shape(b));
    if (st != B2R_OK) return bail(st);
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(bfail(B2R_ERR_CUDA, "batch set-up failed"));
    *out = b;
    return B2R_OK;
}

b2r_status b2r_batch_destroy(b2r_batch* b)
{
    if (!b) return B2R_OK;
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (auto& in : b->host)
        for (int s = 0; s < 2; ++s)
            if (in.buf[s]) cudaFree(in.buf[s]);
    cudaFree(b->d_inst);
    cudaFree(b->d_maps);
    cudaFree(b->d_step_off);
    cudaFree(b->d_active);
    cudaFree(b->d_prefix);
    cudaFree(b->d_head);
    cudaFree(b->d_done);
    cudaFree(b->d_status);
    if (b->staging) cudaFree(b->staging);
    delete b;
    return B2R_OK;
}

b2r_status b2r_batch_upload(b2r_batch* b, int i, const float* src, int src_is_device, void* stream)
{
    if (!b || !src || i < 0 || i >= b->n) return bfail(B2R_ERR_ARG, "invalid argument");
    const InstDev& in = b->host[b->pos[i]];
    const BlockLayout& L = in.L;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const cudaMemcpyKind kind = src_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    for (int s = 0; s < 2; ++s)   // both buffers carry the fixed shell
        BCK(cudaMemcpy2DAsync(in.buf[s] + L.xoff, L.P * sizeof(float), src, L.n[0] * sizeof(float),
                              L.n[0] * sizeof(float), (size_t)L.n[1] * L.n[2], kind, st),
            "upload");
    return B2R_OK;
}

b2r_status b2r_batch_download(b2r_batch* b, int i, float* dst, int dst_is_device, void* stream)
{
    if (!b || !dst || i < 0 || i >= b->n) return bfail(B2R_ERR_ARG, "invalid argument");
    const InstDev& in = b->host[b->pos[i]];
    const BlockLayout& L = in.L;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const float* src = in.buf[in.nsteps & 1];
    BCK(cudaMemcpy2DAsync(dst, L.n[0] * sizeof(float), src + L.xoff, L.P * sizeof(float),
                          L.n[0] * sizeof(float), (size_t)L.n[1] * L.n[2],
                          dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st),
        "download");
    if (!dst_is_device) BCK(cudaStreamSynchronize(st), "download sync");
    return B2R_OK;
}

b2r_status b2r_batch_run(b2r_batch* b, void* stream, int use_graph)
{
    if (!b) return bfail(B2R_ERR_ARG, "null batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (use_graph && st) {
        if (!b->gexec || b->gstream != st) {
            if (b->gexec) cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
            BCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
            b2r_status s = enqueue_run(b, st);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (s != B2R_OK) {
                if (g) cudaGraphDestroy(g);
                return s;
            }
            BCK(e, "end capture");
            e = cudaGraphInstantiate(&b->gexec, g, 0);
            cudaGraphDestroy(g);
            BCK(e, "graph instantiate");
            b->gstream = st;
        }
        BCK(cudaGraphLaunch(b->gexec, st), "graph launch");
    } else {
        b2r_status s = enqueue_run(b, st);
        if (s != B2R_OK) return s;
    }
    count_launches(1);
    return B2R_OK;
}

b2r_status b2r_batch_synchronize(b2r_batch* b, void* stream)
{
    if (!b) return bfail(B2R_ERR_ARG, "null batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int s = 0;
    BCK(cudaMemcpyAsync(&s, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, st), "status");
    BCK(cudaStreamSynchronize(st), "sync");
    if (s != DEV_OK) {
        cudaMemset(b->d_status, 0, sizeof(int));
        return bfail(B2R_ERR_TIMEOUT, "a device-side bounded wait of the batch queue gave up");
    }
    return B2R_OK;
}

int64_t b2r_batch_lups(const b2r_batch* b)
{
    if (!b) return 0;
    int64_t s = 0;
    for (const auto& it : b->items) s += (int64_t)it.env[0] * it.env[1] * it.env[2] * it.nsteps;
    return s;
}

b2r_status b2r_batch_set_zchunk(b2r_batch* b, int zchunk)
{
    if (!b || zchunk < 0) return bfail(B2R_ERR_ARG, "invalid argument");
    b->lz_policy = zchunk;
    return build_schedule(b);
}

b2r_status b2r_batch_autotune(b2r_batch* b, void* stream, int* best_zchunk, double* best_ms)
{
    if (!b) return bfail(B2R_ERR_ARG, "null batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the runs overwrite the instance buffers: keep buffer 0 of every instance
    // (freed on every return path)
    struct SaveBufs {
        std::vector<float*> p;
        ~SaveBufs()
        {
            for (float* q : p)
                if (q) cudaFree(q);
        }
    } saved;
    saved.p.assign(b->n, nullptr);
    std::vector<float*>& save = saved.p;
    for (int k = 0; k < b->n; ++k) {
        const size_t fb = (size_t)b->host[k].L.bstride * sizeof(float);
        BCK(cudaMalloc(&save[k], fb), "autotune save");
        BCK(cudaMemcpyAsync(save[k], b->host[k].buf[0], fb, cudaMemcpyDeviceToDevice, st), "save");
    }
    static const int cands[] = {8, 16, 32, 64, 0};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bestz = b->lz_policy, bests = b->shape;
    b2r_status s = B2R_OK;
    for (int c = 0; c < 3 * 5 && s == B2R_OK; ++c) {
        const int sh = c / 5, z = cands[c % 5];
        if (sh != b->shape && (s = apply_shape(b, sh)) != B2R_OK) break;
        if ((s = b2r_batch_set_zchunk(b, z)) != B2R_OK) break;
        for (int k = 0; k < b->n; ++k)
            cudaMemcpyAsync(b->host[k].buf[0], save[k], (size_t)b->host[k].L.bstride * sizeof(float),
                            cudaMemcpyDeviceToDevice, st);
        cudaEventRecord(e0, st);
        if ((s = enqueue_run(b, st)) != B2R_OK) break;
        cudaEventRecord(e1, st);
        if ((s = b2r_batch_synchronize(b, st)) != B2R_OK) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            bestz = z;
            bests = sh;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // restore every instance even after a failed trial; report the first failure
    cudaError_t rerr = cudaSuccess;
    for (int k = 0; k < b->n; ++k) {
        const cudaError_t e = cudaMemcpyAsync(b->host[k].buf[0], save[k],
                                              (size_t)b->host[k].L.bstride * sizeof(float),
                                              cudaMemcpyDeviceToDevice, st);
        if (rerr == cudaSuccess) rerr = e;
    }
    const cudaError_t se = cudaStreamSynchronize(st);
    if (rerr == cudaSuccess) rerr = se;
    if (s != B2R_OK) return s;
    BCK(rerr, "restoring the instances after the trials");
    if (best_zchunk) *best_zchunk = bestz;
    if (best_ms) *best_ms = best;
    if ((s = apply_shape(b, bests)) != B2R_OK) return s;
    return b2r_batch_set_zchunk(b, bestz);
}

b2r_status b2r_batch_set_tile(b2r_batch* b, int width)
{
    if (!b) return bfail(B2R_ERR_ARG, "null batch");
    int s;
    switch (width) {
    case 0: s = default_shape(b); break;
    case 128: s = 0; break;
    case 64: s = 1; break;
    case 32: s = 2; break;
    default: return bfail(B2R_ERR_ARG, "tile width must be 128, 64, 32 or 0");
    }
    return apply_shape(b, s);
}

int b2r_batch_tile(const b2r_batch* b) { return b ? 4 * kLpr[b->shape] : 0; }

}  // extern "C"
