// batch.cu -- many independent heat instances of uneven sizes and stencil
// orders advanced in ONE persistent launch driven by a device work queue.
//
// No reference counterpart (the reference runs one model per MPI rank); each
// instance is a single-block heat domain with a fixed shell, stepped with the
// scheme of heat-3D.cu:228-231/315-318/410-413/514-517 exactly as the plain
// sweep does, so results are bit-identical to per-instance plain runs.
//
// Work items (round t, instance k, unit u) go through the device work queue
// of work_queue.cuh.  A round is one time step of an instance on one-step
// units (heat_unit.cuh, tile shape per instance) or two of an instance on
// two-step units (heat2_unit.cuh, radius 1; the last round of an odd step
// count takes one), chosen per (order, size class) by the autotuner.
#include <algorithm>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "heat2_unit.cuh"
#include "heat_unit.cuh"
#include "work_queue.cuh"

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
static_assert(kSlot >= h2k::kPlane, "the two-step units stream through the same ring slots");
constexpr size_t kSmem = size_t(kS) * kSlot * sizeof(float) + kS * sizeof(uint64_t) + 16 + 128;
// the two-step units' two stage-1 planes, after the schedule tables
constexpr size_t kSmemS1 = 2 * size_t(h2k::kP1) * sizeof(float) + 128;
// tile shapes 0..2: one step per unit, LPR lanes per row = 32, 16, 8 -> 128,
// 64, 32 cells wide; shape 3: two steps per unit on 128 x 16-cell tiles
// (radius 1 only, heat2_unit.cuh)
constexpr int kShapes = 4;
constexpr int kTwoStep = 3;
constexpr int kLpr[kShapes] = {32, 16, 8, 32};
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
    int shape;                           // tile shape: index into kLpr
    int lpr;                             // its lanes per tile row (kLpr[shape])
    int tb;                              // time steps per unit: 1, or 2 (shape kTwoStep)
    int rounds;                          // rounds of units: nsteps / tb, rounded up
};

struct BatchArgs {
    const InstDev* inst;                 // sorted by rounds, descending
    const CUtensorMap* maps;             // 2 per instance: buffer 0, buffer 1
    const unsigned long long* items;     // the queue: work items in claim order
    unsigned long long* head;            // next item (zeroed per run)
    unsigned* done;                      // finished units per instance (zeroed per run)
    int* status;
    long long total;
};

// the four unit bodies are inlined into the kernel (measured faster than
// separate calls, whose calling convention spills the register queues)
#ifdef B2R_BATCH_NOINLINE
#define B2R_UNIT_INLINE __noinline__
#else
#define B2R_UNIT_INLINE __forceinline__
#endif
// the tile shape is the instance's own (run time), so that instances of
// different shapes share the launch
template <int D>
__device__ B2R_UNIT_INLINE bool run_unit(const BatchArgs& a, const InstDev& in, int k, int t, int u,
                                         heatk::Ring& rg)
{
    const int tx = u % in.ntx;
    const int r = u / in.ntx;
    const int ty = r % in.nty;
    const int zc = r / in.nty;
    const int zi0 = zc * in.Lz;
    const int zi1 = min(in.NZ, zi0 + in.Lz);
    return heatk::sweep_unit<D, RowsPerWarp<D>::value, kS, kSlot, 0>(
        &a.maps[2 * k + (t & 1)], in.buf[(t + 1) & 1], in.L, 0, in.C, 0, tx, ty, zi0, zi1, rg, in.lpr);
}

// A two-step unit: round t = sub-steps 2t, 2t+1 (the last round of an odd
// step count: 2t only), through the same ring (positions gp, issued_hi,
// stop in, updated positions and the success flag out).  Not inlined: its
// register queues would otherwise share the budget of the one-step units'.
__device__ __noinline__ uint4 run_two_step(const BatchArgs& a, int k, int t, int u, unsigned gp,
                                           unsigned issued_hi, unsigned stop, float* s1, float* ring)
{
    const InstDev& in = a.inst[k];
    h2k::H2Ctx c;
    c.ring = ring;
    c.s1 = s1;
    c.bar = reinterpret_cast<uint64_t*>(ring + kS * kSlot);
    c.abort_flag = reinterpret_cast<int*>(c.bar + kS);
    c.tid = threadIdx.x;
    c.lane = threadIdx.x & 31;
    c.warp = threadIdx.x >> 5;
    c.C = in.C;
    c.plane = in.L.plane;
    c.P = in.L.P;
    c.gp = gp;
    c.issued_hi = issued_hi;
    c.stop = stop;
    c.aborted = false;
    const int tx = u % in.ntx, r = u / in.ntx, ty = r % in.nty, zc = r / in.nty;
    const bool ok = h2k::h2_unit<kS, kSlot>(c, &a.maps[2 * k + (t & 1)], in.buf[(t + 1) & 1], in.L, 0, 0, tx,
                                            ty, zc * in.Lz, in.Lz, 2 * t + 1 == in.nsteps);
    return make_uint4(c.gp, c.issued_hi, c.stop, ok ? 1u : 0u);
}

#ifndef B2R_BATCH_MINB
#define B2R_BATCH_MINB 2   // resident CTAs per SM the register budget is fitted to (no spills)
#endif
// TWO: some instance runs on two-step units (a separate instantiation, so
// that runs without them keep the one-step units' register allocation)
template <bool TWO>
__global__ void __launch_bounds__(kThreads, B2R_BATCH_MINB) batch_kernel(const BatchArgs a)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    heatk::Ring rg;
    heatk::ring_init<kS, kSlot>(rg, smem_raw);
    // the two-step units' stage-1 planes after the ring (which ends 16 bytes
    // after its barriers), 128-byte aligned
    float* s1 = reinterpret_cast<float*>(
        (reinterpret_cast<uintptr_t>(rg.abort_flag) + 16 + 127) & ~uintptr_t(127));
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
            wq::unpack_item(a.items[item], t, k, u);
            int ok = 1;
            // wait for round t-1 of this instance (bounded)
            if (t > 0) ok = wq::wait_done(&a.done[k], (unsigned)t * (unsigned)a.inst[k].units) ? 1 : 0;
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
        if (TWO && in.tb == 2) {
            const uint4 r = run_two_step(a, k, t, u, rg.gp, rg.issued_hi, rg.stop, s1, rg.smem);
            rg.gp = r.x;
            rg.issued_hi = r.y;
            rg.stop = r.z;
            ok = r.w != 0;
        } else switch (in.D) {
        case 1: ok = run_unit<1>(a, in, k, t, u, rg); break;
        case 2: ok = run_unit<2>(a, in, k, t, u, rg); break;
        case 3: ok = run_unit<3>(a, in, k, t, u, rg); break;
        default: ok = run_unit<4>(a, in, k, t, u, rg); break;
        }
        if (!ok) {
            if (threadIdx.x == 0) report(a.status, DEV_TIMEOUT);
            heatk::ring_drain<kS>(rg);
            return;
        }
        __syncthreads();                     // every store of this unit is issued
        if (threadIdx.x == 0) wq::release_done(&a.done[k]);
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
    std::vector<InstDev> host;       // sorted by step count
    std::vector<CUtensorMap> maps;   // sorted by step count, 2 per instance
    std::vector<int> sched;          // queue position -> host index (by rounds, descending)
    InstDev* d_inst = nullptr;
    CUtensorMap* d_maps = nullptr;
    unsigned long long* d_items = nullptr;   // the queue (capacity items_cap)
    long long items_cap = 0;
    unsigned long long* d_head = nullptr;
    unsigned* d_done = nullptr;
    int* d_status = nullptr;
    float* staging = nullptr;
    size_t staging_bytes = 0;
    int maxrounds = 0;               // rounds of the current schedule's longest instance
    long long total = 0;
    int lz_policy = 16;              // z chunk cap per unit (autotuned)
    int grid[2] = {0, 0};            // persistent grid (every resident slot) per kernel variant
    bool two = false;                // some instance runs on two-step units
    size_t smem = 0;                 // ring + the two-step units' planes
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

// The tile shape of instance k: the fewest cells computed per plane, narrow
// tiles paying a little for their wider skirt (their boxes re-read a larger
// share of the neighbouring tiles).
int default_shape(const b2r_batch* b, int k)
{
    static const double penalty[3] = {1.0, 1.03, 1.08};
    int best = 0;
    double bc = 1e300;
    for (int s = 0; s < 3; ++s) {
        const double c = (double)plane_cells(b, k, s) * penalty[s];
        if (c < bc - 1e-9) {
            bc = c;
            best = s;
        }
    }
    return best;
}

std::vector<int> default_shapes(const b2r_batch* b)
{
    std::vector<int> sh(b->n);
    for (int k = 0; k < b->n; ++k) sh[k] = default_shape(b, k);
    return sh;
}

b2r_status build_schedule(b2r_batch* b);

// tile counts, steps per unit and tensor-map boxes of every instance for
// its shape sh[k] (two-step units for radius 1 only)
b2r_status apply_shapes(b2r_batch* b, const std::vector<int>& sh)
{
    for (int k = 0; k < b->n; ++k) {
        InstDev& in = b->host[k];
        const BlockLayout& L = in.L;
        const int D = in.D;
        const int s = (sh[k] == kTwoStep && D != 1) ? default_shape(b, k) : sh[k];
        in.shape = s;
        in.lpr = kLpr[s];
        int bw, bh;
        if (s == kTwoStep) {
            in.tb = 2;
            in.ntx = h2k::h2_ntx(L);
            in.nty = h2k::h2_nty(L);
            bw = h2k::kBoxW;
            bh = h2k::kBoxH;
        } else {
            in.tb = 1;
            const int X = L.xoff + L.n[0] - D - ((L.xoff + D) & ~3), Y = L.n[1] - 2 * D;
            const int tw = 4 * kLpr[s], th = kTileY[D][s];
            in.ntx = (X + tw - 1) / tw;
            in.nty = (Y + th - 1) / th;
            bw = tw + 8;
            bh = kBoxH[D][s];
        }
        in.rounds = (in.nsteps + in.tb - 1) / in.tb;
        for (int f = 0; f < 2; ++f)
            if (!make_block_tmap(&b->maps[2 * k + f], in.buf[f], L, 4, bw, bh, 1))
                return bfail(B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    }
    return build_schedule(b);
}

b2r_status apply_shape(b2r_batch* b, int s) { return apply_shapes(b, std::vector<int>(b->n, s)); }

// The queue for the current shapes and Lz policy: work items (round,
// instance, unit) written out in claim order, round-major.  A round is one
// step of a one-step instance or two of a two-step one; the instances are
// sorted by their round count (descending), so those still stepping at round
// t are a prefix.  A unit waits only for the previous round of its own
// instance, which the queue holds earlier, so the queue cannot deadlock.
b2r_status build_schedule(b2r_batch* b)
{
    b->sched.resize(b->n);
    for (int k = 0; k < b->n; ++k) b->sched[k] = k;
    std::stable_sort(b->sched.begin(), b->sched.end(),
                     [&](int x, int y) { return b->host[x].rounds > b->host[y].rounds; });
    std::vector<InstDev> dev(b->n);
    std::vector<CUtensorMap> maps(2 * b->n);
    b->maxrounds = 0;
    b->two = false;
    for (int j = 0; j < b->n; ++j) {
        InstDev& in = b->host[b->sched[j]];
        b->two = b->two || in.tb == 2;
        in.Lz = std::min(in.NZ, b->lz_policy > 0 ? b->lz_policy : in.NZ);
        in.nzc = (in.NZ + in.Lz - 1) / in.Lz;
        in.units = in.ntx * in.nty * in.nzc;
        dev[j] = in;
        maps[2 * j] = b->maps[2 * b->sched[j]];
        maps[2 * j + 1] = b->maps[2 * b->sched[j] + 1];
        b->maxrounds = std::max(b->maxrounds, in.rounds);
    }
    // no run of this batch may still read the queue or the descriptors
    BCK(cudaDeviceSynchronize(), "waiting for the batch's runs");
    std::vector<int> rounds(b->n), units(b->n);
    for (int j = 0; j < b->n; ++j) {
        rounds[j] = dev[j].rounds;
        units[j] = dev[j].units;
    }
    std::vector<unsigned long long> items;
    if (!wq::round_major_items(rounds.data(), units.data(), b->n, items))
        return bfail(B2R_ERR_ARG, "the batch queue is too long (an instance with more than 2^24 units or "
                                  "rounds, or more than 2^28 work items): split the batch");
    b->total = (long long)items.size();
    if (b->total > b->items_cap) {
        cudaFree(b->d_items);
        b->d_items = nullptr;
        b->items_cap = 0;
        BCK(cudaMalloc(&b->d_items, sizeof(unsigned long long) * std::max<long long>(1, b->total)), "queue allocation");
        b->items_cap = b->total;
    }
    BCK(cudaMemcpy(b->d_inst, dev.data(), sizeof(InstDev) * b->n, cudaMemcpyHostToDevice), "copy descriptors");
    BCK(cudaMemcpy(b->d_maps, maps.data(), sizeof(CUtensorMap) * 2 * b->n, cudaMemcpyHostToDevice),
        "copy tensor maps");
    if (b->total > 0)
        BCK(cudaMemcpy(b->d_items, items.data(), sizeof(unsigned long long) * b->total, cudaMemcpyHostToDevice),
            "copy the queue");
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
    a.items = b->d_items;
    a.head = b->d_head;
    a.done = b->d_done;
    a.status = b->d_status;
    a.total = b->total;
    if (b->two) batch_kernel<true><<<b->grid[1], kThreads, b->smem, st>>>(a);
    else batch_kernel<false><<<b->grid[0], kThreads, b->smem, st>>>(a);
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
    }
    if (cudaMalloc(&b->d_inst, sizeof(InstDev) * n) != cudaSuccess ||
        cudaMalloc(&b->d_maps, sizeof(CUtensorMap) * 2 * n) != cudaSuccess ||
        cudaMalloc(&b->d_head, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&b->d_done, sizeof(unsigned) * n) != cudaSuccess ||
        cudaMalloc(&b->d_status, sizeof(int)) != cudaSuccess)
        return bail(bfail(B2R_ERR_OOM, "batch table allocation failed"));
    cudaMemset(b->d_status, 0, sizeof(int));
    // persistent grid: every resident slot
    b->smem = kSmem + 16 + kSmemS1;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    {
        // the limit is per function and device: only ever raised, so that a
        // batch with a smaller schedule does not lower it under one created
        // before it
        static SmemLimit limit[2];
        const void* fns[2] = {(const void*)batch_kernel<false>, (const void*)batch_kernel<true>};
        for (int v = 0; v < 2; ++v) {
            int occ = 0;
            if (raise_smem_limit(limit[v], fns[v], b->smem) != cudaSuccess)
                return bail(bfail(B2R_ERR_CUDA, "smem attribute"));
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fns[v], kThreads, b->smem);
            b->grid[v] = std::max(1, occ) * std::max(1, sms);
        }
    }
    b2r_status st = apply_shapes(b, default_shapes(b));
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
    cudaFree(b->d_items);
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
    const float* src = in.buf[in.rounds & 1];
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
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // one whole run from the saved inputs, timed
    auto trial = [&](float& ms) -> b2r_status {
        for (int k = 0; k < b->n; ++k)
            cudaMemcpyAsync(b->host[k].buf[0], save[k], (size_t)b->host[k].L.bstride * sizeof(float),
                            cudaMemcpyDeviceToDevice, st);
        cudaEventRecord(e0, st);
        b2r_status r = enqueue_run(b, st);
        if (r != B2R_OK) return r;
        cudaEventRecord(e1, st);
        if ((r = b2r_batch_synchronize(b, st)) != B2R_OK) return r;
        cudaEventElapsedTime(&ms, e0, e1);
        return B2R_OK;
    };
    static const int cands[] = {8, 16, 32, 64, 0};
    float best = 1e30f;
    int bestz = b->lz_policy;
    // the z-chunk cap for the current shapes (a change must gain 0.5 %)
    auto tune_zchunk = [&]() -> b2r_status {
        for (int c = 0; c < 5; ++c) {
            float ms = 0.f;
            b2r_status r = b2r_batch_set_zchunk(b, cands[c]);
            if (r == B2R_OK) r = trial(ms);
            if (r != B2R_OK) return r;
            if (ms < best * (cands[c] == bestz ? 1.f : 0.995f)) {
                best = ms;
                bestz = cands[c];
            }
        }
        return b2r_batch_set_zchunk(b, bestz);
    };
    // 1. the z-chunk cap with every instance on its fewest-cells shape
    std::vector<int> sh = default_shapes(b);
    b2r_status s = apply_shapes(b, sh);
    if (s == B2R_OK) s = tune_zchunk();
    // 2. tile shapes per (stencil order, size class): the instances of one
    // class try each other shape while the rest keep theirs (radius 1 also
    // the two-step units); the size class is the interior width (the extent
    // a tile width divides)
    auto cls = [&](int k) {
        const int w = b->items[b->order[k]].env[0];
        return (b->host[k].D - 1) * 3 + (w <= 64 ? 0 : (w <= 128 ? 1 : 2));
    };
    bool changed = false;
    for (int c = 0; c < 12 && s == B2R_OK; ++c)
        for (int t = 0; t < kShapes && s == B2R_OK; ++t) {
            if (t == kTwoStep && c >= 3) continue;      // two-step units: radius 1 only
            std::vector<int> cand = sh;
            bool differs = false;
            for (int k = 0; k < b->n; ++k)
                if (cls(k) == c && cand[k] != t) {
                    cand[k] = t;
                    differs = true;
                }
            if (!differs) continue;
            float ms = 0.f;
            if ((s = apply_shapes(b, cand)) != B2R_OK || (s = trial(ms)) != B2R_OK) break;
            if (ms < best * 0.995f) {
                best = ms;
                sh = cand;
                changed = true;
            }
        }
    // 3. the z-chunk cap again for the shapes picked
    if (s == B2R_OK) s = apply_shapes(b, sh);
    if (s == B2R_OK && changed) s = tune_zchunk();
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
    return B2R_OK;
}

b2r_status b2r_batch_set_tile(b2r_batch* b, int width)
{
    if (!b) return bfail(B2R_ERR_ARG, "null batch");
    switch (width) {
    case 0: return apply_shapes(b, default_shapes(b));
    case 128: return apply_shape(b, 0);
    case 64: return apply_shape(b, 1);
    case 32: return apply_shape(b, 2);
    default: return bfail(B2R_ERR_ARG, "tile width must be 128, 64, 32 or 0");
    }
}

int b2r_batch_tile(const b2r_batch* b)
{
    if (!b) return 0;
    for (int k = 1; k < b->n; ++k)
        if (b->host[k].lpr != b->host[0].lpr) return 0;
    return 4 * b->host[0].lpr;
}

int b2r_batch_instance_tile(const b2r_batch* b, int i)
{
    return b && i >= 0 && i < b->n ? 4 * b->host[b->pos[i]].lpr : 0;
}

b2r_status b2r_batch_set_pass_steps(b2r_batch* b, int steps)
{
    if (!b) return bfail(B2R_ERR_ARG, "null batch");
    if (steps != 1 && steps != 2) return bfail(B2R_ERR_ARG, "steps per pass must be 1 or 2");
    std::vector<int> sh(b->n);
    for (int k = 0; k < b->n; ++k)
        sh[k] = b->host[k].D == 1 ? (steps == 2 ? kTwoStep : default_shape(b, k)) : b->host[k].shape;
    return apply_shapes(b, sh);
}

int b2r_batch_instance_pass_steps(const b2r_batch* b, int i)
{
    return b && i >= 0 && i < b->n ? b->host[b->pos[i]].tb : 0;
}

}  // extern "C"
