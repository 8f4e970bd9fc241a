// eqwp_batch.cu -- many staggered elastic-wave instances of uneven sizes
// advanced in ONE persistent launch driven by a device work queue
// (work_queue.cuh).  No reference counterpart (the reference runs one model
// per MPI rank).
//
// An instance is a staggered elastic-wave handle of one block with a fixed
// shell (its own fields, material and source).  A time step is two rounds
// of the queue: the velocity stage, then the stress stage, each over the
// tiles x z chunks of the stage kernels' grid (eqwp_stag.cuh, the same
// bodies as the stage launches, so results are bit-identical to stepping
// each handle on its own).  The stages update their fields in place; a round
// starts only after every unit of the instance's previous round has
// finished, which orders both the reads of the neighbours' new values and
// the in-place writes after the previous stage's reads.  The fields are
// read through coherent loads (other CTAs update them between rounds); the
// material through the read-only path.
#include <algorithm>
#include <cstdio>
#include <new>
#include <vector>

#include "api_internal.h"
#include "eqwp_stag.cuh"
#include "work_queue.cuh"

namespace b2r {
namespace {

using namespace eqk;

struct EInst {
    BlockLayout L;
    FieldPtrs F;
    MatPtrs M;
    EqwpStagParams p;          // dt, 1/h, source cell (src_host unused here)
    Tiles T;
    const float* amp;          // source increment of each step of the run (device)
    int gx, gy, bx, by;        // tiles per row / column of the stage grid, CTA shape
    int nsteps, rounds, units;
};

struct EArgs {
    const EInst* inst;                   // sorted by rounds, descending
    const unsigned long long* items;     // the queue: work items in claim order
    unsigned long long* head;
    unsigned* done;
    int* status;
    long long total;
};

constexpr int kEThreads = kBX * kBY;   // 256

__global__ void __launch_bounds__(kEThreads, B2R_EQWP_MINB) eqwp_batch_kernel(const EArgs a)
{
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
                // wait for round t-1 of this instance (bounded)
                s_ok = t == 0 || wq::wait_done(&a.done[k], (unsigned)t * (unsigned)a.inst[k].units);
                s_t = t;
                s_k = k;
                s_u = u;
                s_next = (long long)atomicAdd(a.head, 1ull);   // ready when this one is done
            }
        }
        __syncthreads();
        if (s_cur >= a.total) break;
        if (!s_ok) {
            if (threadIdx.x == 0) report(a.status, DEV_TIMEOUT);
            return;
        }
        const int t = s_t, k = s_k, u = s_u;
        const EInst& in = a.inst[k];
        TilePos q;
        q.dx = in.bx;
        q.dy = in.by;
        q.tx = threadIdx.x % in.bx;
        q.ty = threadIdx.x / in.bx;
        q.bx = u % in.gx;
        const int r = u / in.gx;
        q.by = r % in.gy;
        const int zc = r / in.gy;
        if (q.ty < in.by) {                  // the CTA shape may leave threads over
            if (t & 1)
                stag_stress_unit<false>(in.F, in.F, in.M, in.L, 0, in.T, in.p, in.amp[t >> 1], 0, zc, q);
            else
                stag_velocity_unit<false, false>(in.F, in.F, in.M, in.L, 0, in.T, in.p, AccPtrs{}, 0, zc, q);
        }
        __syncthreads();                     // every store of this unit is issued
        if (threadIdx.x == 0) wq::release_done(&a.done[k]);
    }
}

}  // namespace
}  // namespace b2r

struct b2r_eqwp_batch {
    int n = 0;
    std::vector<b2r_handle*> hs;
    std::vector<int> nsteps;
    std::vector<EInst> host;         // caller order
    std::vector<int> sched;          // queue position -> caller index
    EInst* d_inst = nullptr;
    float* d_amp = nullptr;          // every instance's source increments, back to back
    std::vector<long long> amp_off;  // caller index -> offset in d_amp
    unsigned long long* d_items = nullptr;   // the queue (capacity items_cap)
    long long items_cap = 0;
    unsigned long long* d_head = nullptr;
    unsigned* d_done = nullptr;
    int* d_status = nullptr;
    long long total = 0;
    int lz_policy = -1;              // z chunk cap per unit; -1: by the batch's size (auto_lz)
    int grid = 0;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t gstream = nullptr;
    // stream order with the handles' own streams: the run waits for the work
    // already queued on them, and their next work waits for the run
    std::vector<cudaEvent_t> ev_in;  // per handle
    cudaEvent_t ev_out = nullptr;
};

namespace {

thread_local char g_eberr[512];

b2r_status efail(b2r_status s, const char* msg, cudaError_t e = cudaSuccess)
{
    if (e != cudaSuccess) snprintf(g_eberr, sizeof g_eberr, "%s: %s", msg, cudaGetErrorString(e));
    else snprintf(g_eberr, sizeof g_eberr, "%s", msg);
    return s;
}

#define ECK(call, msg)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            cudaGetLastError();                                                              \
            return efail(e_ == cudaErrorMemoryAllocation ? B2R_ERR_OOM : B2R_ERR_CUDA, msg, e_); \
        }                                                                                    \
    } while (0)

// z chunk of the units when the caller set none: short units keep more of a
// round in flight, which small instances need (16 instances of 32-128 cells
// per edge: 36.9 GLUPS at 8 planes, 26.1 at 32), while large ones have work
// enough in 32-plane units and re-read fewer z-skirt planes with them -- 8
// planes when units of 32 would give fewer than 8 per resident CTA in a
// round, else 32.
static int auto_lz(const b2r_eqwp_batch* b)
{
    long long units = 0;
    for (int k = 0; k < b->n; ++k) {
        const EInst& in = b->host[k];
        int lo, hi;
        stage_region(in.L, edge_bits(in.L, 0), 2, 2, lo, hi);
        const int nz = std::max(1, hi - lo + 1);
        units += (long long)in.gx * in.gy * ((nz + 31) / 32);
    }
    return units < 8LL * b->grid ? 8 : 32;
}

// tiles, z chunks and the queue for the current z-chunk policy
b2r_status build(b2r_eqwp_batch* b)
{
    for (int k = 0; k < b->n; ++k) {
        EInst& in = b->host[k];
        const Grid g = stage_grid(in.L, 2);
        in.T = g.t;
        in.bx = (int)g.b.x;
        in.by = (int)g.b.y;
        in.gx = (int)g.g.x;
        in.gy = (int)g.g.y;
    }
    const int policy = b->lz_policy >= 0 ? b->lz_policy : auto_lz(b);
    for (int k = 0; k < b->n; ++k) {
        EInst& in = b->host[k];
        int lo, hi;
        stage_region(in.L, edge_bits(in.L, 0), 2, 2, lo, hi);
        const int nz = std::max(1, hi - lo + 1);
        const int lz = policy > 0 ? std::min(policy, nz) : nz;
        in.T.nzc = (nz + lz - 1) / lz;
        in.units = in.gx * in.gy * in.T.nzc;
        in.rounds = 2 * in.nsteps;
    }
    b->sched.resize(b->n);
    for (int k = 0; k < b->n; ++k) b->sched[k] = k;
    std::stable_sort(b->sched.begin(), b->sched.end(),
                     [&](int x, int y) { return b->host[x].rounds > b->host[y].rounds; });
    std::vector<EInst> dev(b->n);
    std::vector<int> rounds(b->n), units(b->n);
    for (int j = 0; j < b->n; ++j) {
        dev[j] = b->host[b->sched[j]];
        rounds[j] = dev[j].rounds;
        units[j] = dev[j].units;
    }
    // no run of this batch may still read the queue or the descriptors
    ECK(cudaDeviceSynchronize(), "waiting for the batch's runs");
    std::vector<unsigned long long> items;
    if (!wq::round_major_items(rounds.data(), units.data(), b->n, items))
        return efail(B2R_ERR_ARG, "the batch queue is too long (an instance with more than 2^24 units or "
                                  "rounds, or more than 2^28 work items): split the batch");
    b->total = (long long)items.size();
    if (b->total > b->items_cap) {
        cudaFree(b->d_items);
        b->d_items = nullptr;
        b->items_cap = 0;
        ECK(cudaMalloc(&b->d_items, sizeof(unsigned long long) * std::max<long long>(1, b->total)), "queue allocation");
        b->items_cap = b->total;
    }
    ECK(cudaMemcpy(b->d_inst, dev.data(), sizeof(EInst) * b->n, cudaMemcpyHostToDevice), "copy descriptors");
    if (b->total > 0)
        ECK(cudaMemcpy(b->d_items, items.data(), sizeof(unsigned long long) * b->total, cudaMemcpyHostToDevice),
            "copy the queue");
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    return B2R_OK;
}

b2r_status enqueue(b2r_eqwp_batch* b, cudaStream_t st)
{
    ECK(cudaMemsetAsync(b->d_head, 0, sizeof(unsigned long long), st), "reset queue");
    ECK(cudaMemsetAsync(b->d_done, 0, sizeof(unsigned) * b->n, st), "reset counters");
    EArgs a;
    a.inst = b->d_inst;
    a.items = b->d_items;
    a.head = b->d_head;
    a.done = b->d_done;
    a.status = b->d_status;
    a.total = b->total;
    eqwp_batch_kernel<<<b->grid, kEThreads, 0, st>>>(a);
    ECK(cudaGetLastError(), "batch launch");
    return B2R_OK;
}

}  // namespace

extern "C" {

const char* b2r_eqwp_batch_last_error(void) { return g_eberr; }

b2r_status b2r_eqwp_batch_create(b2r_handle* const* hs, const int* nsteps, int n, b2r_eqwp_batch** out)
{
    if (!hs || !nsteps || n <= 0 || !out) return efail(B2R_ERR_ARG, "invalid batch description");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        const b2r_handle* h = hs[i];
        if (!h) return efail(B2R_ERR_ARG, "null handle");
        if (h->cfg.model != B2R_MODEL_EQWP_STAG)
            return efail(B2R_ERR_ARG, "batched elastic-wave instances must be staggered elastic-wave handles");
        if (h->L.nblk != 1 || h->L.periodic)
            return efail(B2R_ERR_ARG, "batched elastic-wave instances must be one block with a fixed shell");
        if (nsteps[i] < 0) return efail(B2R_ERR_ARG, "nsteps must be >= 0");
        for (int j = 0; j < i; ++j)
            if (hs[j] == h) return efail(B2R_ERR_ARG, "a handle appears twice in the batch");
    }
    b2r_eqwp_batch* b = new (std::nothrow) b2r_eqwp_batch();
    if (!b) return efail(B2R_ERR_OOM, "host allocation failed");
    auto bail = [&](b2r_status s) {
        b2r_eqwp_batch_destroy(b);
        return s;
    };
    b->n = n;
    b->hs.assign(hs, hs + n);
    b->nsteps.assign(nsteps, nsteps + n);
    b->host.resize(n);
    b->amp_off.resize(n + 1, 0);
    for (int k = 0; k < n; ++k) {
        const b2r_handle* h = hs[k];
        EInst& in = b->host[k];
        in.L = h->L;
        for (int f = 0; f < 10; ++f) in.F.p[f] = f < h->nfld ? h->fld[f] : nullptr;
        for (int m = 0; m < 3; ++m) in.M.p[m] = h->mat[m];
        in.p.dt = (float)h->cfg.dt;
        in.p.inv_h = (float)(1.0 / h->cfg.h);
        for (int a = 0; a < 3; ++a) in.p.src[a] = h->cfg.src[a];
        in.p.src_host = nullptr;
        in.p.src_len = 0;
        in.nsteps = nsteps[k];
        b->amp_off[k + 1] = b->amp_off[k] + std::max(1, nsteps[k]);
    }
    const long long namp = b->amp_off[n];
    if (cudaMalloc(&b->d_inst, sizeof(EInst) * n) != cudaSuccess ||
        cudaMalloc(&b->d_amp, sizeof(float) * namp) != cudaSuccess ||
        cudaMalloc(&b->d_head, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&b->d_done, sizeof(unsigned) * n) != cudaSuccess ||
        cudaMalloc(&b->d_status, sizeof(int)) != cudaSuccess)
        return bail(efail(B2R_ERR_OOM, "batch table allocation failed"));
    cudaMemset(b->d_status, 0, sizeof(int));
    cudaMemset(b->d_amp, 0, sizeof(float) * namp);
    b->ev_in.assign(n, nullptr);
    for (int k = 0; k < n; ++k)
        if (cudaEventCreateWithFlags(&b->ev_in[k], cudaEventDisableTiming) != cudaSuccess)
            return bail(efail(B2R_ERR_CUDA, "event creation failed"));
    if (cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming) != cudaSuccess)
        return bail(efail(B2R_ERR_CUDA, "event creation failed"));
    for (int k = 0; k < n; ++k) b->host[k].amp = b->d_amp + b->amp_off[k];
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, eqwp_batch_kernel, kEThreads, 0);
    b->grid = std::max(1, occ) * std::max(1, sms);
    b2r_status st = build(b);
    if (st != B2R_OK) return bail(st);
    *out = b;
    return B2R_OK;
}

b2r_status b2r_eqwp_batch_destroy(b2r_eqwp_batch* b)
{
    if (!b) return B2R_OK;
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (cudaEvent_t e : b->ev_in)
        if (e) cudaEventDestroy(e);
    if (b->ev_out) cudaEventDestroy(b->ev_out);
    cudaFree(b->d_inst);
    cudaFree(b->d_amp);
    cudaFree(b->d_items);
    cudaFree(b->d_head);
    cudaFree(b->d_done);
    cudaFree(b->d_status);
    delete b;
    return B2R_OK;
}

b2r_status b2r_eqwp_batch_run(b2r_eqwp_batch* b, void* stream, int use_graph)
{
    if (!b) return efail(B2R_ERR_ARG, "null batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the work already queued on the handles' streams comes first
    for (int k = 0; k < b->n; ++k) {
        if (b->hs[k]->stream == st) continue;
        ECK(cudaEventRecord(b->ev_in[k], b->hs[k]->stream), "order after the handles' work");
        ECK(cudaStreamWaitEvent(st, b->ev_in[k], 0), "order after the handles' work");
    }
    // the handles' current field sets (a one-pass step swaps a handle's two sets)
    bool moved = false;
    for (int k = 0; k < b->n; ++k)
        for (int f = 0; f < b->hs[k]->nfld; ++f)
            if (b->host[k].F.p[f] != b->hs[k]->fld[f]) {
                b->host[k].F.p[f] = b->hs[k]->fld[f];
                moved = true;
            }
    if (moved) {
        b2r_status s = build(b);
        if (s != B2R_OK) return s;
    }
    std::vector<float> amp((size_t)b->amp_off[b->n], 0.f);
    for (int k = 0; k < b->n; ++k) {
        const b2r_handle* h = b->hs[k];
        for (int s = 0; s < b->nsteps[k]; ++s) {
            const long long ts = h->ts + s;
            if (ts >= 0 && ts < (long long)h->src.size()) amp[b->amp_off[k] + s] = h->src[ts];
        }
    }
    ECK(cudaMemcpyAsync(b->d_amp, amp.data(), sizeof(float) * amp.size(), cudaMemcpyHostToDevice, st),
        "copy source increments");
    if (use_graph && st) {
        if (!b->gexec || b->gstream != st) {
            if (b->gexec) cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
            ECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
            b2r_status s = enqueue(b, st);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (s != B2R_OK) {
                if (g) cudaGraphDestroy(g);
                return s;
            }
            ECK(e, "end capture");
            e = cudaGraphInstantiate(&b->gexec, g, 0);
            cudaGraphDestroy(g);
            ECK(e, "graph instantiate");
            b->gstream = st;
        }
        ECK(cudaGraphLaunch(b->gexec, st), "graph launch");
    } else {
        b2r_status s = enqueue(b, st);
        if (s != B2R_OK) return s;
    }
    count_launches(1);
    // and the handles' next work comes after the run
    ECK(cudaEventRecord(b->ev_out, st), "order the handles' next work");
    for (int k = 0; k < b->n; ++k)
        if (b->hs[k]->stream != st) ECK(cudaStreamWaitEvent(b->hs[k]->stream, b->ev_out, 0), "order the handles' next work");
    for (int k = 0; k < b->n; ++k) {
        b->hs[k]->ts += b->nsteps[k];
        b->hs[k]->halos_fresh = false;
        b->hs[k]->upmask = 0;
    }
    return B2R_OK;
}

b2r_status b2r_eqwp_batch_synchronize(b2r_eqwp_batch* b, void* stream)
{
    if (!b) return efail(B2R_ERR_ARG, "null batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int s = 0;
    ECK(cudaMemcpyAsync(&s, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, st), "status");
    ECK(cudaStreamSynchronize(st), "sync");
    if (s != DEV_OK) {
        cudaMemset(b->d_status, 0, sizeof(int));
        return efail(B2R_ERR_TIMEOUT, "a device-side bounded wait of the batch queue gave up");
    }
    return B2R_OK;
}

int64_t b2r_eqwp_batch_lups(const b2r_eqwp_batch* b)
{
    if (!b) return 0;
    int64_t s = 0;
    for (int k = 0; k < b->n; ++k) {
        const int* e = b->hs[k]->cfg.env;
        s += (int64_t)e[0] * e[1] * e[2] * b->nsteps[k];
    }
    return s;
}

b2r_status b2r_eqwp_batch_set_zchunk(b2r_eqwp_batch* b, int zchunk)
{
    if (!b || zchunk < 0) return efail(B2R_ERR_ARG, "invalid argument");
    b->lz_policy = zchunk;
    return build(b);
}

}  // extern "C"
