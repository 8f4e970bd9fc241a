// api_internal.h -- what the translation units of the C ABI share: the
// handle, the error helper and the period driver (b2r_api.cu); the
// autotuners (api_tune.cu) and the adjoint drivers (api_adjoint.cu) use them.
#pragma once
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <map>
#include <mutex>
#include <algorithm>
#include <string>
#include <tuple>
#include <vector>
#include <cudaTypedefs.h>
#include "b2r_common.cuh"
#include "eqwp.h"
#include "gol.h"
#include "halo.h"
#include "heat.h"

using namespace b2r;

struct b2r_handle {
    b2r_config cfg{};
    BlockLayout L{};
    int cell_bytes = 4;
    int shell = 1;              // depth of the fixed shell in domain arrays
    cudaStream_t stream = nullptr;
    // heat / GoL: one field, two ping-pong buffers
    void* buf[2] = {nullptr, nullptr};
    int cur = 0;
    CUtensorMap tmap[2];
    CUtensorMap tmap2[2];       // boxes of the two-step kernel (D = 1)
    CUtensorMap tmap3[2];       // boxes of the several-step kernel's 128 x 32 tiles (D = 1) or of the radius-2 two-step kernel
    CUtensorMap tmap4[2];       // boxes of its 64 x 64 tiles
    HeatCoef hc{};
    HeatTune tune{};
    // elastic wave: fields and material
    float* fld[kMaxFields] = {};
    int nfld = 0;
    // staggered model: the second field set of the one-pass step (v^n, s^n
    // -> v^{n+1}, s^{n+1} out of place) and tensor maps of both sets'
    // stresses; fld is always the current set
    float* fld2[kMaxFields] = {};
    StressMaps smaps[2];
    bool eqwp_fused = false;   // two-pass by default: faster on this GPU so far
    bool eqwp_tma = false;     // two-pass: the stress stage with TMA-streamed inputs (eqwp_tma.cu)
    // two-pass, several blocks: the halo exchange of the next period runs on
    // the stream xs while the last stress stage of a period finishes the
    // tiles that the exchange does not read (opt-in: on one GPU the exchange
    // is a copy that competes for the same HBM, and the split stage costs
    // more than the overlap returns)
    bool eqwp_overlap = false;
    bool xdone = false;        // the last sub-step issued the next period's exchange
    cudaStream_t xs = nullptr;
    cudaEvent_t xev[2] = {};   // [band tiles done, exchange done]
    std::map<int, EqwpStressMaps> emaps;   // its tensor maps per tile width (threads per row), built
    const void* emaps_of[11] = {};         // for the field pointers in emaps_of
    bool gol_bytes = false;    // Game of Life: byte-SWAR kernel instead of bit-sliced cells
    bool adj_fused = true;     // adjoint: stress adjoint + lambda/mu gradients in one sweep
    bool gol_push = false;     // Game of Life: period-end passes fill the next period's halos (opt-in: slower so far)
    int gol_rows = 0;          // Game of Life several-generation pass: output rows per band at most (0 = 32)
    float* mat[3] = {};
    std::vector<float> src;     // per-step source increment of sxx/syy/szz (STAG)
    void* staging = nullptr;
    size_t staging_bytes = 0;
    // pipelined host runs: two input and two output device buffers, a copy
    // stream per direction, and the events that order them
    void* pipe[4] = {};
    size_t pipe_bytes = 0;
    cudaStream_t cin = nullptr, cout = nullptr;
    cudaEvent_t ev[4][2] = {};   // [in ready, input consumed, output gathered, output copied][slot]
    void* bounce = nullptr;
    size_t bounce_bytes = 0;
    int* d_status = nullptr;
    long long ts = 0;
    bool halos_fresh = false;
    unsigned upmask = 0;         // fields uploaded since the last step while the halos were not fresh
    unsigned xmask = 0;          // fields exchanged by the caller at time step xts
    long long xts = -1;
    // CUDA graphs of whole periods (heat, GoL on a non-default stream)
    bool graphs = true;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};   // by ping-pong buffer at start
    bool gflip[2] = {false, false};                   // the graph ends on the other buffer
    int gsteps = 0;                                   // time steps per graph launch
    long long gkernels = 0;                           // kernels per graph launch
    // misfit-gradient workspace (checkpoints, replay, adjoint fields, FP64
    // gradients), kept for the next call on this handle
    void* adj_ws = nullptr;
    size_t adj_ws_bytes = 0;
    std::string err;
};

namespace b2r_api __attribute__((visibility("hidden"))) {

struct TuneKey {
    int model, D, n0, n1, n2, nblk;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(model, D, n0, n1, n2, nblk) < std::tie(o.model, o.D, o.n0, o.n1, o.n2, o.nblk);
    }
};

#define CK(h, call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            cudaGetLastError(); /* a non-sticky error must not resurface in a later check */ \
            return fail(h, e_ == cudaErrorMemoryAllocation ? B2R_ERR_OOM : B2R_ERR_CUDA,     \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
        }                                                                                    \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
};

// Two timing events, destroyed on every return path.
struct EventPair {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    EventPair() = default;
    EventPair(const EventPair&) = delete;
    EventPair& operator=(const EventPair&) = delete;
    cudaError_t create()
    {
        cudaError_t e = cudaEventCreate(&e0);
        if (e != cudaSuccess) {
            e0 = nullptr;
            return e;
        }
        e = cudaEventCreate(&e1);
        if (e != cudaSuccess) e1 = nullptr;
        return e;
    }
    // seconds between the two recorded events (0 when unavailable)
    double seconds() const
    {
        float ms = 0.f;
        return cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess ? ms / 1000.0 : 0.0;
    }
    ~EventPair()
    {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
};

inline int roundup(int v, int m) { return (v + m - 1) / m * m; }

extern std::mutex g_tune_mu;
extern std::map<TuneKey, HeatTune> g_tune_cache;
TuneKey key_of(const b2r_handle* h);
extern thread_local std::string g_err;
b2r_status fail(b2r_handle* h, b2r_status s, const char* fmt, ...);
int halo_per_step(const b2r_config& c);
void fill_layout(BlockLayout& L, const int n[3], const int B[3], const int nb[3], int H, int cell_bytes,
                 int periodic, int fixed_edge);
size_t field_bytes(const b2r_handle* h);
size_t domain_cells(const b2r_handle* h);
b2r_status ensure_kappa(b2r_handle* h);
b2r_status ensure_staging(b2r_handle* h, size_t bytes);
b2r_status build_heat_maps(b2r_handle* h);
int heat_pass_steps(const b2r_handle* h, int i, int left);
int gol_pass_gens(const b2r_handle* h, int i, int left);
b2r_status check_status(b2r_handle* h);
b2r_status exchange_all(b2r_handle* h, bool staged, cudaStream_t xst = nullptr);   // xst: another stream than the handle's
b2r_status exchange_one(b2r_handle* h, int field, bool staged);
EqwpStagParams stag_params(const b2r_handle* h);
// One sub-step i of a period.  xnext: the caller starts the next period
// without an exchange if h->xdone is set afterwards (the sub-step may then
// issue that exchange itself, overlapped with its last stage).
b2r_status substep(b2r_handle* h, int i, bool xnext = false);
b2r_status substep2(b2r_handle* h, int i);
void drop_graphs(b2r_handle* h);
b2r_status advance(b2r_handle* h, int n);
b2r_status capture_graph(b2r_handle* h, int c, int periods);

// heat_3D_gpu_main on one host block, in two halves so that host work can
// run between them: begin() allocates the two ping-pong device blocks and
// the status word, copies the block in (both buffers) and enqueues the R
// shrinking sub-steps on st; end() copies planes [R*D, Ngz-R*D) of the
// result into h_out and waits for the stream.  edge: the fixed-shell face
// bits of BlockLayout::fixed_edge.  The destructor frees what begin()
// allocated.
struct HeatBlockRun {
    BlockLayout L{};
    void* buf[2] = {nullptr, nullptr};
    void* status = nullptr;
    EventPair ev;
    cudaStream_t st = nullptr;
    int R = 0, H = 0, Ngz = 0, cur = 0;
    HeatBlockRun() = default;
    HeatBlockRun(const HeatBlockRun&) = delete;
    HeatBlockRun& operator=(const HeatBlockRun&) = delete;
    b2r_status begin(const float* h_in, int R, int D, int edge, int Ngx, int Ngy, int Ngz, double alpha_dt,
                     double dx, double dy, double dz, cudaStream_t st);
    b2r_status end(float* h_out, double* gpu_seconds);
    ~HeatBlockRun();
};
// edge_flag[3] in {-1, 0, 1} (NULL: 0, 0, 0) as face bits
int edge_bits_of_flags(const char* edge_flag);

}  // namespace b2r_api
