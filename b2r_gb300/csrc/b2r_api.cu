// b2r_api.cu -- the C ABI of libb2r (include/b2r.h): handles, geometry,
// device memory of the resident subdomains, the period driver (halo
// exchange + R sub-steps, b2r.cpp:179-221) and the reference-shaped per-block
// entries (heat_3D_gpu_main, gol_3D_gpu_main, eqwp_gpu_main).
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
    bool gol_bytes = false;    // Game of Life: byte-SWAR kernel instead of bit-sliced cells
    bool adj_fused = true;     // adjoint: stress adjoint + lambda/mu gradients in one sweep
    bool gol_push = false;     // Game of Life: period-end passes fill the next period's halos (opt-in: slower so far)
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

namespace {

// autotuning results per (model, D, block size, blocks), shared by handles

struct TuneKey {
    int model, D, n0, n1, n2, nblk;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(model, D, n0, n1, n2, nblk) < std::tie(o.model, o.D, o.n0, o.n1, o.n2, o.nblk);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, HeatTune> g_tune_cache;

TuneKey key_of(const b2r_handle* h)
{
    return TuneKey{h->cfg.model, h->cfg.D, h->L.n[0], h->L.n[1], h->L.n[2], h->L.nblk};
}


thread_local std::string g_err;

b2r_status fail(b2r_handle* h, b2r_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    g_err = buf;
    return s;
}

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

inline int roundup(int v, int m) { return (v + m - 1) / m * m; }

// cells consumed from the halo by one time step
int halo_per_step(const b2r_config& c)
{
    switch (c.model) {
    case B2R_MODEL_HEAT: return c.D;
    case B2R_MODEL_GOL: return 1;
    default: return 2 * c.D;   // elastic wave: two stages of radius D
    }
}

void fill_layout(BlockLayout& L, const int n[3], const int B[3], const int nb[3], int H,
                 int cell_bytes, int periodic, int fixed_edge)
{
    const int A = 128 / cell_bytes;      // 128-byte row alignment
    const int m = 16 / cell_bytes;       // >= 16 bytes of pad before x = 0
    for (int a = 0; a < 3; ++a) {
        L.n[a] = n[a];
        L.B[a] = B[a];
        L.nb[a] = nb[a];
    }
    L.nblk = nb[0] * nb[1] * nb[2];
    L.H = H;
    L.xoff = roundup(H + m, A) - H;
    L.P = roundup(L.xoff + n[0] + 2 * m, A);   // >= 32 bytes of pad after the row
    L.periodic = periodic;
    L.fixed_edge = fixed_edge;
    L.plane = (long long)L.P * n[1];
    L.bstride = L.plane * n[2];
}

size_t field_bytes(const b2r_handle* h) { return (size_t)h->L.bstride * h->L.nblk * h->cell_bytes; }

size_t domain_cells(const b2r_handle* h)
{
    size_t c = 1;
    for (int a = 0; a < 3; ++a) c *= (size_t)(h->cfg.env[a] + 2 * h->shell);
    return c;
}


// the heat model's conductivity field, allocated on first use and set to 1
b2r_status ensure_kappa(b2r_handle* h)
{
    if (h->mat[0]) return B2R_OK;
    const size_t fb = field_bytes(h);
    CK(h, cudaMalloc(&h->mat[0], fb));
    CK(h, launch_fill(h->mat[0], fb / sizeof(float), 1.0f, h->stream));
    return B2R_OK;
}

b2r_status ensure_staging(b2r_handle* h, size_t bytes)
{
    if (h->staging_bytes >= bytes) return B2R_OK;
    if (h->staging) cudaFree(h->staging);
    h->staging = nullptr;
    h->staging_bytes = 0;
    CK(h, cudaMalloc(&h->staging, bytes));
    h->staging_bytes = bytes;
    return B2R_OK;
}

b2r_status build_heat_maps(b2r_handle* h)
{
    for (int b = 0; b < 2; ++b) {
        if (!make_block_tmap(&h->tmap[b], h->buf[b], h->L, 4, heat_box_w(), heat_box_h(h->cfg.D), 1))
            return fail(h, B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed for the heat field");
        if (h->cfg.D == 1 &&
            !make_block_tmap(&h->tmap2[b], h->buf[b], h->L, 4, heat2_box_w(), heat2_box_h(), 1))
            return fail(h, B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed for the heat field");
    }
    return B2R_OK;
}

// Can sub-steps i and i+1 run in one two-step launch?  Radius 1 only, and no
// halo exchange may fall between them: within one period, or always when the
// exchange is empty (one block, not periodic).
bool heat_fuse_ok(const b2r_handle* h, int i)
{
    if (h->cfg.model != B2R_MODEL_HEAT || h->cfg.D != 1 || h->tune.tblock < 2) return false;
    if (h->L.nblk == 1 && !h->L.periodic) return true;
    return i + 1 < h->cfg.R;
}

// Game of Life generations that one pass may advance from sub-step i with
// `left` steps to go: up to the period's end (no exchange in between), or
// unbounded when the exchange is empty; 1 = the one-generation kernel.
// Bit-sliced cells take several generations per pass by default (tblock >=
// 2); byte cells only with tblock >= 4 (slower than one per pass so far).
int gol_pass_gens(const b2r_handle* h, int i, int left)
{
    if (h->cfg.model != B2R_MODEL_GOL || h->tune.tblock < (h->gol_bytes ? 4 : 2)) return 1;
    int g = std::min(left, h->gol_bytes ? gol_max_generations_per_pass() : gol_bits_max_generations_per_pass());
    if (!(h->L.nblk == 1 && !h->L.periodic)) g = std::min(g, h->cfg.R - i);
    return std::max(g, 1);
}

b2r_status check_status(b2r_handle* h)
{
    int s = 0;
    CK(h, cudaMemcpyAsync(&s, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (s != DEV_OK) {
        int zero = 0;
        cudaMemcpy(h->d_status, &zero, sizeof(int), cudaMemcpyHostToDevice);
        return fail(h, B2R_ERR_TIMEOUT, "a device-side bounded wait gave up (code %d)", s);
    }
    return B2R_OK;
}

b2r_status exchange_all(b2r_handle* h, bool staged)
{
    const BlockLayout& L = h->L;
    void* bounce = nullptr;
    int nf = 1;
    if (h->cfg.model == B2R_MODEL_EQWP_REF || h->cfg.model == B2R_MODEL_EQWP_STAG) nf = h->nfld;
    if (staged) {
        size_t need = halo_bounce_elems(L) * nf * h->cell_bytes;
        if (h->bounce_bytes < need) {
            if (h->bounce) cudaFree(h->bounce);
            h->bounce = nullptr;
            h->bounce_bytes = 0;
            CK(h, cudaMalloc(&h->bounce, need));
            h->bounce_bytes = need;
        }
        bounce = h->bounce;
    }
    // unstaged: one launch copying every halo cell from its owner block
    const bool gather = !staged && (long long)nf * L.nblk <= 65535;
    if (h->cell_bytes == 1) {
        FieldSet<uint8_t> fs{};
        fs.p[0] = static_cast<uint8_t*>(h->buf[h->cur]);
        if (gather) CK(h, launch_halo_gather<uint8_t>(fs, 1, L, h->stream));
        else CK(h, launch_halo_exchange<uint8_t>(fs, 1, L, static_cast<uint8_t*>(bounce), h->stream));
    } else {
        FieldSet<float> fs{};
        if (nf == 1) fs.p[0] = static_cast<float*>(h->buf[h->cur]);
        else
            for (int f = 0; f < nf; ++f) fs.p[f] = h->fld[f];
        if (gather) CK(h, launch_halo_gather<float>(fs, nf, L, h->stream));
        else CK(h, launch_halo_exchange<float>(fs, nf, L, static_cast<float*>(bounce), h->stream));
    }
    return B2R_OK;
}

b2r_status exchange_one(b2r_handle* h, int field, bool staged)
{
    const BlockLayout& L = h->L;
    void* bounce = nullptr;
    if (staged) {
        size_t need = halo_bounce_elems(L) * h->cell_bytes;
        if (h->bounce_bytes < need) {
            if (h->bounce) cudaFree(h->bounce);
            h->bounce = nullptr;
            h->bounce_bytes = 0;
            CK(h, cudaMalloc(&h->bounce, need));
            h->bounce_bytes = need;
        }
        bounce = h->bounce;
    }
    if (h->cell_bytes == 1) {
        FieldSet<uint8_t> fs{};
        fs.p[0] = static_cast<uint8_t*>(h->buf[h->cur]);
        CK(h, launch_halo_exchange<uint8_t>(fs, 1, L, static_cast<uint8_t*>(bounce), h->stream));
    } else {
        FieldSet<float> fs{};
        fs.p[0] = (h->nfld > 0) ? h->fld[field] : static_cast<float*>(h->buf[h->cur]);
        CK(h, launch_halo_exchange<float>(fs, 1, L, static_cast<float*>(bounce), h->stream));
    }
    return B2R_OK;
}

EqwpStagParams stag_params(const b2r_handle* h)
{
    EqwpStagParams p{};
    p.dt = (float)h->cfg.dt;
    p.inv_h = (float)(1.0 / h->cfg.h);
    for (int a = 0; a < 3; ++a) p.src[a] = h->cfg.src[a];
    p.src_host = h->src.empty() ? nullptr : h->src.data();
    p.src_len = (int)h->src.size();
    return p;
}

b2r_status substep(b2r_handle* h, int i)
{
    switch (h->cfg.model) {
    case B2R_MODEL_HEAT:
        CK(h, launch_heat_substep(&h->tmap[h->cur], static_cast<float*>(h->buf[1 - h->cur]), h->L,
                                  h->cfg.D, i, h->hc, h->d_status, h->stream, h->tune));
        h->cur = 1 - h->cur;
        return B2R_OK;
    case B2R_MODEL_GOL:
        if (h->gol_bytes)
            CK(h, launch_gol_substep(static_cast<const uint8_t*>(h->buf[h->cur]),
                                     static_cast<uint8_t*>(h->buf[1 - h->cur]), h->L, i, h->stream));
        else
            CK(h, launch_gol_bits_substep(static_cast<const uint8_t*>(h->buf[h->cur]),
                                          static_cast<uint8_t*>(h->buf[1 - h->cur]), h->L, i, h->stream));
        h->cur = 1 - h->cur;
        return B2R_OK;
    case B2R_MODEL_EQWP_REF: {
        EqwpRefParams p = eqwp_ref_params(h->L);
        CK(h, launch_eqwp_ref_substep(h->fld, h->L, i, (int)(h->ts - i), p, h->stream));
        return B2R_OK;
    }
    case B2R_MODEL_EQWP_STAG: {
        const EqwpStagParams p = stag_params(h);
        if (h->eqwp_fused) {
            CK(h, launch_eqwp_stag_fused(h->smaps[0], h->fld, h->fld2, h->fld2 + B2R_F_SXX, h->mat, h->L, i,
                                         (int)h->ts, p, h->d_status, h->stream));
            for (int f = 0; f < h->nfld; ++f) std::swap(h->fld[f], h->fld2[f]);
            std::swap(h->smaps[0], h->smaps[1]);
            return B2R_OK;
        }
        CK(h, launch_eqwp_stag_substep(h->fld, h->mat, h->L, i, (int)h->ts, p, h->stream));
        return B2R_OK;
    }
    default:
        return fail(h, B2R_ERR_ARG, "unknown model %d", h->cfg.model);
    }
}

void drop_graphs(b2r_handle* h)
{
    for (int c = 0; c < 2; ++c)
        if (h->gexec[c]) {
            cudaGraphExecDestroy(h->gexec[c]);
            h->gexec[c] = nullptr;
        }
    h->gsteps = 0;
}

b2r_status substep2(b2r_handle* h, int i);

// Advance n time steps from h->ts: a halo exchange at every period start
// (skipped right after an upload, whose scatter filled the halos), two steps
// per launch where heat_fuse_ok allows, one otherwise.
b2r_status advance(b2r_handle* h, int n)
{
    b2r_status st;
    for (int s = 0; s < n;) {
        const int i = (int)(h->ts % h->cfg.R);
        if (i == 0 && !h->halos_fresh)
            if ((st = exchange_all(h, false)) != B2R_OK) return st;
        h->halos_fresh = false;
        const int gg = gol_pass_gens(h, i, n - s);
        // a bit-sliced pass that ends a period stores the next period's halos
        // itself, so that period starts without the gather
        const bool push = gg >= 2 && !h->gol_bytes && h->gol_push && i + gg == h->cfg.R &&
                          (h->L.nblk > 1 || h->L.periodic) && h->L.B[0] % 32 == 0;
        if (gg >= 2) {
            if (h->gol_bytes)
                CK(h, launch_gol_period(static_cast<const uint8_t*>(h->buf[h->cur]),
                                        static_cast<uint8_t*>(h->buf[1 - h->cur]), h->L, i, gg, h->stream));
            else
                CK(h, launch_gol_bits_period(static_cast<const uint8_t*>(h->buf[h->cur]),
                                             static_cast<uint8_t*>(h->buf[1 - h->cur]), h->L, i, gg, push,
                                             h->stream));
            h->cur = 1 - h->cur;
            h->ts += gg;
            s += gg;
            h->halos_fresh = push;
        } else if (n - s >= 2 && heat_fuse_ok(h, i)) {
            if ((st = substep2(h, i)) != B2R_OK) return st;
            h->ts += 2;
            s += 2;
        } else {
            if ((st = substep(h, i)) != B2R_OK) return st;
            h->ts++;
            ++s;
        }
    }
    return B2R_OK;
}

// Capture `periods` whole periods starting from ping-pong buffer `c` at a
// period start.
b2r_status capture_graph(b2r_handle* h, int c, int periods)
{
    const int save_cur = h->cur;
    const long long save_ts = h->ts;
    const bool save_fresh = h->halos_fresh;
    h->cur = c;
    h->ts = 0;
    h->halos_fresh = false;
    const long long k0 = b2r_kernel_launches();
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    b2r_status st = advance(h, periods * h->cfg.R);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    const long long nk = b2r_kernel_launches() - k0;
    b2r::count_launches(-nk);               // captured, not launched
    h->gflip[c] = (h->cur != c);
    h->cur = save_cur;
    h->ts = save_ts;
    h->halos_fresh = save_fresh;
    if (st != B2R_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return fail(h, B2R_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&h->gexec[c], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, B2R_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    h->gkernels = nk;
    return B2R_OK;
}

b2r_status substep2(b2r_handle* h, int i)
{
    CK(h, launch_heat_substep2(&h->tmap2[h->cur], static_cast<float*>(h->buf[1 - h->cur]), h->L, i, h->hc,
                               h->d_status, h->stream, h->tune.zchunk2));
    h->cur = 1 - h->cur;
    return B2R_OK;
}

}  // namespace

namespace b2r {

static std::atomic<long long> g_launches{0};
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

bool make_block_tmap(CUtensorMap* map, const void* base, const BlockLayout& L, int elem_bytes,
                     int box_x, int box_y, int box_z)
{
    static PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
    if (!enc) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return false;
        enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    cuuint64_t dims[4] = {(cuuint64_t)L.P, (cuuint64_t)L.n[1], (cuuint64_t)L.n[2],
                          (cuuint64_t)L.nblk};
    cuuint64_t strides[3] = {(cuuint64_t)L.P * elem_bytes, (cuuint64_t)L.plane * elem_bytes,
                             (cuuint64_t)L.bstride * elem_bytes};
    cuuint32_t box[4] = {(cuuint32_t)box_x, (cuuint32_t)box_y, (cuuint32_t)box_z, 1};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = enc(map, elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT8,
                     4, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace b2r

extern "C" {

b2r_status b2r_create(const b2r_config* cfg, b2r_handle** out)
{
    if (!cfg || !out) return fail(nullptr, B2R_ERR_ARG, "null argument");
    *out = nullptr;
    const b2r_config& c = *cfg;
    if (c.model < B2R_MODEL_HEAT || c.model > B2R_MODEL_EQWP_STAG)
        return fail(nullptr, B2R_ERR_ARG, "unknown model %d", c.model);
    int B[3];
    for (int a = 0; a < 3; ++a) {
        if (c.env[a] <= 0 || c.blocks[a] <= 0)
            return fail(nullptr, B2R_ERR_ARG, "env and blocks must be positive");
        if (c.env[a] % c.blocks[a] != 0)   // b2r.cpp:154-159
            return fail(nullptr, B2R_ERR_ARG,
                        "ENV_DIM (%d) must be divisible by BLOCK_DIM (%d) on axis %d", c.env[a],
                        c.blocks[a], a);
        B[a] = c.env[a] / c.blocks[a];
    }
    if (c.model == B2R_MODEL_HEAT && (c.D < 1 || c.D > 4))
        return fail(nullptr, B2R_ERR_ARG, "heat stencil radius D must be 1..4 (got %d)", c.D);
    if (c.model == B2R_MODEL_GOL && c.D != 1)
        return fail(nullptr, B2R_ERR_ARG, "Game of Life has radius D = 1");
    if ((c.model == B2R_MODEL_EQWP_REF || c.model == B2R_MODEL_EQWP_STAG) && c.D != 2)
        return fail(nullptr, B2R_ERR_ARG, "the elastic-wave models have radius D = 2");
    if (c.R < 1) return fail(nullptr, B2R_ERR_ARG, "R must be >= 1");
    const int minB = B[0] < B[1] ? (B[0] < B[2] ? B[0] : B[2]) : (B[1] < B[2] ? B[1] : B[2]);
    if (c.R * c.D > minB / 2)   // b2r.cpp:54
        return fail(nullptr, B2R_ERR_ARG, "should meet condition: 1 <= R*D <= min(B)/2 (R*D=%d, min B=%d)",
                    c.R * c.D, minB);
    const int H = c.R * halo_per_step(c);
    if (H > minB)
        return fail(nullptr, B2R_ERR_ARG, "halo depth %d exceeds the subdomain size %d", H, minB);
    if (c.boundary != B2R_BC_SHELL && c.boundary != B2R_BC_PERIODIC)
        return fail(nullptr, B2R_ERR_ARG, "unknown boundary kind %d", c.boundary);

    b2r_handle* h = new (std::nothrow) b2r_handle();
    if (!h) return fail(nullptr, B2R_ERR_OOM, "host allocation failed");
    h->cfg = c;
    h->cell_bytes = (c.model == B2R_MODEL_GOL) ? 1 : 4;
    h->shell = (c.boundary == B2R_BC_PERIODIC) ? 0 : halo_per_step(c) / (c.model >= B2R_MODEL_EQWP_REF ? 2 : 1);
    int n[3];
    for (int a = 0; a < 3; ++a) n[a] = B[a] + 2 * H;
    fill_layout(h->L, n, B, c.blocks, H, h->cell_bytes, c.boundary == B2R_BC_PERIODIC, -1);

    b2r_status st = B2R_OK;
    auto bail = [&](b2r_status s) {
        b2r_destroy(h);
        cudaGetLastError();   // a failed allocation must not surface in the caller's next launch check
        return s;
    };
    if (cudaMalloc(&h->d_status, sizeof(int)) != cudaSuccess)
        return bail(fail(nullptr, B2R_ERR_CUDA, "cudaMalloc(status) failed"));
    cudaMemset(h->d_status, 0, sizeof(int));
    const size_t fb = field_bytes(h);
    if (c.model == B2R_MODEL_HEAT || c.model == B2R_MODEL_GOL) {
        for (int b = 0; b < 2; ++b) {
            if (cudaMalloc(&h->buf[b], fb) != cudaSuccess)
                return bail(fail(nullptr, B2R_ERR_OOM, "cudaMalloc of %zu bytes failed", fb));
            cudaMemset(h->buf[b], 0, fb);
        }
        if (c.model == B2R_MODEL_HEAT) {
            h->hc = heat_coef(c.D, c.alpha_dt, c.dx, c.dy, c.dz);
            {
                std::lock_guard<std::mutex> lock(g_tune_mu);
                auto it = g_tune_cache.find(key_of(h));
                if (it != g_tune_cache.end()) h->tune = it->second;
            }
            if ((st = build_heat_maps(h)) != B2R_OK) {
                g_err = h->err;
                return bail(st);
            }
        }
    } else {
        h->nfld = (c.model == B2R_MODEL_EQWP_REF) ? 10 : 9;
        for (int f = 0; f < h->nfld; ++f) {
            if (cudaMalloc(&h->fld[f], fb) != cudaSuccess)
                return bail(fail(nullptr, B2R_ERR_OOM, "cudaMalloc of %zu bytes failed", fb));
            cudaMemset(h->fld[f], 0, fb);
        }
        if (c.model == B2R_MODEL_EQWP_STAG) {
            for (int m = 0; m < 3; ++m) {
                if (cudaMalloc(&h->mat[m], fb) != cudaSuccess)
                    return bail(fail(nullptr, B2R_ERR_OOM, "cudaMalloc of %zu bytes failed", fb));
                cudaMemset(h->mat[m], 0, fb);
            }
            for (int f = 0; f < h->nfld; ++f) {
                if (cudaMalloc(&h->fld2[f], fb) != cudaSuccess)
                    return bail(fail(nullptr, B2R_ERR_OOM, "cudaMalloc of %zu bytes failed", fb));
                cudaMemset(h->fld2[f], 0, fb);
            }
            const int box = eqwp_fused_box();
            for (int f = 0; f < 6; ++f)
                if (!make_block_tmap(&h->smaps[0].m[f], h->fld[B2R_F_SXX + f], h->L, 4, box, box, 1) ||
                    !make_block_tmap(&h->smaps[1].m[f], h->fld2[B2R_F_SXX + f], h->L, 4, box, box, 1))
                    return bail(fail(nullptr, B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed"));
        }
    }
    if (cudaDeviceSynchronize() != cudaSuccess)
        return bail(fail(nullptr, B2R_ERR_CUDA, "device initialisation failed"));
    *out = h;
    return B2R_OK;
}

b2r_status b2r_destroy(b2r_handle* h)
{
    if (!h) return B2R_OK;
    drop_graphs(h);
    if (h->adj_ws) cudaFree(h->adj_ws);
    for (int b = 0; b < 2; ++b)
        if (h->buf[b]) cudaFree(h->buf[b]);
    for (int f = 0; f < kMaxFields; ++f) {
        if (h->fld[f]) cudaFree(h->fld[f]);
        if (h->fld2[f]) cudaFree(h->fld2[f]);
    }
    for (int m = 0; m < 3; ++m)
        if (h->mat[m]) cudaFree(h->mat[m]);
    if (h->staging) cudaFree(h->staging);
    for (void* p : h->pipe)
        if (p) cudaFree(p);
    for (auto& e2 : h->ev)
        for (cudaEvent_t e : e2)
            if (e) cudaEventDestroy(e);
    if (h->cin) cudaStreamDestroy(h->cin);
    if (h->cout) cudaStreamDestroy(h->cout);
    if (h->bounce) cudaFree(h->bounce);
    if (h->d_status) cudaFree(h->d_status);
    delete h;
    return B2R_OK;
}

int64_t b2r_kernel_launches(void) { return g_launches.load(); }

const char* b2r_last_error(const b2r_handle* h)
{
    if (h) return h->err.c_str();
    return g_err.c_str();
}

b2r_status b2r_set_stream(b2r_handle* h, void* s)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    h->stream = static_cast<cudaStream_t>(s);
    return B2R_OK;
}

b2r_status b2r_synchronize(b2r_handle* h)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    CK(h, cudaStreamSynchronize(h->stream));
    return check_status(h);
}

b2r_status b2r_geometry(const b2r_handle* h, int block_n[3], int* halo, int domain_n[3],
                        int* cell_bytes)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    for (int a = 0; a < 3; ++a) {
        if (block_n) block_n[a] = h->L.n[a];
        if (domain_n) domain_n[a] = h->cfg.env[a] + 2 * h->shell;
    }
    if (halo) *halo = h->L.H;
    if (cell_bytes) *cell_bytes = h->cell_bytes;
    return B2R_OK;
}

int64_t b2r_cells(const b2r_handle* h)
{
    if (!h) return 0;
    return (int64_t)h->cfg.env[0] * h->cfg.env[1] * h->cfg.env[2];
}

int64_t b2r_time_step(const b2r_handle* h) { return h ? h->ts : -1; }

b2r_status b2r_upload(b2r_handle* h, int field, const void* src, int src_is_device)
{
    if (!h || !src) return fail(h, B2R_ERR_ARG, "null argument");
    const bool eq = h->nfld > 0;
    const bool is_kappa = field == B2R_F_KAPPA;
    const bool is_mat = eq && field >= B2R_F_LAMBDA && field <= B2R_F_BUOY;
    if (is_kappa && h->cfg.model != B2R_MODEL_HEAT)
        return fail(h, B2R_ERR_ARG, "the conductivity field exists only for the heat model");
    if (!is_mat && !is_kappa && (field < 0 || field >= (eq ? h->nfld : 1)))
        return fail(h, B2R_ERR_ARG, "invalid field id %d", field);
    if (is_mat && h->cfg.model != B2R_MODEL_EQWP_STAG)
        return fail(h, B2R_ERR_ARG, "material fields exist only for the staggered model");
    const size_t bytes = domain_cells(h) * h->cell_bytes;
    const void* dsrc = src;
    b2r_status st;
    if (is_kappa && (st = ensure_kappa(h)) != B2R_OK) return st;
    if (!src_is_device) {
        if ((st = ensure_staging(h, bytes)) != B2R_OK) return st;
        CK(h, cudaMemcpyAsync(h->staging, src, bytes, cudaMemcpyHostToDevice, h->stream));
        dsrc = h->staging;
    }
    void* dst;
    if (is_kappa) {
        CK(h, launch_scatter<float>(static_cast<const float*>(dsrc), h->mat[0], h->L, h->shell, h->stream));
        return B2R_OK;
    }
    if (is_mat) dst = h->mat[field - B2R_F_LAMBDA];
    else if (eq) dst = h->fld[field];
    else dst = h->buf[h->cur];
    if (h->cell_bytes == 1)
        CK(h, launch_scatter<uint8_t>(static_cast<const uint8_t*>(dsrc), static_cast<uint8_t*>(dst),
                                      h->L, h->shell, h->stream));
    else
        CK(h, launch_scatter<float>(static_cast<const float*>(dsrc), static_cast<float*>(dst), h->L,
                                    h->shell, h->stream));
    if (!eq)  // both ping-pong buffers carry the shell (heat-3D.cu:591-592)
        CK(h, cudaMemcpyAsync(h->buf[1 - h->cur], h->buf[h->cur], field_bytes(h),
                              cudaMemcpyDeviceToDevice, h->stream));
    else if (!is_mat && h->fld2[field])   // so do both staggered field sets
        CK(h, cudaMemcpyAsync(h->fld2[field], h->fld[field], field_bytes(h), cudaMemcpyDeviceToDevice,
                              h->stream));
    h->ts = 0;
    h->halos_fresh = true;
    return B2R_OK;
}

b2r_status b2r_download(b2r_handle* h, int field, void* dst, int dst_is_device)
{
    if (!h || !dst) return fail(h, B2R_ERR_ARG, "null argument");
    const bool eq = h->nfld > 0;
    if (field < 0 || field >= (eq ? h->nfld : 1))
        return fail(h, B2R_ERR_ARG, "invalid field id %d", field);
    const size_t bytes = domain_cells(h) * h->cell_bytes;
    void* ddst = dst;
    b2r_status st;
    if (!dst_is_device) {
        if ((st = ensure_staging(h, bytes)) != B2R_OK) return st;
        ddst = h->staging;
    }
    const void* srcb = eq ? (const void*)h->fld[field] : h->buf[h->cur];
    if (h->cell_bytes == 1)
        CK(h, launch_gather<uint8_t>(static_cast<uint8_t*>(ddst), static_cast<const uint8_t*>(srcb),
                                     h->L, h->shell, h->stream));
    else
        CK(h, launch_gather<float>(static_cast<float*>(ddst), static_cast<const float*>(srcb), h->L,
                                   h->shell, h->stream));
    if (!dst_is_device) {
        CK(h, cudaMemcpyAsync(dst, h->staging, bytes, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    return B2R_OK;
}

b2r_status b2r_download_blocks(b2r_handle* h, int field, void* dst, int dst_is_device)
{
    if (!h || !dst) return fail(h, B2R_ERR_ARG, "null argument");
    const bool eq = h->nfld > 0;
    const bool is_mat = eq && field >= B2R_F_LAMBDA && field <= B2R_F_BUOY && h->mat[0];
    if (!is_mat && (field < 0 || field >= (eq ? h->nfld : 1)))
        return fail(h, B2R_ERR_ARG, "invalid field id %d", field);
    const char* srcb = static_cast<const char*>(
        is_mat ? (const void*)h->mat[field - B2R_F_LAMBDA]
               : (eq ? (const void*)h->fld[field] : h->buf[h->cur]));
    const BlockLayout& L = h->L;
    const size_t cb = h->cell_bytes;
    CK(h, cudaMemcpy2DAsync(dst, L.n[0] * cb, srcb + L.xoff * cb, L.P * cb, L.n[0] * cb,
                            (size_t)L.nblk * L.n[1] * L.n[2],
                            dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            h->stream));
    if (!dst_is_device) CK(h, cudaStreamSynchronize(h->stream));
    return B2R_OK;
}

b2r_status b2r_step(b2r_handle* h, int nsteps)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (nsteps < 0) return fail(h, B2R_ERR_ARG, "nsteps must be >= 0");
    b2r_status st;
    const bool use_graphs = h->graphs && h->stream != nullptr &&
                            (h->cfg.model == B2R_MODEL_HEAT || h->cfg.model == B2R_MODEL_GOL);
    int s = 0;
    while (s < nsteps) {
        const int i = (int)(h->ts % h->cfg.R);
        if (use_graphs && i == 0) {
            // whole periods replayed from a graph: >= 32 time steps per launch
            const int periods = (32 + h->cfg.R - 1) / h->cfg.R;
            const int unit = periods * h->cfg.R;
            if (nsteps - s >= unit) {
                if (h->gsteps != unit) {
                    drop_graphs(h);
                    h->gsteps = unit;
                }
                if (!h->gexec[h->cur])
                    if ((st = capture_graph(h, h->cur, periods)) != B2R_OK) return st;
                CK(h, cudaGraphLaunch(h->gexec[h->cur], h->stream));
                b2r::count_launches(h->gkernels);
                if (h->gflip[h->cur]) h->cur = 1 - h->cur;
                h->ts += unit;
                h->halos_fresh = false;
                s += unit;
                continue;
            }
        }
        // up to the next period start (or all of it when nothing is graphed)
        int chunk = nsteps - s;
        if (use_graphs && i != 0) chunk = std::min(chunk, h->cfg.R - i);
        if (use_graphs && i == 0) {
            const int periods = (32 + h->cfg.R - 1) / h->cfg.R;
            chunk = std::min(chunk, periods * h->cfg.R);
        }
        if ((st = advance(h, chunk)) != B2R_OK) return st;
        s += chunk;
    }
    return B2R_OK;
}

b2r_status b2r_set_graphs(b2r_handle* h, int enable)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    h->graphs = enable != 0;
    if (!h->graphs) drop_graphs(h);
    return B2R_OK;
}

b2r_status b2r_run_host(b2r_handle* h, int field, const void* host_in, int nsteps, void* host_out)
{
    b2r_status st;
    if ((st = b2r_upload(h, field, host_in, 0)) != B2R_OK) return st;
    if ((st = b2r_step(h, nsteps)) != B2R_OK) return st;
    if ((st = b2r_download(h, field, host_out, 0)) != B2R_OK) return st;
    return check_status(h);
}

// Pipelined b2r_run_host over `count` independent inputs: while problem i
// steps on the handle's stream, the input of problem i+1 is copied in on one
// copy stream and the result of problem i-1 copied out on the other.
b2r_status b2r_run_host_batch(b2r_handle* h, int field, const void* const* host_in, void* const* host_out,
                              int count, int nsteps)
{
    if (!h || !host_in || !host_out || count < 0) return fail(h, B2R_ERR_ARG, "invalid argument");
    if (h->nfld > 0) return fail(h, B2R_ERR_ARG, "pipelined host runs cover the heat and Game-of-Life models");
    if (field != 0) return fail(h, B2R_ERR_ARG, "invalid field id %d", field);
    for (int i = 0; i < count; ++i)
        if (!host_in[i] || !host_out[i]) return fail(h, B2R_ERR_ARG, "null buffer for problem %d", i);
    const size_t bytes = domain_cells(h) * h->cell_bytes;
    if (h->pipe_bytes < bytes) {
        for (void*& p : h->pipe) {
            if (p) cudaFree(p);
            p = nullptr;
        }
        h->pipe_bytes = 0;
        for (void*& p : h->pipe) CK(h, cudaMalloc(&p, bytes));
        h->pipe_bytes = bytes;
    }
    if (!h->cin) {
        CK(h, cudaStreamCreateWithFlags(&h->cin, cudaStreamNonBlocking));
        CK(h, cudaStreamCreateWithFlags(&h->cout, cudaStreamNonBlocking));
        for (auto& e2 : h->ev)
            for (cudaEvent_t& e : e2) CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    enum { IN_READY, IN_FREE, OUT_READY, OUT_FREE };
    void* const* in = h->pipe;
    void* const* out = h->pipe + 2;
    // nothing is pending from an earlier call: every wait below refers to an
    // event recorded in this call or never recorded (a no-op)
    CK(h, cudaStreamSynchronize(h->cin));
    CK(h, cudaStreamSynchronize(h->cout));
    for (auto& e2 : h->ev)
        for (cudaEvent_t& e : e2) {
            cudaEventDestroy(e);
            CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
    if (count > 0) {
        CK(h, cudaMemcpyAsync(in[0], host_in[0], bytes, cudaMemcpyHostToDevice, h->cin));
        CK(h, cudaEventRecord(h->ev[IN_READY][0], h->cin));
    }
    b2r_status st;
    for (int i = 0; i < count; ++i) {
        const int k = i & 1, k1 = (i + 1) & 1;
        if (i + 1 < count) {   // next input, once problem i-1 has consumed that slot
            CK(h, cudaStreamWaitEvent(h->cin, h->ev[IN_FREE][k1], 0));
            CK(h, cudaMemcpyAsync(in[k1], host_in[i + 1], bytes, cudaMemcpyHostToDevice, h->cin));
            CK(h, cudaEventRecord(h->ev[IN_READY][k1], h->cin));
        }
        CK(h, cudaStreamWaitEvent(h->stream, h->ev[IN_READY][k], 0));
        if ((st = b2r_upload(h, field, in[k], 1)) != B2R_OK) return st;
        CK(h, cudaEventRecord(h->ev[IN_FREE][k], h->stream));
        if ((st = b2r_step(h, nsteps)) != B2R_OK) return st;
        CK(h, cudaStreamWaitEvent(h->stream, h->ev[OUT_FREE][k], 0));   // result of problem i-2 copied out
        if ((st = b2r_download(h, field, out[k], 1)) != B2R_OK) return st;
        CK(h, cudaEventRecord(h->ev[OUT_READY][k], h->stream));
        CK(h, cudaStreamWaitEvent(h->cout, h->ev[OUT_READY][k], 0));
        CK(h, cudaMemcpyAsync(host_out[i], out[k], bytes, cudaMemcpyDeviceToHost, h->cout));
        CK(h, cudaEventRecord(h->ev[OUT_FREE][k], h->cout));
    }
    CK(h, cudaStreamSynchronize(h->cout));
    CK(h, cudaStreamSynchronize(h->stream));
    return check_status(h);
}

b2r_status b2r_set_source(b2r_handle* h, const float* amps, int n)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (n < 0 || (n > 0 && !amps)) return fail(h, B2R_ERR_ARG, "invalid source series");
    h->src.assign(amps, amps + n);
    return B2R_OK;
}

// A caller that exchanges every field at a period start (b2r.cpp:197-206)
// leaves the halos fresh: the next b2r_step starts without its own exchange.
static b2r_status note_exchange(b2r_handle* h, int field, b2r_status st)
{
    if (st != B2R_OK || h->ts % h->cfg.R != 0) return st;
    if (h->xts != h->ts) {
        h->xmask = 0;
        h->xts = h->ts;
    }
    h->xmask |= 1u << field;
    const int nf = (h->cfg.model == B2R_MODEL_EQWP_REF || h->cfg.model == B2R_MODEL_EQWP_STAG) ? h->nfld : 1;
    if (h->xmask == (nf >= 32 ? ~0u : (1u << nf) - 1u)) h->halos_fresh = true;
    return st;
}

b2r_status b2r_boundary_updating_direct(b2r_handle* h, int time_step, int field)
{
    (void)time_step;
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (field < 0 || field >= (h->nfld > 0 ? h->nfld : 1))
        return fail(h, B2R_ERR_ARG, "invalid field id %d", field);
    return note_exchange(h, field, exchange_one(h, field, false));
}

b2r_status b2r_boundary_updating(b2r_handle* h, int time_step, int field)
{
    (void)time_step;
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (field < 0 || field >= (h->nfld > 0 ? h->nfld : 1))
        return fail(h, B2R_ERR_ARG, "invalid field id %d", field);
    return note_exchange(h, field, exchange_one(h, field, true));
}

// ---------------------------------------------------------------- autotuning

b2r_status b2r_set_tuning(b2r_handle* h, int key, int value)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    switch (key) {
    case B2R_TUNE_ZCHUNK: h->tune.zchunk = value; break;
    case B2R_TUNE_CTAS_PER_SM: h->tune.ctas_per_sm = value; break;
    case B2R_TUNE_PDL: h->tune.pdl = value != 0; break;
    case B2R_TUNE_TBLOCK: h->tune.tblock = value; break;
    case B2R_TUNE_ZCHUNK2: h->tune.zchunk2 = value; break;
    case B2R_TUNE_EQWP_FUSED: h->eqwp_fused = value != 0; break;
    case B2R_TUNE_GOL_BYTES: h->gol_bytes = value != 0; break;
    case B2R_TUNE_ADJ_FUSED: h->adj_fused = value != 0; break;
    case B2R_TUNE_GOL_PUSH: h->gol_push = value != 0; break;
    default: return fail(h, B2R_ERR_ARG, "unknown tuning key %d", key);
    }
    drop_graphs(h);
    return B2R_OK;
}

b2r_status b2r_get_tuning(const b2r_handle* h, int key, int* value)
{
    if (!h || !value) return fail(nullptr, B2R_ERR_ARG, "null argument");
    switch (key) {
    case B2R_TUNE_ZCHUNK: *value = h->tune.zchunk; break;
    case B2R_TUNE_CTAS_PER_SM: *value = h->tune.ctas_per_sm; break;
    case B2R_TUNE_PDL: *value = h->tune.pdl ? 1 : 0; break;
    case B2R_TUNE_TBLOCK: *value = h->tune.tblock; break;
    case B2R_TUNE_ZCHUNK2: *value = h->tune.zchunk2; break;
    case B2R_TUNE_EQWP_FUSED: *value = h->eqwp_fused ? 1 : 0; break;
    case B2R_TUNE_GOL_BYTES: *value = h->gol_bytes ? 1 : 0; break;
    case B2R_TUNE_ADJ_FUSED: *value = h->adj_fused ? 1 : 0; break;
    case B2R_TUNE_GOL_PUSH: *value = h->gol_push ? 1 : 0; break;
    default: return fail(nullptr, B2R_ERR_ARG, "unknown tuning key %d", key);
    }
    return B2R_OK;
}

// Game of Life and the staggered elastic wave: the same timed search over
// their kernel choices -- generations per pass, bit-sliced or byte cells and
// the period-end halo fill (GoL); the one-pass or two-pass step (elastic
// wave).  Trials run on the live fields, which are restored afterwards.
struct KnobSet {
    int tblock, gol_bytes, gol_push, eqwp_fused;
};
static std::map<TuneKey, KnobSet> g_knob_cache;

static void apply_knobs(b2r_handle* h, const KnobSet& k)
{
    h->tune.tblock = k.tblock;
    h->gol_bytes = k.gol_bytes != 0;
    h->gol_push = k.gol_push != 0;
    h->eqwp_fused = k.eqwp_fused != 0;
}

static b2r_status autotune_knobs(b2r_handle* h, int trial_steps, int best[3], double* best_ms)
{
    auto report = [&](const KnobSet& k, double ms) {
        if (best) {
            best[0] = k.tblock;
            best[1] = h->cfg.model == B2R_MODEL_GOL ? k.gol_bytes : k.eqwp_fused;
            best[2] = k.gol_push;
        }
        if (best_ms) *best_ms = ms;
    };
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_knob_cache.find(key_of(h));
        if (it != g_knob_cache.end()) {
            apply_knobs(h, it->second);
            report(it->second, -1.0);
            drop_graphs(h);
            return B2R_OK;
        }
    }
    std::vector<KnobSet> cands;
    const KnobSet cur{h->tune.tblock, h->gol_bytes, h->gol_push, h->eqwp_fused};
    if (h->cfg.model == B2R_MODEL_GOL) {
        for (int tb : {1, 2, 4})
            for (int bytes = 0; bytes < 2; ++bytes)
                for (int push = 0; push < 2; ++push)
                    if (!push || (tb >= 2 && !bytes)) cands.push_back({tb, bytes, push, cur.eqwp_fused});
    } else {
        for (int fused = 0; fused < 2; ++fused) cands.push_back({cur.tblock, cur.gol_bytes, cur.gol_push, fused});
    }
    // the state the trials overwrite: the current buffer (GoL) or every
    // field of the current set with the set's pointers (elastic wave)
    const size_t fb = field_bytes(h);
    const bool eq = h->nfld > 0;
    const int nsave = eq ? h->nfld : 1;
    struct SaveBufs {
        std::vector<void*> p;
        ~SaveBufs()
        {
            for (void* q : p)
                if (q) cudaFree(q);
        }
    } keep;
    keep.p.assign((size_t)nsave, nullptr);
    std::vector<void*>& save = keep.p;
    float* save_fld[kMaxFields];
    float* save_fld2[kMaxFields];
    StressMaps save_smaps[2] = {h->smaps[0], h->smaps[1]};
    std::memcpy(save_fld, h->fld, sizeof save_fld);
    std::memcpy(save_fld2, h->fld2, sizeof save_fld2);
    for (int f = 0; f < nsave; ++f) {
        if (cudaMalloc(&save[(size_t)f], fb) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, B2R_ERR_OOM, "autotuning needs %zu bytes to keep the fields", fb * nsave);
        }
        const void* src = eq ? (const void*)h->fld[f] : h->buf[h->cur];
        CK(h, cudaMemcpyAsync(save[(size_t)f], src, fb, cudaMemcpyDeviceToDevice, h->stream));
    }
    const int save_cur = h->cur;
    const long long save_ts = h->ts;
    const bool save_fresh = h->halos_fresh;
    // trials run as the stepping will (graph replay included, each
    // candidate's graphs captured in its warm run) and over whole periods:
    // a single period would not show what a choice costs at period ends
    const int trial = h->cfg.model == B2R_MODEL_GOL ? std::max(trial_steps, 16 * h->cfg.R) : trial_steps;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    KnobSet bestK = cur;
    float bestMs = 1e30f;
    b2r_status st = B2R_OK;
    for (const KnobSet& k : cands) {
        apply_knobs(h, k);
        drop_graphs(h);
        if ((st = b2r_step(h, trial)) != B2R_OK) break;   // warm (captures graphs)
        cudaEventRecord(e0, h->stream);
        if ((st = b2r_step(h, trial)) != B2R_OK) break;
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < bestMs) {
            bestMs = ms;
            bestK = k;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::memcpy(h->fld, save_fld, sizeof save_fld);
    std::memcpy(h->fld2, save_fld2, sizeof save_fld2);
    h->smaps[0] = save_smaps[0];
    h->smaps[1] = save_smaps[1];
    h->cur = save_cur;
    h->ts = save_ts;
    h->halos_fresh = save_fresh;
    for (int f = 0; f < nsave; ++f) {
        void* dst = eq ? (void*)h->fld[f] : h->buf[h->cur];
        cudaMemcpyAsync(dst, save[(size_t)f], fb, cudaMemcpyDeviceToDevice, h->stream);
    }
    cudaStreamSynchronize(h->stream);
    apply_knobs(h, st == B2R_OK ? bestK : cur);
    drop_graphs(h);
    if (st != B2R_OK) return st;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_knob_cache[key_of(h)] = bestK;
    }
    report(bestK, bestMs / trial);
    return check_status(h);
}

b2r_status b2r_autotune(b2r_handle* h, int trial_steps, int best[3], double* best_ms)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (trial_steps < 1) trial_steps = 4;
    if (h->cfg.model == B2R_MODEL_GOL || h->cfg.model == B2R_MODEL_EQWP_STAG)
        return autotune_knobs(h, trial_steps, best, best_ms);
    if (h->cfg.model != B2R_MODEL_HEAT)
        return fail(h, B2R_ERR_ARG, "autotuning covers heat, Game of Life and the staggered elastic wave");
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key_of(h));
        if (it != g_tune_cache.end()) {
            h->tune = it->second;
            if (best) { best[0] = h->tune.zchunk; best[1] = h->tune.ctas_per_sm; best[2] = h->tune.pdl; }
            if (best_ms) *best_ms = -1.0;
            drop_graphs(h);
            return B2R_OK;
        }
    }
    // keep the simulation state: trials run on the live buffers, which are
    // restored afterwards
    const size_t fb = field_bytes(h);
    DevBuf keep;
    CK(h, cudaMalloc(&keep.p, fb));
    void* const save = keep.p;
    CK(h, cudaMemcpyAsync(save, h->buf[h->cur], fb, cudaMemcpyDeviceToDevice, h->stream));
    const int save_cur = h->cur;
    const long long save_ts = h->ts;
    const bool save_fresh = h->halos_fresh;
    const bool save_graphs = h->graphs;
    h->graphs = false;
    static const int zchunks[] = {0, 16, 32, 64, 128, 256};
    static const int persist[] = {0, 1, 2, 3, 4, 5, 6};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    HeatTune bestT = h->tune;
    float bestMs = 1e30f;
    b2r_status st = B2R_OK;
    // candidates: the two-step sweep (radius 1) by z-chunk, then the one-step
    // sweep by z-chunk x persistent CTAs per SM x PDL
    struct Cand { int tb, zc2, zc, cp, pdl; };
    std::vector<Cand> cands;
    if (h->cfg.D == 1)
        for (int z2 : {4, 8, 16, 32, 64}) cands.push_back({2, z2, 0, 0, 1});
    for (int pdl = 0; pdl < 2; ++pdl)
        for (int zc : zchunks)
            for (int cp : persist)
                if (zc <= h->L.n[2]) cands.push_back({1, 0, zc, cp, pdl});
    for (const Cand& cd : cands)
            {
                if (st != B2R_OK) break;
                h->tune.tblock = cd.tb;
                h->tune.zchunk2 = cd.zc2;
                h->tune.zchunk = cd.zc;
                h->tune.ctas_per_sm = cd.cp;
                h->tune.pdl = cd.pdl;
                if ((st = b2r_step(h, 1)) != B2R_OK) break;       // warm
                cudaEventRecord(e0, h->stream);
                if ((st = b2r_step(h, trial_steps)) != B2R_OK) break;
                cudaEventRecord(e1, h->stream);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < bestMs) {
                    bestMs = ms;
                    bestT = h->tune;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->tune = bestT;
    h->cur = save_cur;
    h->ts = save_ts;
    h->halos_fresh = save_fresh;
    h->graphs = save_graphs;
    cudaMemcpyAsync(h->buf[h->cur], save, fb, cudaMemcpyDeviceToDevice, h->stream);
    cudaStreamSynchronize(h->stream);
    if (st != B2R_OK) return st;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key_of(h)] = bestT;
    }
    drop_graphs(h);
    if (best) { best[0] = bestT.tblock == 2 ? bestT.zchunk2 : bestT.zchunk; best[1] = bestT.ctas_per_sm; best[2] = bestT.pdl; }
    if (best_ms) *best_ms = bestMs / trial_steps;
    return check_status(h);
}

// ---------------------------------------------------------------- adjoint (staggered model)
namespace {


b2r_status adj_check(b2r_handle* h)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (h->cfg.model != B2R_MODEL_EQWP_STAG)
        return fail(h, B2R_ERR_ARG, "the adjoint covers the staggered elastic-wave model");
    if (h->L.nblk != 1 || h->cfg.R != 1)
        return fail(h, B2R_ERR_ARG, "the adjoint runs on one block with R = 1");
    return B2R_OK;
}

// receiver element offsets (global interior coordinates -> block storage)
b2r_status rec_offsets(b2r_handle* h, int nrec, const int* rec_xyz, std::vector<long long>& idx)
{
    idx.resize(nrec);
    for (int r = 0; r < nrec; ++r) {
        int c[3];
        for (int a = 0; a < 3; ++a) {
            c[a] = rec_xyz[3 * r + a];
            if (c[a] < 0 || c[a] >= h->cfg.env[a]) return fail(h, B2R_ERR_ARG, "receiver %d outside the domain", r);
            c[a] += h->L.H;
        }
        idx[r] = (long long)c[2] * h->L.plane + (long long)c[1] * h->L.P + h->L.xoff + c[0];
    }
    return B2R_OK;
}

}  // namespace

b2r_status b2r_eqwp_record(b2r_handle* h, int nsteps, int nrec, const int* rec_xyz, float* d_out)
{
    b2r_status st;
    if ((st = adj_check(h)) != B2R_OK) return st;
    if (nsteps < 0 || nrec <= 0 || !rec_xyz || !d_out) return fail(h, B2R_ERR_ARG, "invalid receivers");
    std::vector<long long> idx;
    if ((st = rec_offsets(h, nrec, rec_xyz, idx)) != B2R_OK) return st;
    DevBuf d_idx, d_rec;
    CK(h, cudaMalloc(&d_idx.p, sizeof(long long) * nrec));
    CK(h, cudaMalloc(&d_rec.p, sizeof(float) * (size_t)nrec * (nsteps > 0 ? nsteps : 1)));
    CK(h, cudaMemcpyAsync(d_idx.p, idx.data(), sizeof(long long) * nrec, cudaMemcpyHostToDevice, h->stream));
    h->ts = 0;
    for (int n = 0; n < nsteps; ++n) {
        if ((st = substep(h, 0)) != B2R_OK) return st;
        h->ts++;
        CK(h, adjoint_sample(h->fld[B2R_F_VY], (const long long*)d_idx.p, nrec, (float*)d_rec.p + (size_t)n * nrec,
                             h->stream));
    }
    CK(h, cudaMemcpyAsync(d_out, d_rec.p, sizeof(float) * (size_t)nrec * nsteps, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return check_status(h);
}

b2r_status b2r_eqwp_misfit_gradient(b2r_handle* h, int nsteps, int nrec, const int* rec_xyz,
                                    const float* d_obs, int ckpt_every, double* misfit,
                                    double* grad_lambda, double* grad_mu, double* grad_rho,
                                    float* d_syn)
{
    b2r_status st;
    if ((st = adj_check(h)) != B2R_OK) return st;
    if (nsteps <= 0 || nrec <= 0 || !rec_xyz || !d_obs) return fail(h, B2R_ERR_ARG, "invalid receivers / steps");
    const int K = ckpt_every > 0 ? ckpt_every : nsteps;
    std::vector<long long> idx;
    if ((st = rec_offsets(h, nrec, rec_xyz, idx)) != B2R_OK) return st;
    const size_t fb = field_bytes(h);
    const size_t nseg = (size_t)(nsteps + K - 1) / K;
    // workspace, carved from one allocation kept on the handle: checkpoints
    // (9 fields each), the replayed velocities v^{n0+k} (k = 1..K; k = 0 is
    // the checkpoint) and stencil sums of a segment, the replay's stresses,
    // the adjoint fields and the FP64 gradients
    // Two replay buffers when the workspace fits: segment s-1 is replayed
    // on a second stream while segment s runs its reverse steps.
    const size_t gbytes = (size_t)h->L.bstride * sizeof(double);
    const size_t nf_ckpt = nseg * 9, nf_v = (size_t)(K + 1) * 3, nf_a = (size_t)K * 3;
    const size_t fba = (fb + 255) & ~(size_t)255, gba = (gbytes + 255) & ~(size_t)255;
    int nbuf = nseg > 1 ? 2 : 1;
    for (;; --nbuf) {
        const size_t nfields = nf_ckpt + nbuf * (nf_v + nf_a + 6) + 18;
        const size_t need = nfields * fba + 3 * gba;
        if (h->adj_ws_bytes >= need) break;
        if (h->adj_ws) cudaFree(h->adj_ws);
        h->adj_ws = nullptr;
        h->adj_ws_bytes = 0;
        if (cudaMalloc(&h->adj_ws, need) == cudaSuccess) {
            h->adj_ws_bytes = need;
            break;
        }
        cudaGetLastError();
        h->adj_ws = nullptr;
        if (nbuf == 1) return fail(h, B2R_ERR_OOM, "misfit gradient needs %zu bytes of workspace", need);
    }
    char* ws = static_cast<char*>(h->adj_ws);
    auto carve = [&](size_t n, std::vector<float*>& out) {
        out.resize(n);
        for (size_t i = 0; i < n; ++i, ws += fba) out[i] = reinterpret_cast<float*>(ws);
    };
    std::vector<float*> ckpt, vrep, arep, srep, tmp;
    carve(nf_ckpt, ckpt);
    carve(nf_v * nbuf, vrep);   // buffer b: entries [b * nf_v, (b + 1) * nf_v)
    carve(nf_a * nbuf, arep);
    carve(6 * (size_t)nbuf, srep);
    carve(18, tmp);
    double* gp[3];
    for (int m = 0; m < 3; ++m, ws += gba) {
        gp[m] = reinterpret_cast<double*>(ws);
        CK(h, cudaMemsetAsync(gp[m], 0, gbytes, h->stream));
    }
    DevBuf d_idx, d_rec, d_res;
    // cells outside the update window never change: every replay slot starts
    // as a copy of the initial state there
    for (size_t k = 0; k < vrep.size(); ++k)
        CK(h, cudaMemcpyAsync(vrep[k], h->fld[B2R_F_VX + k % 3], fb, cudaMemcpyDeviceToDevice, h->stream));
    for (float* b : arep) CK(h, cudaMemsetAsync(b, 0, fb, h->stream));
    for (float* b : tmp) CK(h, cudaMemsetAsync(b, 0, fb, h->stream));
    CK(h, cudaMalloc(&d_idx.p, sizeof(long long) * nrec));
    CK(h, cudaMalloc(&d_rec.p, sizeof(float) * (size_t)nrec * nsteps));
    CK(h, cudaMalloc(&d_res.p, sizeof(float) * (size_t)nrec * nsteps));
    CK(h, cudaMemcpyAsync(d_idx.p, idx.data(), sizeof(long long) * nrec, cudaMemcpyHostToDevice, h->stream));
    const long long* didx = (const long long*)d_idx.p;

    // forward with checkpoints every K steps and receiver samples
    h->ts = 0;
    for (int n = 0; n < nsteps; ++n) {
        if (n % K == 0)
            for (int f = 0; f < 9; ++f)
                CK(h, cudaMemcpyAsync(ckpt[(n / K) * 9 + f], h->fld[f], fb, cudaMemcpyDeviceToDevice, h->stream));
        if ((st = substep(h, 0)) != B2R_OK) return st;
        h->ts++;
        CK(h, adjoint_sample(h->fld[B2R_F_VY], didx, nrec, (float*)d_rec.p + (size_t)n * nrec, h->stream));
    }
    // misfit and residual (host, FP64)
    std::vector<float> syn((size_t)nrec * nsteps), res((size_t)nrec * nsteps);
    CK(h, cudaMemcpyAsync(syn.data(), d_rec.p, sizeof(float) * syn.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    double J = 0.0;
    for (size_t i = 0; i < syn.size(); ++i) {
        const double r = (double)syn[i] - (double)d_obs[i];
        res[i] = (float)r;
        J += 0.5 * r * r;
    }
    if (misfit) *misfit = J;
    if (d_syn) std::copy(syn.begin(), syn.end(), d_syn);
    CK(h, cudaMemcpyAsync(d_res.p, res.data(), sizeof(float) * res.size(), cudaMemcpyHostToDevice, h->stream));

    // reverse sweep, segment by segment: each segment is replayed forward
    // from its checkpoint into replay buffer sgi % nbuf (velocities and
    // stencil sums of every step kept), then its reverse steps run.  With two
    // buffers the replay of the segment below runs on a second stream while
    // this segment's reverse steps run; the results are the same bits.
    float* const* tp = tmp.data();
    const float* mat[3] = {h->mat[0], h->mat[1], h->mat[2]};
    const float dt_h = (float)(h->cfg.dt / h->cfg.h);
    const EqwpStagParams sp = stag_params(h);
    struct AuxStream {
        cudaStream_t s = nullptr;
        cudaEvent_t start = nullptr, rep[2] = {}, rev[2] = {};
        ~AuxStream()
        {
            for (cudaEvent_t e : {start, rep[0], rep[1], rev[0], rev[1]})
                if (e) cudaEventDestroy(e);
            if (s) cudaStreamDestroy(s);
        }
    } ax;
    cudaStream_t aux = h->stream;
    if (nbuf == 2) {
        CK(h, cudaStreamCreateWithFlags(&ax.s, cudaStreamNonBlocking));
        for (cudaEvent_t* e : {&ax.start, &ax.rep[0], &ax.rep[1], &ax.rev[0], &ax.rev[1]})
            CK(h, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        aux = ax.s;
        CK(h, cudaEventRecord(ax.start, h->stream));   // the forward and the residual are in place
        CK(h, cudaStreamWaitEvent(aux, ax.start, 0));
    }
    // v^{n0+k} of segment sgi: the checkpoint's velocities for k = 0, replay
    // slot k of the segment's buffer after
    auto vslot = [&](long long sgi, int k, int f) -> float* {
        return k == 0 ? ckpt[sgi * 9 + B2R_F_VX + f] : vrep[(size_t)(sgi % nbuf) * nf_v + (size_t)k * 3 + f];
    };
    auto aslot = [&](long long sgi, int k) -> float* const* {
        return &arep[(size_t)(sgi % nbuf) * nf_a + (size_t)k * 3];
    };
    auto replay = [&](long long sgi, cudaStream_t st) -> b2r_status {
        const int n0 = (int)sgi * K, n1 = std::min(nsteps, n0 + K);
        float* const* s6 = srep.data() + 6 * (sgi % nbuf);
        for (int f = 0; f < 6; ++f)
            CK(h, cudaMemcpyAsync(s6[f], ckpt[sgi * 9 + B2R_F_SXX + f], fb, cudaMemcpyDeviceToDevice, st));
        for (int n = n0; n < n1; ++n) {
            const int k = n - n0;
            const float* vin[3] = {vslot(sgi, k, 0), vslot(sgi, k, 1), vslot(sgi, k, 2)};
            float* vout[3] = {vslot(sgi, k + 1, 0), vslot(sgi, k + 1, 1), vslot(sgi, k + 1, 2)};
            CK(h, launch_eqwp_stag_step_replay(vin, s6, vout, aslot(sgi, k), h->mat, h->L, n, sp, st));
        }
        return B2R_OK;
    };
    if ((st = replay((long long)nseg - 1, aux)) != B2R_OK) return st;
    if (nbuf == 2) CK(h, cudaEventRecord(ax.rep[(nseg - 1) % 2], aux));
    for (long long sgi = (long long)nseg - 1; sgi >= 0; --sgi) {
        const int n0 = (int)sgi * K;
        const int n1 = std::min(nsteps, n0 + K);
        if (nbuf == 2) {
            CK(h, cudaStreamWaitEvent(h->stream, ax.rep[sgi % 2], 0));
            if (sgi >= 1) {
                const int b1 = (int)((sgi - 1) % 2);
                // that buffer last served segment sgi + 1, whose reverse steps are queued
                if (sgi + 1 < (long long)nseg) CK(h, cudaStreamWaitEvent(aux, ax.rev[b1], 0));
                if ((st = replay(sgi - 1, aux)) != B2R_OK) return st;
                CK(h, cudaEventRecord(ax.rep[b1], aux));
            }
        }
        for (int n = n1 - 1; n >= n0; --n) {
            const int k = n - n0;
            CK(h, adjoint_inject(tp[1], didx, nrec, (const float*)d_res.p + (size_t)n * nrec, h->stream));
            const float* vn[3] = {vslot(sgi, k, 0), vslot(sgi, k, 1), vslot(sgi, k, 2)};
            float* const* a = aslot(sgi, k);
            const float* an[3] = {a[0], a[1], a[2]};
            CK(h, adjoint_step(tp, vn, an, mat, gp, h->L, dt_h, n == 0, h->adj_fused, h->stream));
        }
        if (nbuf == 2) CK(h, cudaEventRecord(ax.rev[sgi % 2], h->stream));
        else if (sgi >= 1 && (st = replay(sgi - 1, h->stream)) != B2R_OK) return st;
    }
    // gradients out (interior cells, x fastest), g_rho = -g_b / rho^2
    double* outs[3] = {grad_lambda, grad_mu, grad_rho};
    const size_t ncell = (size_t)h->cfg.env[0] * h->cfg.env[1] * h->cfg.env[2];
    DevBuf d_out;
    CK(h, cudaMalloc(&d_out.p, ncell * sizeof(double)));
    for (int m = 0; m < 3; ++m) {
        if (!outs[m]) continue;
        CK(h, adjoint_grad_out(gp[m], h->mat[2], m == 2, h->L, (double*)d_out.p, h->stream));
        CK(h, cudaMemcpyAsync(outs[m], d_out.p, ncell * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    h->ts = nsteps;
    h->halos_fresh = false;
    return check_status(h);
}

namespace {

b2r_status heat_adj_check(b2r_handle* h)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (h->cfg.model != B2R_MODEL_HEAT) return fail(h, B2R_ERR_ARG, "the heat adjoint needs the heat model");
    if (h->L.nblk != 1 || h->L.periodic)
        return fail(h, B2R_ERR_ARG, "the heat adjoint runs on one block with a fixed shell");
    return ensure_kappa(h);
}

HeatLap heat_lap_of(const b2r_handle* h)
{
    return heat_lap(h->cfg.D, h->cfg.alpha_dt, h->cfg.dx, h->cfg.dy, h->cfg.dz);
}

}  // namespace

b2r_status b2r_heat_record(b2r_handle* h, int nsteps, int nrec, const int* rec_xyz, float* d_out)
{
    b2r_status st;
    if ((st = heat_adj_check(h)) != B2R_OK) return st;
    if (nsteps < 0 || nrec <= 0 || !rec_xyz || !d_out) return fail(h, B2R_ERR_ARG, "invalid receivers");
    std::vector<long long> idx;
    if ((st = rec_offsets(h, nrec, rec_xyz, idx)) != B2R_OK) return st;
    DevBuf d_idx, d_rec;
    CK(h, cudaMalloc(&d_idx.p, sizeof(long long) * nrec));
    CK(h, cudaMalloc(&d_rec.p, sizeof(float) * (size_t)nrec * (nsteps > 0 ? nsteps : 1)));
    CK(h, cudaMemcpyAsync(d_idx.p, idx.data(), sizeof(long long) * nrec, cudaMemcpyHostToDevice, h->stream));
    const HeatLap c = heat_lap_of(h);
    for (int n = 0; n < nsteps; ++n) {
        float* in = static_cast<float*>(h->buf[h->cur]);
        float* out = static_cast<float*>(h->buf[1 - h->cur]);
        CK(h, launch_heat_kappa_step(in, out, h->mat[0], h->L, h->cfg.D, c, h->stream));
        h->cur = 1 - h->cur;
        CK(h, adjoint_sample(out, (const long long*)d_idx.p, nrec, (float*)d_rec.p + (size_t)n * nrec, h->stream));
    }
    h->ts += nsteps;
    CK(h, cudaMemcpyAsync(d_out, d_rec.p, sizeof(float) * (size_t)nrec * nsteps, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return check_status(h);
}

b2r_status b2r_heat_misfit_gradient(b2r_handle* h, int nsteps, int nrec, const int* rec_xyz,
                                    const float* d_obs, int ckpt_every, double* misfit,
                                    double* grad_kappa, float* d_syn)
{
    b2r_status st;
    if ((st = heat_adj_check(h)) != B2R_OK) return st;
    if (nsteps <= 0 || nrec <= 0 || !rec_xyz || !d_obs) return fail(h, B2R_ERR_ARG, "invalid receivers / steps");
    const int K = ckpt_every > 0 ? ckpt_every : nsteps;
    std::vector<long long> idx;
    if ((st = rec_offsets(h, nrec, rec_xyz, idx)) != B2R_OK) return st;
    const size_t fb = field_bytes(h);
    const size_t nseg = (size_t)(nsteps + K - 1) / K;
    // workspace on the handle: checkpoints, replay slots 1..K, lam, y, FP64 gradient
    const size_t fba = (fb + 255) & ~(size_t)255;
    const size_t gba = ((size_t)h->L.bstride * sizeof(double) + 255) & ~(size_t)255;
    const size_t need = (nseg + (size_t)K + 1 + 2) * fba + gba;
    if (h->adj_ws_bytes < need) {
        if (h->adj_ws) cudaFree(h->adj_ws);
        h->adj_ws = nullptr;
        h->adj_ws_bytes = 0;
        if (cudaMalloc(&h->adj_ws, need) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, B2R_ERR_OOM, "heat gradient needs %zu bytes of workspace", need);
        }
        h->adj_ws_bytes = need;
    }
    char* ws = static_cast<char*>(h->adj_ws);
    std::vector<float*> ckpt(nseg), slot((size_t)K + 1);
    for (auto& p : ckpt) p = reinterpret_cast<float*>(ws), ws += fba;
    for (auto& p : slot) p = reinterpret_cast<float*>(ws), ws += fba;
    float* lam = reinterpret_cast<float*>(ws);
    ws += fba;
    float* yb = reinterpret_cast<float*>(ws);
    ws += fba;
    double* g = reinterpret_cast<double*>(ws);
    CK(h, cudaMemsetAsync(lam, 0, fb, h->stream));
    CK(h, cudaMemsetAsync(yb, 0, fb, h->stream));
    CK(h, cudaMemsetAsync(g, 0, (size_t)h->L.bstride * sizeof(double), h->stream));
    // shell cells never change: every replay slot starts as the initial state
    for (size_t k = 1; k < slot.size(); ++k)
        CK(h, cudaMemcpyAsync(slot[k], h->buf[h->cur], fb, cudaMemcpyDeviceToDevice, h->stream));
    DevBuf d_idx, d_rec, d_res;
    CK(h, cudaMalloc(&d_idx.p, sizeof(long long) * nrec));
    CK(h, cudaMalloc(&d_rec.p, sizeof(float) * (size_t)nrec * nsteps));
    CK(h, cudaMalloc(&d_res.p, sizeof(float) * (size_t)nrec * nsteps));
    CK(h, cudaMemcpyAsync(d_idx.p, idx.data(), sizeof(long long) * nrec, cudaMemcpyHostToDevice, h->stream));
    const long long* didx = (const long long*)d_idx.p;
    const HeatLap c = heat_lap_of(h);
    const int D = h->cfg.D;

    // forward with checkpoints and receiver samples
    for (int n = 0; n < nsteps; ++n) {
        float* in = static_cast<float*>(h->buf[h->cur]);
        float* out = static_cast<float*>(h->buf[1 - h->cur]);
        if (n % K == 0) CK(h, cudaMemcpyAsync(ckpt[n / K], in, fb, cudaMemcpyDeviceToDevice, h->stream));
        CK(h, launch_heat_kappa_step(in, out, h->mat[0], h->L, D, c, h->stream));
        h->cur = 1 - h->cur;
        CK(h, adjoint_sample(out, didx, nrec, (float*)d_rec.p + (size_t)n * nrec, h->stream));
    }
    std::vector<float> syn((size_t)nrec * nsteps), res((size_t)nrec * nsteps);
    CK(h, cudaMemcpyAsync(syn.data(), d_rec.p, sizeof(float) * syn.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    double J = 0.0;
    for (size_t i = 0; i < syn.size(); ++i) {
        const double r = (double)syn[i] - (double)d_obs[i];
        res[i] = (float)r;
        J += 0.5 * r * r;
    }
    if (misfit) *misfit = J;
    if (d_syn) std::copy(syn.begin(), syn.end(), d_syn);
    CK(h, cudaMemcpyAsync(d_res.p, res.data(), sizeof(float) * res.size(), cudaMemcpyHostToDevice, h->stream));

    // reverse sweep, segment by segment with recomputation
    for (long long sgi = (long long)nseg - 1; sgi >= 0; --sgi) {
        const int n0 = (int)sgi * K;
        const int n1 = std::min(nsteps, n0 + K);
        auto u_at = [&](int k) -> float* { return k == 0 ? ckpt[sgi] : slot[(size_t)k]; };
        for (int n = n0; n < n1; ++n)
            CK(h, launch_heat_kappa_step(u_at(n - n0), u_at(n - n0 + 1), h->mat[0], h->L, D, c, h->stream));
        for (int n = n1 - 1; n >= n0; --n) {
            CK(h, adjoint_inject(lam, didx, nrec, (const float*)d_res.p + (size_t)n * nrec, h->stream));
            CK(h, launch_heat_adjoint_step(lam, yb, u_at(n - n0), h->mat[0], g, h->L, D, c, h->stream));
        }
    }
    if (grad_kappa) {
        const size_t ncell = (size_t)h->cfg.env[0] * h->cfg.env[1] * h->cfg.env[2];
        DevBuf d_out;
        CK(h, cudaMalloc(&d_out.p, ncell * sizeof(double)));
        CK(h, adjoint_grad_out(g, nullptr, 0, h->L, (double*)d_out.p, h->stream));
        CK(h, cudaMemcpyAsync(grad_kappa, d_out.p, ncell * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    h->ts = nsteps;
    return check_status(h);
}

// ---------------------------------------------------------------- per-block entries
namespace {

int edge_from_flags(const char* ef)
{
    if (!ef) return 0;
    int e = 0;
    for (int a = 0; a < 3; ++a) {
        // plain char is unsigned on aarch64: read the flags as signed bytes
        const signed char v = static_cast<signed char>(ef[a]);
        if (v < 0) e |= 1 << (2 * a);
        if (v > 0) e |= 1 << (2 * a + 1);
    }
    return e;
}

struct Scratch {
    void* p[2] = {nullptr, nullptr};
    ~Scratch()
    {
        for (int i = 0; i < 2; ++i)
            if (p[i]) cudaFree(p[i]);
    }
};

}  // namespace

b2r_status b2r_heat_3D_gpu_main(float* h_in, int R, int D, const char* edge_flag, int Ngx, int Ngy,
                                int Ngz, double alpha_dt, double dx, double dy, double dz,
                                void* cuda_stream, double* gpu_seconds)
{
    if (!h_in) return fail(nullptr, B2R_ERR_ARG, "null h_in");
    if (D < 1 || D > 4) return fail(nullptr, B2R_ERR_ARG, "unsupported delta %d", D);
    if (R < 1) return fail(nullptr, B2R_ERR_ARG, "R must be >= 1");
    const int H = R * D;
    const int n[3] = {Ngx, Ngy, Ngz};
    int B[3];
    for (int a = 0; a < 3; ++a) {
        B[a] = n[a] - 2 * H;
        if (B[a] < 1) return fail(nullptr, B2R_ERR_ARG, "block too small for R*D = %d", H);
    }
    const int nb[3] = {1, 1, 1};
    BlockLayout L{};
    fill_layout(L, n, B, nb, H, 4, 0, edge_from_flags(edge_flag));
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    const size_t fb = (size_t)L.bstride * sizeof(float);
    Scratch s;
    int* d_status = nullptr;
    CK(nullptr, cudaMalloc(&s.p[0], fb));
    CK(nullptr, cudaMalloc(&s.p[1], fb));
    CK(nullptr, cudaMalloc(&d_status, sizeof(int)));
    CK(nullptr, cudaMemsetAsync(d_status, 0, sizeof(int), st));
    // host block (dense rows of Ngx) -> pitched device rows (heat-3D.cu:590-592)
    for (int b = 0; b < 2; ++b)
        CK(nullptr, cudaMemcpy2DAsync((float*)s.p[b] + L.xoff, L.P * sizeof(float), h_in,
                                      Ngx * sizeof(float), Ngx * sizeof(float), (size_t)Ngy * Ngz,
                                      cudaMemcpyHostToDevice, st));
    CUtensorMap tm[2];
    for (int b = 0; b < 2; ++b)
        if (!make_block_tmap(&tm[b], s.p[b], L, 4, heat_box_w(), heat_box_h(D), 1)) {
            cudaFree(d_status);
            return fail(nullptr, B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed");
        }
    const HeatCoef hc = heat_coef(D, alpha_dt, dx, dy, dz);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    int cur = 0;
    for (int i = 0; i < R; ++i) {   // heat-3D.cu:602-628
        cudaError_t e = launch_heat_substep(&tm[cur], (float*)s.p[1 - cur], L, D, i, hc, d_status, st);
        if (e != cudaSuccess) {
            cudaFree(d_status);
            return fail(nullptr, B2R_ERR_CUDA, "heat launch: %s", cudaGetErrorString(e));
        }
        cur = 1 - cur;
    }
    cudaEventRecord(e1, st);
    // planes [R*D, Ngz-R*D) back to the host (heat-3D.cu:633-635)
    const int zc = Ngz - 2 * H;
    CK(nullptr, cudaMemcpy2DAsync(h_in + (size_t)H * Ngx * Ngy, Ngx * sizeof(float),
                                  (float*)s.p[cur] + L.xoff + (size_t)H * L.plane, L.P * sizeof(float),
                                  Ngx * sizeof(float), (size_t)Ngy * zc, cudaMemcpyDeviceToHost, st));
    int dev_st = 0;
    CK(nullptr, cudaMemcpyAsync(&dev_st, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_status);
    if (gpu_seconds) *gpu_seconds = ms / 1000.0;
    if (dev_st != DEV_OK) return fail(nullptr, B2R_ERR_TIMEOUT, "device wait gave up (code %d)", dev_st);
    return B2R_OK;
}

b2r_status b2r_gol_3D_gpu_main(uint8_t* h_in, int R, const char* edge_flag, int Ngx, int Ngy,
                               int Ngz, void* cuda_stream, double* gpu_seconds)
{
    if (!h_in) return fail(nullptr, B2R_ERR_ARG, "null h_in");
    if (R < 1) return fail(nullptr, B2R_ERR_ARG, "R must be >= 1");
    const int H = R;
    const int n[3] = {Ngx, Ngy, Ngz};
    int B[3];
    for (int a = 0; a < 3; ++a) {
        B[a] = n[a] - 2 * H;
        if (B[a] < 1) return fail(nullptr, B2R_ERR_ARG, "block too small for R = %d", R);
    }
    const int nb[3] = {1, 1, 1};
    BlockLayout L{};
    fill_layout(L, n, B, nb, H, 1, 0, edge_from_flags(edge_flag));
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    const size_t fb = (size_t)L.bstride;
    Scratch s;
    CK(nullptr, cudaMalloc(&s.p[0], fb));
    CK(nullptr, cudaMalloc(&s.p[1], fb));
    for (int b = 0; b < 2; ++b)   // gol-3D.cu:126-129
        CK(nullptr, cudaMemcpy2DAsync((uint8_t*)s.p[b] + L.xoff, L.P, h_in, Ngx, Ngx,
                                      (size_t)Ngy * Ngz, cudaMemcpyHostToDevice, st));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    int cur = 0;
    for (int i = 0; i < R; ++i) {  // gol-3D.cu:138-145
        cudaError_t e = launch_gol_substep((const uint8_t*)s.p[cur], (uint8_t*)s.p[1 - cur], L, i, st);
        if (e != cudaSuccess) return fail(nullptr, B2R_ERR_CUDA, "gol launch: %s", cudaGetErrorString(e));
        cur = 1 - cur;
    }
    cudaEventRecord(e1, st);
    // whole block back (gol-3D.cu:149)
    CK(nullptr, cudaMemcpy2DAsync(h_in, Ngx, (uint8_t*)s.p[cur] + L.xoff, L.P, Ngx, (size_t)Ngy * Ngz,
                                  cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (gpu_seconds) *gpu_seconds = ms / 1000.0;
    return B2R_OK;
}

b2r_status b2r_write_block_data(b2r_handle* h, int field, int block, int time_step, const char* dir,
                                int text, char* path_out, int path_cap)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (h->cfg.model == B2R_MODEL_GOL) return fail(h, B2R_ERR_ARG, "block data files hold float cells");
    if (block < 0 || block >= h->L.nblk) return fail(h, B2R_ERR_ARG, "block %d outside 0..%d", block, h->L.nblk - 1);
    static const char* const eq_names[10] = {"vx", "vy", "vz", "sxx", "sxy", "sxz",
                                             "syy", "syz", "szz", "displacement"};
    const char* name = nullptr;
    const void* src = nullptr;
    if (h->cfg.model == B2R_MODEL_HEAT) {
        if (field == 0) {
            name = "u";
            src = h->buf[h->cur];
        } else if (field == B2R_F_KAPPA && h->mat[0]) {
            name = "kappa";
            src = h->mat[0];
        }
    } else if (field >= 0 && field < h->nfld) {
        name = eq_names[field];
        src = h->fld[field];
    } else if (field >= B2R_F_LAMBDA && field <= B2R_F_BUOY && h->mat[0]) {
        static const char* const mat_names[3] = {"lambda", "mu", "buoyancy"};
        name = mat_names[field - B2R_F_LAMBDA];
        src = h->mat[field - B2R_F_LAMBDA];
    }
    if (!src) return fail(h, B2R_ERR_ARG, "field %d has no data on this handle", field);
    const BlockLayout& L = h->L;
    std::string path = dir && dir[0] ? std::string(dir) + "/" : std::string();
    path += name;
    if (block > 0) path += "-b" + std::to_string(block);
    path += "-" + std::to_string(time_step) + (text ? ".txt" : ".bin");
    const size_t ncell = (size_t)L.n[0] * L.n[1] * L.n[2];
    std::vector<float> cells(ncell);
    const float* blk = static_cast<const float*>(src) + (size_t)block * L.bstride + L.xoff;
    CK(h, cudaMemcpy2DAsync(cells.data(), L.n[0] * sizeof(float), blk, L.P * sizeof(float),
                            L.n[0] * sizeof(float), (size_t)L.n[1] * L.n[2], cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    std::ofstream out(path, std::ios::binary);
    if (!out) return fail(h, B2R_ERR_ARG, "cannot open %s", path.c_str());
    if (text) {
        for (int z = 0; z < L.n[2]; ++z)
            for (int y = 0; y < L.n[1]; ++y) {
                const float* row = cells.data() + ((size_t)z * L.n[1] + y) * L.n[0];
                for (int x = 0; x < L.n[0]; ++x) out << row[x] << ",";
                out << "\n";
            }
    } else {
        const int32_t hdr[3] = {L.n[0], L.n[1], L.n[2]};
        out.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
        out.write(reinterpret_cast<const char*>(cells.data()), (std::streamsize)(ncell * sizeof(float)));
    }
    out.close();
    if (!out) return fail(h, B2R_ERR_ARG, "writing %s failed", path.c_str());
    if (path_out && path_cap > 0) std::snprintf(path_out, (size_t)path_cap, "%s", path.c_str());
    return B2R_OK;
}

b2r_status b2r_eqwp_gpu_main(b2r_handle* h, int ts, int R, double* gpu_seconds)
{
    if (!h) return fail(nullptr, B2R_ERR_ARG, "null handle");
    if (h->cfg.model != B2R_MODEL_EQWP_REF)
        return fail(h, B2R_ERR_ARG, "eqwp_gpu_main needs a B2R_MODEL_EQWP_REF handle");
    if (R < 1 || R > h->cfg.R) return fail(h, B2R_ERR_ARG, "R must be in 1..%d", h->cfg.R);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, h->stream);
    b2r_status st = B2R_OK;
    const long long save = h->ts;
    for (int i = 0; i < R && st == B2R_OK; ++i) {   // eqwp.cu:677-686
        h->ts = ts + i;
        st = substep(h, i);
    }
    h->ts = save;
    cudaEventRecord(e1, h->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (gpu_seconds) *gpu_seconds = ms / 1000.0;
    if (st != B2R_OK) return st;
    return check_status(h);
}

}  // extern "C"
