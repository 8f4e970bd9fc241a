// b2r_api.cu -- the C ABI of libb2r (include/b2r.h): handles, geometry,
// device memory of the resident subdomains, the period driver (halo
// exchange + R sub-steps, b2r.cpp:179-221), host runs and block data files,
// and the reference-shaped per-block entries (heat_3D_gpu_main,
// gol_3D_gpu_main, eqwp_gpu_main).  The tuning knobs and autotuners are in
// api_tune.cu, the misfit-gradient drivers in api_adjoint.cu.
#include "api_internal.h"

namespace b2r_api {


// autotuning results per (model, D, block size, blocks), shared by handles

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
            (!make_block_tmap(&h->tmap2[b], h->buf[b], h->L, 4, heat2_box_w(), heat2_box_h(), 1) ||
             !make_block_tmap(&h->tmap3[b], h->buf[b], h->L, 4, heat_tb_box_w(0), heat_tb_box_h(0), 1) ||
             !make_block_tmap(&h->tmap4[b], h->buf[b], h->L, 4, heat_tb_box_w(1), heat_tb_box_h(1), 1)))
            return fail(h, B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed for the heat field");
        if (h->cfg.D == 2 &&
            !make_block_tmap(&h->tmap3[b], h->buf[b], h->L, 4, heat_tb2_box_w(), heat_tb2_box_h(), 1))
            return fail(h, B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed for the heat field");
    }
    return B2R_OK;
}

// Steps per HBM pass the heat schedule allows: radius 1 up to tblock (<= 4),
// radius 2 two (tblock >= 2); 1 = the one-step sweep.
int heat_max_pass_steps(const b2r_handle* h)
{
    if (h->cfg.model != B2R_MODEL_HEAT || h->tune.tblock < 2) return 1;
    if (h->cfg.D == 1) return std::min(h->tune.tblock, 4);
    return h->cfg.D == 2 && h->tune.r2 ? 2 : 1;
}

// Time steps one heat launch may take from sub-step i with `left` to go: up
// to heat_max_pass_steps, and no halo exchange may fall between them --
// within one period, or any number when the exchange is empty (one block,
// not periodic); 1 = the one-step sweep.
int heat_pass_steps(const b2r_handle* h, int i, int left)
{
    if (heat_max_pass_steps(h) < 2) return 1;
    int k = std::min(heat_max_pass_steps(h), left);
    if (!(h->L.nblk == 1 && !h->L.periodic)) k = std::min(k, h->cfg.R - i);
    return std::max(k, 1);
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

// Periods per graph replay: at least 32 time steps; when heat passes may
// run across period starts (radius 1, several steps per pass, nothing to
// exchange), also a multiple of the steps per pass, so that no replay ends
// with a shorter pass.
int graph_periods(const b2r_handle* h)
{
    int m = (32 + h->cfg.R - 1) / h->cfg.R;
    const int k = heat_max_pass_steps(h);
    if (k >= 2 && h->L.nblk == 1 && !h->L.periodic)
        while ((m * h->cfg.R) % k) ++m;
    return m;
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

b2r_status exchange_all(b2r_handle* h, bool staged, cudaStream_t xst)
{
    const BlockLayout& L = h->L;
    const cudaStream_t st = xst ? xst : h->stream;
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
        if (gather) CK(h, launch_halo_gather<uint8_t>(fs, 1, L, st));
        else CK(h, launch_halo_exchange<uint8_t>(fs, 1, L, static_cast<uint8_t*>(bounce), st));
    } else {
        FieldSet<float> fs{};
        if (nf == 1) fs.p[0] = static_cast<float*>(h->buf[h->cur]);
        else
            for (int f = 0; f < nf; ++f) fs.p[f] = h->fld[f];
        if (gather) CK(h, launch_halo_gather<float>(fs, nf, L, st));
        else CK(h, launch_halo_exchange<float>(fs, nf, L, static_cast<float*>(bounce), st));
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

b2r_status substep(b2r_handle* h, int i, bool xnext)
{
    h->upmask = 0;
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
        if (h->eqwp_tma) {
            // tensor maps of the current field set (built on first use and
            // whenever a one-pass step has swapped the sets)
            const void* want[11] = {h->fld[B2R_F_VX], h->fld[B2R_F_VY], h->fld[B2R_F_VZ],
                                    h->fld[B2R_F_SXX], h->fld[B2R_F_SYY], h->fld[B2R_F_SZZ],
                                    h->fld[B2R_F_SXY], h->fld[B2R_F_SXZ], h->fld[B2R_F_SYZ], h->mat[0], h->mat[1]};
            if (!std::equal(want, want + 11, h->emaps_of)) {
                h->emaps.clear();
                std::copy(want, want + 11, h->emaps_of);
            }
            int tx = 0, ty = 0;
            eqwp_stress_tma_shape(h->L, i, &tx, &ty);
            auto it = h->emaps.find(tx);
            if (it == h->emaps.end()) {
                EqwpStressMaps m{};
                for (int k = 0; k < 11; ++k) {
                    const bool v = k < 3;
                    if (!make_block_tmap(v ? &m.v[k] : &m.o[k - 3], want[k], h->L, 4, v ? 4 * tx + 8 : 4 * tx,
                                         v ? ty + 4 : ty, 1))
                        return fail(h, B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed for the elastic-wave fields");
                }
                it = h->emaps.emplace(tx, m).first;
            }
            const int ts = (int)h->ts;
            const float amp = (p.src_host && ts >= 0 && ts < p.src_len) ? p.src_host[ts] : 0.f;
            CK(h, launch_eqwp_stag_velocity(h->fld, h->mat, h->L, i, p, h->stream));
            CK(h, launch_eqwp_stress_tma(it->second, tx, h->fld, h->L, i, amp, p, h->d_status, h->stream));
            return B2R_OK;
        }
        if (xnext && h->eqwp_overlap && i == h->cfg.R - 1 && (h->L.nblk > 1 || h->L.periodic)) {
            // the last sub-step of a period: the stress tiles that hold the
            // cells the next exchange reads, then that exchange on the stream
            // xs while the other tiles finish (they read no halo cell)
            if (!h->xs) {   // the stream and its two events, kept only all together
                int lo = 0, hi = 0;
                cudaStream_t xs = nullptr;
                cudaEvent_t ev[2] = {};
                cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
                if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&xs, cudaStreamNonBlocking, hi);
                for (int k = 0; k < 2 && e == cudaSuccess; ++k)
                    e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
                if (e != cudaSuccess) {
                    for (cudaEvent_t x : ev)
                        if (x) cudaEventDestroy(x);
                    if (xs) cudaStreamDestroy(xs);
                    return fail(h, B2R_ERR_CUDA, "exchange stream: %s", cudaGetErrorString(e));
                }
                h->xs = xs;
                h->xev[0] = ev[0];
                h->xev[1] = ev[1];
            }
            CK(h, launch_eqwp_stag_velocity(h->fld, h->mat, h->L, i, p, h->stream));
            CK(h, launch_eqwp_stag_stress(h->fld, h->mat, h->L, i, (int)h->ts, p, 1, h->stream));
            CK(h, cudaEventRecord(h->xev[0], h->stream));
            CK(h, cudaStreamWaitEvent(h->xs, h->xev[0], 0));
            if (b2r_status st = exchange_all(h, false, h->xs); st != B2R_OK) return st;
            CK(h, cudaEventRecord(h->xev[1], h->xs));
            CK(h, launch_eqwp_stag_stress(h->fld, h->mat, h->L, i, (int)h->ts, p, 2, h->stream));
            CK(h, cudaStreamWaitEvent(h->stream, h->xev[1], 0));
            h->xdone = true;
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
// (skipped right after an upload, whose scatter filled the halos), several
// steps per launch where heat_pass_steps or gol_pass_gens allow, one
// otherwise.
b2r_status advance(b2r_handle* h, int n)
{
    b2r_status st;
    if (n > 0) h->upmask = 0;
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
                                             h->stream, h->gol_rows));
            h->cur = 1 - h->cur;
            h->ts += gg;
            s += gg;
            h->halos_fresh = push;
        } else if (const int k = heat_pass_steps(h, i, n - s); k >= 2) {
            if (h->cfg.D == 2) {
                CK(h, launch_heat_substep_tb2(&h->tmap3[h->cur], static_cast<float*>(h->buf[1 - h->cur]), h->L, i,
                                              h->hc, h->d_status, h->stream, h->tune.zchunk2));
                h->cur = 1 - h->cur;
            } else if (k == 2 && !h->tune.tb16) {
                if ((st = substep2(h, i)) != B2R_OK) return st;
            } else {
                CK(h, launch_heat_substep_tb(k, h->tune.tbn, h->tune.tbn ? &h->tmap4[h->cur] : &h->tmap3[h->cur],
                                             static_cast<float*>(h->buf[1 - h->cur]), h->L,
                                             i, h->hc, h->d_status, h->stream, h->tune.zchunk2));
                h->cur = 1 - h->cur;
            }
            h->ts += k;
            s += k;
        } else {
            if ((st = substep(h, i, true)) != B2R_OK) return st;
            h->ts++;
            ++s;
            // the next period's halos were exchanged inside the sub-step
            h->halos_fresh = h->xdone;
            h->xdone = false;
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

}  // namespace b2r_api

using namespace b2r_api;


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
    if (h->xs) cudaStreamDestroy(h->xs);
    for (cudaEvent_t e : h->xev)
        if (e) cudaEventDestroy(e);
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
        CK(h, launch_scatter<float>(static_cast<const float*>(dsrc), h->mat[0], nullptr, h->L, h->shell,
                                    h->stream));
        return B2R_OK;
    }
    void* dst2 = nullptr;   // written with the same cells in the same pass
    if (is_mat) {
        dst = h->mat[field - B2R_F_LAMBDA];
    } else if (eq) {
        dst = h->fld[field];
        dst2 = h->fld2[field];   // both staggered field sets carry the shell
    } else {
        dst = h->buf[h->cur];
        dst2 = h->buf[1 - h->cur];   // so do both ping-pong buffers (heat-3D.cu:591-592)
    }
    if (h->cell_bytes == 1)
        CK(h, launch_scatter<uint8_t>(static_cast<const uint8_t*>(dsrc), static_cast<uint8_t*>(dst),
                                      static_cast<uint8_t*>(dst2), h->L, h->shell, h->stream));
    else
        CK(h, launch_scatter<float>(static_cast<const float*>(dsrc), static_cast<float*>(dst),
                                    static_cast<float*>(dst2), h->L, h->shell, h->stream));
    h->ts = 0;
    // the scatter filled this field's halos; the others are fresh only if
    // they were, or once every field has been uploaded since the last step
    if (!h->halos_fresh && !is_mat) {   // material never changes: its halos stay consistent
        const int nf = eq ? h->nfld : 1;
        h->upmask |= 1u << (eq ? field : 0);
        h->halos_fresh = h->upmask == (nf >= 32 ? ~0u : (1u << nf) - 1u);
    }
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
            const int periods = graph_periods(h);
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
                h->upmask = 0;
                s += unit;
                continue;
            }
        }
        // up to the next period start (or all of it when nothing is graphed)
        int chunk = nsteps - s;
        if (use_graphs && i != 0) chunk = std::min(chunk, h->cfg.R - i);
        if (use_graphs && i == 0) chunk = std::min(chunk, graph_periods(h) * h->cfg.R);
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
    if (field != 0) return fail(h, B2R_ERR_ARG, "invalid field id %d", field);
    for (int i = 0; i < count; ++i)
        if (!host_in[i] || !host_out[i]) return fail(h, B2R_ERR_ARG, "null buffer for problem %d", i);
    // a problem is every field of the model, back to back in field-id order
    // (the elastic wave's wavefield components; one field for heat and GoL)
    const int nf = h->nfld > 0 ? h->nfld : 1;
    const size_t fbytes = domain_cells(h) * h->cell_bytes;
    const size_t bytes = fbytes * nf;
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
            if (e) cudaEventDestroy(e);
            e = nullptr;
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
        for (int f = 0; f < nf; ++f)
            if ((st = b2r_upload(h, f, static_cast<const char*>(in[k]) + f * fbytes, 1)) != B2R_OK) return st;
        CK(h, cudaEventRecord(h->ev[IN_FREE][k], h->stream));
        if ((st = b2r_step(h, nsteps)) != B2R_OK) return st;
        CK(h, cudaStreamWaitEvent(h->stream, h->ev[OUT_FREE][k], 0));   // result of problem i-2 copied out
        for (int f = 0; f < nf; ++f)
            if ((st = b2r_download(h, f, static_cast<char*>(out[k]) + f * fbytes, 1)) != B2R_OK) return st;
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

}  // extern "C"

namespace b2r_api {

b2r_status HeatBlockRun::begin(const float* h_in, int R_, int D, int edge, int Ngx, int Ngy, int Ngz_,
                               double alpha_dt, double dx, double dy, double dz, cudaStream_t st_)
{
    R = R_;
    H = R_ * D;
    Ngz = Ngz_;
    st = st_;
    const int n[3] = {Ngx, Ngy, Ngz};
    int B[3];
    for (int a = 0; a < 3; ++a) {
        B[a] = n[a] - 2 * H;
        if (B[a] < 1) return fail(nullptr, B2R_ERR_ARG, "block too small for R*D = %d", H);
    }
    const int nb[3] = {1, 1, 1};
    fill_layout(L, n, B, nb, H, 4, 0, edge);
    const size_t fb = (size_t)L.bstride * sizeof(float);
    CK(nullptr, cudaMalloc(&buf[0], fb));
    CK(nullptr, cudaMalloc(&buf[1], fb));
    CK(nullptr, cudaMalloc(&status, sizeof(int)));
    CK(nullptr, cudaMemsetAsync(status, 0, sizeof(int), st));
    // host block (dense rows of Ngx) -> pitched device rows (heat-3D.cu:590-592)
    for (int b = 0; b < 2; ++b)
        CK(nullptr, cudaMemcpy2DAsync(static_cast<float*>(buf[b]) + L.xoff, L.P * sizeof(float), h_in,
                                      Ngx * sizeof(float), Ngx * sizeof(float), (size_t)Ngy * Ngz,
                                      cudaMemcpyHostToDevice, st));
    CUtensorMap tm[2];
    for (int b = 0; b < 2; ++b)
        if (!make_block_tmap(&tm[b], buf[b], L, 4, heat_box_w(), heat_box_h(D), 1))
            return fail(nullptr, B2R_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    const HeatCoef hc = heat_coef(D, alpha_dt, dx, dy, dz);
    CK(nullptr, ev.create());
    CK(nullptr, cudaEventRecord(ev.e0, st));
    cur = 0;
    for (int i = 0; i < R; ++i) {   // heat-3D.cu:602-628
        cudaError_t e = launch_heat_substep(&tm[cur], static_cast<float*>(buf[1 - cur]), L, D, i, hc,
                                            static_cast<int*>(status), st);
        if (e != cudaSuccess) return fail(nullptr, B2R_ERR_CUDA, "heat launch: %s", cudaGetErrorString(e));
        cur = 1 - cur;
    }
    CK(nullptr, cudaEventRecord(ev.e1, st));
    return B2R_OK;
}

b2r_status HeatBlockRun::end(float* h_out, double* gpu_seconds)
{
    // planes [R*D, Ngz-R*D) back to the host (heat-3D.cu:633-635)
    const int Ngx = L.n[0], Ngy = L.n[1];
    const int zc = Ngz - 2 * H;
    CK(nullptr, cudaMemcpy2DAsync(h_out + (size_t)H * Ngx * Ngy, Ngx * sizeof(float),
                                  static_cast<float*>(buf[cur]) + L.xoff + (size_t)H * L.plane,
                                  L.P * sizeof(float), Ngx * sizeof(float), (size_t)Ngy * zc,
                                  cudaMemcpyDeviceToHost, st));
    int dev_st = 0;
    CK(nullptr, cudaMemcpyAsync(&dev_st, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaStreamSynchronize(st));
    if (gpu_seconds) *gpu_seconds = ev.seconds();
    if (dev_st != DEV_OK) return fail(nullptr, B2R_ERR_TIMEOUT, "device wait gave up (code %d)", dev_st);
    return B2R_OK;
}

HeatBlockRun::~HeatBlockRun()
{
    for (int i = 0; i < 2; ++i)
        if (buf[i]) cudaFree(buf[i]);
    if (status) cudaFree(status);
}

int edge_bits_of_flags(const char* edge_flag) { return edge_from_flags(edge_flag); }

}  // namespace b2r_api

extern "C" {

b2r_status b2r_heat_3D_gpu_main(float* h_in, int R, int D, const char* edge_flag, int Ngx, int Ngy,
                                int Ngz, double alpha_dt, double dx, double dy, double dz,
                                void* cuda_stream, double* gpu_seconds)
{
    if (!h_in) return fail(nullptr, B2R_ERR_ARG, "null h_in");
    if (D < 1 || D > 4) return fail(nullptr, B2R_ERR_ARG, "unsupported delta %d", D);
    if (R < 1) return fail(nullptr, B2R_ERR_ARG, "R must be >= 1");
    HeatBlockRun run;
    b2r_status s = run.begin(h_in, R, D, edge_from_flags(edge_flag), Ngx, Ngy, Ngz, alpha_dt, dx, dy, dz,
                             static_cast<cudaStream_t>(cuda_stream));
    if (s != B2R_OK) return s;
    return run.end(h_in, gpu_seconds);
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
    EventPair ev;
    CK(nullptr, ev.create());
    CK(nullptr, cudaEventRecord(ev.e0, st));
    int cur = 0;
    for (int i = 0; i < R; ++i) {  // gol-3D.cu:138-145
        cudaError_t e = launch_gol_substep((const uint8_t*)s.p[cur], (uint8_t*)s.p[1 - cur], L, i, st);
        if (e != cudaSuccess) return fail(nullptr, B2R_ERR_CUDA, "gol launch: %s", cudaGetErrorString(e));
        cur = 1 - cur;
    }
    CK(nullptr, cudaEventRecord(ev.e1, st));
    // whole block back (gol-3D.cu:149)
    CK(nullptr, cudaMemcpy2DAsync(h_in, Ngx, (uint8_t*)s.p[cur] + L.xoff, L.P, Ngx, (size_t)Ngy * Ngz,
                                  cudaMemcpyDeviceToHost, st));
    CK(nullptr, cudaStreamSynchronize(st));
    if (gpu_seconds) *gpu_seconds = ev.seconds();
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
