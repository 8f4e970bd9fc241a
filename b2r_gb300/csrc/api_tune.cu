// api_tune.cu -- the launch-schedule knobs of a handle (b2r_set_tuning,
// b2r_get_tuning) and the autotuners that time them on the live fields.
#include "api_internal.h"

using namespace b2r_api;

extern "C" {


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
    case B2R_TUNE_TB16: h->tune.tb16 = value != 0; break;
    case B2R_TUNE_TB_NARROW: h->tune.tbn = value != 0; break;
    case B2R_TUNE_TB_R2: h->tune.r2 = value != 0; break;
    case B2R_TUNE_EQWP_TMA: h->eqwp_tma = value != 0; break;
    case B2R_TUNE_EQWP_OVERLAP: h->eqwp_overlap = value != 0; break;
    case B2R_TUNE_GOL_ROWS: h->gol_rows = value < 0 ? 0 : value; break;
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
    case B2R_TUNE_TB16: *value = h->tune.tb16; break;
    case B2R_TUNE_TB_NARROW: *value = h->tune.tbn; break;
    case B2R_TUNE_TB_R2: *value = h->tune.r2; break;
    case B2R_TUNE_EQWP_TMA: *value = h->eqwp_tma ? 1 : 0; break;
    case B2R_TUNE_EQWP_OVERLAP: *value = h->eqwp_overlap ? 1 : 0; break;
    case B2R_TUNE_GOL_ROWS: *value = h->gol_rows; break;
    default: return fail(nullptr, B2R_ERR_ARG, "unknown tuning key %d", key);
    }
    return B2R_OK;
}

// Game of Life and the staggered elastic wave: the same timed search over
// their kernel choices -- generations per pass, bit-sliced or byte cells and
// the period-end halo fill (GoL); the one-pass or two-pass step (elastic
// wave).  Trials run on the live fields, which are restored afterwards.
struct KnobSet {
    int tblock, gol_bytes, gol_push, eqwp_fused, eqwp_tma = 0, eqwp_overlap = 0, gol_rows = 0;
};
static std::map<TuneKey, KnobSet> g_knob_cache;

static void apply_knobs(b2r_handle* h, const KnobSet& k)
{
    h->tune.tblock = k.tblock;
    h->gol_bytes = k.gol_bytes != 0;
    h->gol_push = k.gol_push != 0;
    h->eqwp_fused = k.eqwp_fused != 0;
    h->eqwp_tma = k.eqwp_tma != 0;
    h->eqwp_overlap = k.eqwp_overlap != 0;
    h->gol_rows = k.gol_rows;
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
    const KnobSet cur{h->tune.tblock, h->gol_bytes, h->gol_push, h->eqwp_fused, h->eqwp_tma, h->eqwp_overlap,
                      h->gol_rows};
    if (h->cfg.model == B2R_MODEL_GOL) {
        // the several-generation bit-sliced pass also by its band height:
        // 32 rows, 48, or the whole block (one band)
        for (int tb : {1, 2, 4})
            for (int bytes = 0; bytes < 2; ++bytes)
                for (int push = 0; push < 2; ++push)
                    if (!push || (tb >= 2 && !bytes))
                        for (int rows : {0, 48, 1 << 20})
                            if (rows == 0 || (tb >= 2 && !bytes))
                                cands.push_back({tb, bytes, push, cur.eqwp_fused, cur.eqwp_tma, cur.eqwp_overlap,
                                                 rows});
    } else {
        // the two-pass step with plain-load or TMA-streamed stress stage (and,
        // on several blocks, with the exchange overlapped), the one-pass step
        const bool stag = h->cfg.model == B2R_MODEL_EQWP_STAG;
        cands.push_back({cur.tblock, cur.gol_bytes, cur.gol_push, 0, 0, 0, cur.gol_rows});
        if (stag) cands.push_back({cur.tblock, cur.gol_bytes, cur.gol_push, 0, 1, 0, cur.gol_rows});
        if (stag && (h->L.nblk > 1 || h->L.periodic))
            cands.push_back({cur.tblock, cur.gol_bytes, cur.gol_push, 0, 0, 1, cur.gol_rows});
        cands.push_back({cur.tblock, cur.gol_bytes, cur.gol_push, 1, 0, 0, cur.gol_rows});
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
    // restore every field even after a failed trial; report the first failure
    cudaError_t rerr = cudaSuccess;
    for (int f = 0; f < nsave; ++f) {
        void* dst = eq ? (void*)h->fld[f] : h->buf[h->cur];
        const cudaError_t e = cudaMemcpyAsync(dst, save[(size_t)f], fb, cudaMemcpyDeviceToDevice, h->stream);
        if (rerr == cudaSuccess) rerr = e;
    }
    const cudaError_t se = cudaStreamSynchronize(h->stream);
    if (rerr == cudaSuccess) rerr = se;
    apply_knobs(h, st == B2R_OK ? bestK : cur);
    drop_graphs(h);
    if (st != B2R_OK) return st;
    CK(h, rerr);
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
    // candidates: the several-step sweeps (radius 1: two, three and four steps
    // per pass) by z-chunk, then the one-step sweep by z-chunk x persistent
    // CTAs per SM x PDL.  Every trial advances a multiple of 12 time steps,
    // so that each schedule runs whole passes.
    struct Cand { int tb, zc2, zc, cp, pdl, tb16, tbn, r2 = 0; };
    std::vector<Cand> cands;
    if (h->cfg.D == 1) {
        for (int z2 : {4, 8, 16, 32, 64}) cands.push_back({2, z2, 0, 0, 1, 0, 0});
        for (int tbn = 0; tbn < 2; ++tbn) {
            for (int z2 : {0, 32, 96}) cands.push_back({2, z2, 0, 0, 1, 1, tbn});
            for (int tb : {3, 4})
                for (int z2 : {0, 32, 48, 96, 128}) cands.push_back({tb, z2, 0, 0, 1, 0, tbn});
        }
        trial_steps = (trial_steps + 11) / 12 * 12;
    } else if (h->cfg.D == 2) {
        for (int z2 : {0, 32, 64, 96, 128}) cands.push_back({2, z2, 0, 0, 1, 0, 0, 1});
        trial_steps = (trial_steps + 1) / 2 * 2;
    }
    for (int pdl = 0; pdl < 2; ++pdl)
        for (int zc : zchunks)
            for (int cp : persist)
                if (zc <= h->L.n[2]) cands.push_back({1, 0, zc, cp, pdl, 0, 0});
    for (const Cand& cd : cands) {
        if (st != B2R_OK) break;
        h->tune.tb16 = cd.tb16;
        h->tune.tbn = cd.tbn;
        h->tune.r2 = cd.r2;
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
    // restore the field even after a failed trial; report the first failure
    cudaError_t rerr = cudaMemcpyAsync(h->buf[h->cur], save, fb, cudaMemcpyDeviceToDevice, h->stream);
    const cudaError_t se = cudaStreamSynchronize(h->stream);
    if (rerr == cudaSuccess) rerr = se;
    if (st != B2R_OK) return st;
    CK(h, rerr);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key_of(h)] = bestT;
    }
    drop_graphs(h);
    if (best) { best[0] = bestT.tblock == 2 ? bestT.zchunk2 : bestT.zchunk; best[1] = bestT.ctas_per_sm; best[2] = bestT.pdl; }
    if (best_ms) *best_ms = bestMs / trial_steps;
    return check_status(h);
}

}  // extern "C"
