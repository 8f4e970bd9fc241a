// api_adjoint.cu -- the misfit-gradient drivers of the C ABI: receiver
// recordings, checkpointed forward runs, segment replays and the reverse
// sweeps of the elastic-wave and heat adjoints (adjoint.cu, heat_adjoint.cu).
#include "api_internal.h"

using namespace b2r_api;

extern "C" {

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
        const size_t nfields = nf_ckpt + nbuf * (nf_v + nf_a + 6) + 18 + 3;
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
    std::vector<float*> g32;            // FP32 partial gradient sums, folded into gp
    carve(3, g32);
    double* gp[3];
    for (int m = 0; m < 3; ++m, ws += gba) {
        gp[m] = reinterpret_cast<double*>(ws);
        CK(h, cudaMemsetAsync(gp[m], 0, gbytes, h->stream));
    }
    for (float* b : g32) CK(h, cudaMemsetAsync(b, 0, fb, h->stream));
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
            CK(h, adjoint_step(tp, vn, an, mat, g32.data(), h->L, dt_h, n == 0, h->adj_fused, h->stream));
            // the partial sums into FP64 on a fixed schedule of step numbers
            // (step 0 is the last reverse step, so nothing is left behind)
            if (n % adjoint_fold_steps() == 0) CK(h, adjoint_fold(g32.data(), gp, h->L, h->stream));
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
    h->upmask = 0;
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

}  // extern "C"
