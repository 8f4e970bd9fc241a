// b2r_main.cpp -- the B2R simulation main (b2r.cpp:120-250) on one GB300,
// through the C ABI of libb2r only: no MPI, the Bx*By*Bz subdomains live on
// one GPU and boundary_updating is the device-side exchange between them.
//
//   b2r_main R Bx By Bz [--model eqwp|stag|heat|gol] [--env X Y Z]
//            [--iters N] [--D d] [--direct] [--snapshot DIR] [--log]
//
// As in the reference: R and the block counts come from argv
// (b2r.cpp:139-146); ENV must divide by the block counts (b2r.cpp:154) and
// R*D <= min(B)/2 (b2r.cpp:54, checked by b2r_create); every R steps each
// field's halos are exchanged (b2r.cpp:197-206) and the model advances R
// steps (b2r.cpp:215); the summary lines follow b2r.cpp:226-238, with the
// MPI synchronisation time reported as the halo exchange time.  Defaults are
// the reference's compile-time settings (b2r_config.h:6-10, b2r.h:12):
// elastic wave, 3000 x 200 x 3000, D = 2, 600 iterations.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "b2r.h"

namespace {

struct Options {
    int R = 0, nb[3] = {0, 0, 0};
    std::string model = "eqwp";
    int env[3] = {3000, 200, 3000};
    int iters = 600;
    int D = -1;
    bool direct = false, log = false;
    std::string snapshot;
};

void usage()
{
    std::printf("not sufficient parameter given for execution.\n");
    std::printf("please set parameter B2R_B_R, BLOCK_DIM_(X,Y,Z)\n");
    std::printf("usage: b2r_main R Bx By Bz [--model eqwp|stag|heat|gol] [--env X Y Z] [--iters N]\n"
                "                [--D d] [--direct] [--snapshot DIR] [--log]\n");
}

bool parse(int argc, char** argv, Options& o)
{
    if (argc < 5) return false;
    o.R = std::atoi(argv[1]);
    for (int a = 0; a < 3; ++a) o.nb[a] = std::atoi(argv[2 + a]);
    for (int i = 5; i < argc; ++i) {
        const std::string k = argv[i];
        auto need = [&](int n) { return i + n < argc; };
        if (k == "--model" && need(1)) o.model = argv[++i];
        else if (k == "--env" && need(3))
            for (int a = 0; a < 3; ++a) o.env[a] = std::atoi(argv[++i]);
        else if (k == "--iters" && need(1)) o.iters = std::atoi(argv[++i]);
        else if (k == "--D" && need(1)) o.D = std::atoi(argv[++i]);
        else if (k == "--direct") o.direct = true;
        else if (k == "--snapshot" && need(1)) o.snapshot = argv[++i];
        else if (k == "--log") o.log = true;
        else {
            std::printf("unknown argument %s\n", k.c_str());
            return false;
        }
    }
    return o.R >= 1 && o.nb[0] >= 1 && o.nb[1] >= 1 && o.nb[2] >= 1 && o.iters >= 0;
}

}  // namespace

namespace {

double seconds_since(const std::chrono::steady_clock::time_point& t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

bool ok(b2r_status st, b2r_handle* h, const char* what)
{
    if (st == B2R_OK) return true;
    std::printf("%s failed: %s\n", what, b2r_last_error(h));
    return false;
}

// Initial state of the models that start from data: heat U[0,1) inside a
// zero shell (seed 1), Game of Life Bernoulli(0.3) on the torus (seed 2),
// and for the staggered elastic wave eight layers along y with vp in
// [2000, 4000] m/s, vs = vp / sqrt(3), rho in [2000, 2600] kg/m^3 (seed 3),
// dt at half the CFL limit and a 10 Hz Ricker source at the centre.
bool initialise(b2r_handle* h, const b2r_config& c)
{
    int n[3];
    const int shell = c.boundary == B2R_BC_PERIODIC ? 0 : c.D;
    for (int a = 0; a < 3; ++a) n[a] = c.env[a] + 2 * shell;
    const size_t cells = (size_t)n[0] * n[1] * n[2];
    auto inside = [&](size_t e) {
        const int x = (int)(e % n[0]), y = (int)((e / n[0]) % n[1]), z = (int)(e / ((size_t)n[0] * n[1]));
        return x >= shell && x < n[0] - shell && y >= shell && y < n[1] - shell && z >= shell && z < n[2] - shell;
    };
    if (c.model == B2R_MODEL_HEAT) {
        std::mt19937_64 rng(1);
        std::uniform_real_distribution<float> u(0.f, 1.f);
        std::vector<float> f(cells, 0.f);
        for (size_t e = 0; e < cells; ++e)
            if (inside(e)) f[e] = u(rng);
        return ok(b2r_upload(h, 0, f.data(), 0), h, "b2r_upload");
    }
    if (c.model == B2R_MODEL_GOL) {
        std::mt19937_64 rng(2);
        std::bernoulli_distribution b(0.3);
        std::vector<uint8_t> f(cells);
        for (auto& v : f) v = b(rng) ? 1 : 0;
        return ok(b2r_upload(h, 0, f.data(), 0), h, "b2r_upload");
    }
    if (c.model != B2R_MODEL_EQWP_STAG) return true;   // the reference model starts at rest
    std::mt19937_64 rng(3);
    std::uniform_real_distribution<double> uvp(2000.0, 4000.0), urho(2000.0, 2600.0);
    const int layers = 8;
    double vp[layers], rho[layers];
    for (int l = 0; l < layers; ++l) {
        vp[l] = uvp(rng);
        rho[l] = urho(rng);
    }
    std::vector<float> lam(cells), mu(cells), buoy(cells);
    for (size_t e = 0; e < cells; ++e) {
        const int y = (int)((e / n[0]) % n[1]);
        const int l = std::min(y * layers / n[1], layers - 1);
        const double m = rho[l] * vp[l] * vp[l] / 3.0;
        mu[e] = (float)m;
        lam[e] = (float)(rho[l] * vp[l] * vp[l] - 2.0 * m);
        buoy[e] = (float)(1.0 / rho[l]);
    }
    if (!ok(b2r_upload(h, B2R_F_LAMBDA, lam.data(), 0), h, "b2r_upload") ||
        !ok(b2r_upload(h, B2R_F_MU, mu.data(), 0), h, "b2r_upload") ||
        !ok(b2r_upload(h, B2R_F_BUOY, buoy.data(), 0), h, "b2r_upload"))
        return false;
    return true;
}

}  // namespace

int main(int argc, char** argv)
{
    Options o;
    if (!parse(argc, argv, o)) {
        usage();
        return 1;
    }
    std::printf("arguments received, where: B2R_R = %d, BLOCK_DIM_X = %d, BLOCK_DIM_Y = %d, BLOCK_DIM_Z = %d\n",
                o.R, o.nb[0], o.nb[1], o.nb[2]);
    if (o.env[0] % o.nb[0] || o.env[1] % o.nb[1] || o.env[2] % o.nb[2]) {   // b2r.cpp:154-158
        std::printf("GBL_ENV_(X,Y,Z) should be perfectly divisible by the given block size "
                    "BLOCK_DIM_(X,Y,Z) separately!\n");
        return 1;
    }
    b2r_config c;
    std::memset(&c, 0, sizeof c);
    if (o.model == "eqwp") c.model = B2R_MODEL_EQWP_REF;
    else if (o.model == "stag") c.model = B2R_MODEL_EQWP_STAG;
    else if (o.model == "heat") c.model = B2R_MODEL_HEAT;
    else if (o.model == "gol") c.model = B2R_MODEL_GOL;
    else {
        std::printf("unknown model %s\n", o.model.c_str());
        return 1;
    }
    for (int a = 0; a < 3; ++a) {
        c.env[a] = o.env[a];
        c.blocks[a] = o.nb[a];
    }
    c.R = o.R;
    c.D = o.D > 0 ? o.D : (c.model == B2R_MODEL_GOL ? 1 : 2);
    c.boundary = c.model == B2R_MODEL_GOL ? B2R_BC_PERIODIC : B2R_BC_SHELL;
    c.alpha_dt = 0.1;
    c.dx = c.dy = c.dz = 1.0;
    c.h = 10.0;
    c.dt = 0.5 * c.h / (4000.0 * std::sqrt(3.0) * (9.0 / 8.0 + 1.0 / 24.0));
    for (int a = 0; a < 3; ++a) c.src[a] = c.env[a] / 2;
    const int D = c.D;
    if (o.log) {   // b2r.cpp:88-97
        char name[160];
        std::snprintf(name, sizeof name, "R-%d-D-%d-ENV-%dX%dX%d-BLOCK-%dX%dX%d-GPU.txt", o.R, D, o.env[0],
                      o.env[1], o.env[2], o.nb[0], o.nb[1], o.nb[2]);
        if (!std::freopen(name, "w", stdout)) return 1;
    }
    b2r_handle* h = nullptr;
    if (b2r_create(&c, &h) != B2R_OK) {
        std::printf("%s\n", b2r_last_error(h));
        return 1;
    }
    if (!initialise(h, c)) return 1;
    if (c.model == B2R_MODEL_EQWP_STAG) {   // Ricker, f0 = 10 Hz, explosive at the centre
        std::vector<float> amps((size_t)o.iters);
        const double f0 = 10.0, pi = 3.14159265358979323846;
        for (int n = 0; n < o.iters; ++n) {
            const double t = n * c.dt - 1.2 / f0, a = (pi * f0 * t) * (pi * f0 * t);
            amps[(size_t)n] = (float)(1e7 * c.dt * (1.0 - 2.0 * a) * std::exp(-a));
        }
        if (!ok(b2r_set_source(h, amps.data(), o.iters), h, "b2r_set_source")) return 1;
    }
    int nf = 1;
    if (c.model == B2R_MODEL_EQWP_REF) nf = 10;
    if (c.model == B2R_MODEL_EQWP_STAG) nf = 9;
    if (!ok(b2r_synchronize(h), h, "b2r_synchronize")) return 1;

    double sync_time = 0.0, device_time = 0.0;
    const auto t_all = std::chrono::steady_clock::now();
    for (int i = 0; i < o.iters; i += o.R) {   // b2r.cpp:179
        const int r = std::min(o.R, o.iters - i);
        auto ts = std::chrono::steady_clock::now();
        for (int f = 0; f < nf; ++f) {   // b2r.cpp:197-206
            const b2r_status st = o.direct ? b2r_boundary_updating_direct(h, i, f) : b2r_boundary_updating(h, i, f);
            if (!ok(st, h, "boundary_updating")) return 1;
        }
        if (!ok(b2r_synchronize(h), h, "b2r_synchronize")) return 1;
        sync_time += seconds_since(ts);
        if (c.model == B2R_MODEL_EQWP_REF) {   // b2r.cpp:215
            double secs = 0.0;
            if (!ok(b2r_eqwp_gpu_main(h, i, r, &secs), h, "b2r_eqwp_gpu_main")) return 1;
            device_time += secs;
        } else {
            auto tc = std::chrono::steady_clock::now();
            if (!ok(b2r_step(h, r), h, "b2r_step") || !ok(b2r_synchronize(h), h, "b2r_synchronize")) return 1;
            device_time += seconds_since(tc);
        }
    }
    const double elapsed = seconds_since(t_all);
    std::printf("Execution/Model Parameters: B2R_R = %d, B2R_D: %d, ENV: %d X %d X %d, BLOCK_DIM_X = %d, "
                "BLOCK_DIM_Y = %d, BLOCK_DIM_Z = %d, model: %s\n",
                o.R, D, o.env[0], o.env[1], o.env[2], o.nb[0], o.nb[1], o.nb[2], o.model.c_str());
    std::printf("%d Iterations with B2R_R=%d took: %g seconds\n", o.iters, o.R, elapsed);
    std::printf("h <-> d took: %g seconds\n", 0.0);
    std::printf("device computation took: %g seconds\n", device_time);
    std::printf("halo synchronization took: %g seconds\n", sync_time);
    std::printf("GLUPS: %g\n", (double)o.env[0] * o.env[1] * o.env[2] * o.iters / std::max(elapsed, 1e-9) / 1e9);
    if (!o.snapshot.empty() && c.model == B2R_MODEL_GOL) {
        std::printf("block data files hold float cells: no snapshot of Game-of-Life bytes\n");
    } else if (!o.snapshot.empty()) {   // eqwp.cu:700-707: the displacement (or field 0) of every block
        const int field = c.model == B2R_MODEL_EQWP_REF ? B2R_F_DISP : 0;
        for (int b = 0; b < o.nb[0] * o.nb[1] * o.nb[2]; ++b) {
            char path[1024];
            if (!ok(b2r_write_block_data(h, field, b, o.iters, o.snapshot.c_str(), 0, path, sizeof path), h,
                    "b2r_write_block_data"))
                return 1;
            std::printf("wrote %s\n", path);
        }
    }
    b2r_destroy(h);
    return 0;
}
