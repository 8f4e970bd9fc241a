// heat_cpu.cu -- the heat model on the host cores, and the block split
// between the host cores and the GPU.
//
// b2r_heat_3D_cpu_main replaces heat_3D_cpu_main (heat-3D.hpp:12,
// heat-3D.cpp:136-184): R shrinking sub-steps of the order-D stencil on one
// padded host block, ping-ponged between two copies of it, then planes
// [R*D, Ngz-R*D) of the result written back -- the contract of
// b2r_heat_3D_gpu_main.  Every cell is computed with the GPU sweep's float
// operations in the GPU sweep's order (a0*u, then per ring k the x, y and z
// pair sums folded in by fused multiply-adds), so the host result is
// bit-identical to the GPU's.  It is an entry of its own: no GPU entry of
// the library ever falls back to it.
//
// b2r_heat_3D_hybrid_main is the CPU+GPU split that heat-3D.cpp:47,170 point
// at: the block is cut along z; the host cores take the last cpu_planes
// result planes and the GPU the rest.  Each side gets its part plus R*D
// planes of the other side's (B2R's deep halo along the cut), so both run
// their R sub-steps with no exchange between them, at the same time; the
// cut face of each part shrinks as an interior face does.  The result is
// bit-identical to b2r_heat_3D_gpu_main's.
#include <chrono>
#include <cmath>
#include <thread>
#include <vector>

#include "api_internal.h"

namespace b2r {
namespace {

// One sub-step (shrink D*(step_i+1)) of a dense block (x fastest, rows of
// n[0] cells) from `in` into `out` over z planes [z0, z1) of the window.
void heat_cpu_rows(const float* in, float* out, const int n[3], int D, const HeatCoef& c, const int lo[3],
                   const int hi[3], int z0, int z1)
{
    const long long sx = 1, sy = n[0], sz = (long long)n[0] * n[1];
    for (int z = z0; z < z1; ++z)
        for (int y = lo[1]; y <= hi[1]; ++y) {
            const long long row = z * sz + y * sy;
            for (int x = lo[0]; x <= hi[0]; ++x) {
                const long long i = row + x * sx;
                float r = c.a0 * in[i];
                for (int k = 1; k <= D; ++k) {
                    r = std::fmaf(c.ax[k - 1], in[i - k * sx] + in[i + k * sx], r);
                    r = std::fmaf(c.ay[k - 1], in[i - k * sy] + in[i + k * sy], r);
                    r = std::fmaf(c.az[k - 1], in[i - k * sz] + in[i + k * sz], r);
                }
                out[i] = r;
            }
        }
}

// R sub-steps on a host block with face bits `edge` (BlockLayout::fixed_edge),
// on nthreads threads; h_out gets planes [R*D, Ngz-R*D) of the result.
void heat_cpu_block(const float* h_in, float* h_out, int R, int D, int edge, const int n[3], const HeatCoef& c,
                    int nthreads)
{
    const size_t cells = (size_t)n[0] * n[1] * n[2];
    std::vector<float> buf[2] = {std::vector<float>(h_in, h_in + cells), std::vector<float>(h_in, h_in + cells)};
    // the window of each sub-step: the shrinking region of heat-3D.cu:191 with
    // the fixed shell of heat-3D.cu:81-114 (stage_region, as the GPU uses it)
    BlockLayout L{};
    const int H = R * D;
    for (int a = 0; a < 3; ++a) L.n[a] = n[a];
    L.H = H;
    int cur = 0;
    for (int i = 0; i < R; ++i) {
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) stage_region(L, edge, a, D * (i + 1), lo[a], hi[a]);
        const float* in = buf[cur].data();
        float* out = buf[1 - cur].data();
        const int nz = hi[2] - lo[2] + 1;
        const int nt = std::max(1, std::min(nthreads, nz));
        if (nt == 1) {
            heat_cpu_rows(in, out, n, D, c, lo, hi, lo[2], hi[2] + 1);
        } else {
            std::vector<std::thread> th;
            for (int t = 0; t < nt; ++t) {
                const int z0 = lo[2] + (int)((long long)nz * t / nt);
                const int z1 = lo[2] + (int)((long long)nz * (t + 1) / nt);
                th.emplace_back(heat_cpu_rows, in, out, n, D, std::cref(c), lo, hi, z0, z1);
            }
            for (auto& x : th) x.join();
        }
        cur = 1 - cur;
    }
    const size_t plane = (size_t)n[0] * n[1];
    std::copy(buf[cur].begin() + (size_t)H * plane, buf[cur].begin() + (size_t)(n[2] - H) * plane,
              h_out + (size_t)H * plane);
}

int host_threads(int nthreads)
{
    if (nthreads > 0) return nthreads;
    const unsigned hc = std::thread::hardware_concurrency();
    return hc > 0 ? (int)hc : 1;
}

b2r_status check_block(const float* h_in, int R, int D, int Ngx, int Ngy, int Ngz)
{
    if (!h_in) return b2r_api::fail(nullptr, B2R_ERR_ARG, "null h_in");
    if (D < 1 || D > 4) return b2r_api::fail(nullptr, B2R_ERR_ARG, "unsupported delta %d", D);
    if (R < 1) return b2r_api::fail(nullptr, B2R_ERR_ARG, "R must be >= 1");
    const int n[3] = {Ngx, Ngy, Ngz};
    for (int a = 0; a < 3; ++a)
        if (n[a] - 2 * R * D < 1) return b2r_api::fail(nullptr, B2R_ERR_ARG, "block too small for R*D = %d", R * D);
    return B2R_OK;
}

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace
}  // namespace b2r

using namespace b2r;

extern "C" b2r_status b2r_heat_3D_cpu_main(float* h_in, int R, int D, const char* edge_flag, int Ngx, int Ngy,
                                          int Ngz, double alpha_dt, double dx, double dy, double dz,
                                          int nthreads, double* cpu_seconds)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (b2r_status s = check_block(h_in, R, D, Ngx, Ngy, Ngz)) return s;
    const int n[3] = {Ngx, Ngy, Ngz};
    heat_cpu_block(h_in, h_in, R, D, b2r_api::edge_bits_of_flags(edge_flag), n,
                   heat_coef(D, alpha_dt, dx, dy, dz), host_threads(nthreads));
    if (cpu_seconds) *cpu_seconds = seconds_since(t0);   // wall clock, as heat-3D.cpp:141,181
    return B2R_OK;
}

extern "C" b2r_status b2r_heat_3D_hybrid_main(float* h_in, int R, int D, const char* edge_flag, int Ngx, int Ngy,
                                             int Ngz, double alpha_dt, double dx, double dy, double dz,
                                             int cpu_planes, int nthreads, void* cuda_stream, double* seconds)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (b2r_status s = check_block(h_in, R, D, Ngx, Ngy, Ngz)) return s;
    const int H = R * D;
    const int inner = Ngz - 2 * H;                  // result planes
    if (cpu_planes < 0) return b2r_api::fail(nullptr, B2R_ERR_ARG, "cpu_planes must be >= 0");
    if (cpu_planes > inner) cpu_planes = inner;
    const int edge = b2r_api::edge_bits_of_flags(edge_flag);
    const HeatCoef hc = heat_coef(D, alpha_dt, dx, dy, dz);
    if (cpu_planes == 0) {
        b2r_api::HeatBlockRun run;
        b2r_status s = run.begin(h_in, R, D, edge, Ngx, Ngy, Ngz, alpha_dt, dx, dy, dz,
                                 static_cast<cudaStream_t>(cuda_stream));
        if (s == B2R_OK) s = run.end(h_in, nullptr);
        if (seconds) *seconds = seconds_since(t0);
        return s;
    }
    // A part's deep halo must not cross a fixed face of the block: the fixed
    // shell is never updated, while a part would update it as the interior
    // side of its cut.  So with the high z face fixed the host takes no
    // fewer than H planes, and with the low z face fixed the GPU part keeps
    // no fewer than H result planes (else the host takes the whole block).
    if ((edge >> 5) & 1) cpu_planes = std::max(cpu_planes, H);
    if (((edge >> 4) & 1) && inner - cpu_planes < H) cpu_planes = inner;
    if (cpu_planes > inner) cpu_planes = inner;
    const int cut = Ngz - H - cpu_planes;           // first plane of the host's result
    const size_t plane = (size_t)Ngx * Ngy;
    // the host part, planes [cut-H, Ngz): copied out before the GPU's result
    // lands in h_in; its low z face is the cut (interior), its high face the
    // block's own
    const int nc[3] = {Ngx, Ngy, Ngz - cut + H};
    std::vector<float> host_part(h_in + (size_t)(cut - H) * plane, h_in + (size_t)Ngz * plane);
    const int cpu_edge = cut > H ? edge & ~(1 << 4) : edge;   // the whole block on the host: its own faces
    b2r_api::HeatBlockRun run;
    if (cut > H) {
        // the GPU part, planes [0, cut+H): its high z face is the cut
        const int gpu_edge = edge & ~(1 << 5);
        b2r_status s = run.begin(h_in, R, D, gpu_edge, Ngx, Ngy, cut + H, alpha_dt, dx, dy, dz,
                                 static_cast<cudaStream_t>(cuda_stream));
        if (s != B2R_OK) return s;
    }
    // host cores while the GPU's sub-steps run
    heat_cpu_block(host_part.data(), host_part.data(), R, D, cpu_edge, nc, hc, host_threads(nthreads));
    if (cut > H) {
        b2r_status s = run.end(h_in, nullptr);
        if (s != B2R_OK) return s;
    }
    std::copy(host_part.begin() + (size_t)H * plane, host_part.begin() + (size_t)(nc[2] - H) * plane,
              h_in + (size_t)cut * plane);
    if (seconds) *seconds = seconds_since(t0);
    return B2R_OK;
}
