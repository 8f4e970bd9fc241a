// heat_ref_wrap.cpp -- C entry point onto the reference's own CPU heat code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles this file together
// with the unmodified heat-3D.cpp of the reference (heat-3D.cpp:136 defines
// heat_3D_cpu_main with C++ linkage) into oracle/_ref/libheat_ref.so.  The
// tests use it to pin the CPU restatement bit-for-bit; bench.py may time it
// as the reference CPU baseline.
#include <omp.h>

float heat_3D_cpu_main(float* h_in, int b2r_R, int b2r_D, int Ngx, int Ngy, int Ngz);

extern "C" float ref_heat_3D_cpu_main(float* h_in, int R, int D, int nx, int ny, int nz,
                                      int nthreads)
{
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return heat_3D_cpu_main(h_in, R, D, nx, ny, nz);
}
