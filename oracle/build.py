"""Build recipe for the oracle (test infrastructure only).

* ``liborc.so``  -- the CPU restatement in b2r_oracle.c (always built).
* ``_ref/eqwp_ref.cubin``, ``_ref/gol_ref.cubin``, ``_ref/heat_ref.cubin``,
  ``_ref/heat_ref_d{2,3,4}.cubin`` -- the reference's own eqwp.cu, gol-3D.cu
  and heat-3D.cu kernels, device code only, heat-3D.cu once per stencil
  radius B2R_D (its shared tiles are sized by it, heat-3D.cu:175,252);
  oracle/refgpu.py runs them on the GPU as a second oracle.
* ``_ref/libheat_ref.so`` -- the reference's own heat-3D.cpp compiled from
  its source tree, with a two-line config shim for its
  ``#include "../b2r_config.h"`` (heat-3D.cpp:16) and
  ``CPU_N_THRD`` (used at heat-3D.cpp:51,66,87,111, defined nowhere in the
  reference) set to the OpenMP runtime thread count.  Built only where the
  reference source tree is present; the output stays in ``oracle/_ref/``.

Both are compiled with ``-ffp-contract=off`` so float/double expressions are
evaluated exactly as written on x86-64 and aarch64.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference's source tree: B2R_REFERENCE_SRC, else a "reference" folder
# beside this repository
REF_SRC = os.environ.get("B2R_REFERENCE_SRC",
                         os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
CFLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "b2r_oracle.c")
    out = os.path.join(HERE, "liborc.so")
    hdr = os.path.join(HERE, "b2r_oracle.h")
    if force or not _newer(out, [src, hdr]):
        subprocess.check_call(["gcc", "-std=gnu11", *CFLAGS, "-o", out, src, "-lm"])
    return out


def build_ref(force=False):
    """Compile the reference's heat-3D.cpp; returns the .so path or None."""
    ref = os.path.join(REF_SRC, "heat-3D.cpp")
    if not os.path.exists(ref):
        return None
    refdir = os.path.join(HERE, "_ref")
    inc = os.path.join(refdir, "inc")
    sub = os.path.join(inc, "sub")
    os.makedirs(sub, exist_ok=True)
    with open(os.path.join(inc, "b2r_config.h"), "w") as f:
        f.write("#pragma once\n#define B2R_D 1\n")
    wrap = os.path.join(HERE, "ref_shim", "heat_ref_wrap.cpp")
    out = os.path.join(refdir, "libheat_ref.so")
    if force or not _newer(out, [ref, wrap]):
        subprocess.check_call(["g++", *CFLAGS, "-I", sub, "-include", "omp.h",
                               "-DCPU_N_THRD=omp_get_max_threads()",
                               "-o", out, ref, wrap])
    return out


def build_ref_cubin(force=False):
    """Compile the reference's eqwp.cu, gol-3D.cu and heat-3D.cu, unmodified,
    into cubins of their device code for sm_103a (nvcc defaults otherwise,
    as the reference is built; the host code of the last two calls
    cudaThreadSynchronize, which CUDA 13 no longer declares, so that name is
    defined to its successor on the command line; heat-3D.cu gets the
    delta-1 config shim that its CPU build uses).  Returns the eqwp cubin's path, or None
    where the source tree is absent.  A cubin is GPU code, so the prebuilt
    files serve the machine with the GPU."""
    ref = os.path.join(REF_SRC, "eqwp.cu")
    if not os.path.exists(ref):
        return None
    refdir = os.path.join(HERE, "_ref")
    os.makedirs(refdir, exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    outs = []
    sync = "-DcudaThreadSynchronize=cudaDeviceSynchronize"
    jobs = [("eqwp.cu", "eqwp_ref.cubin", []), ("gol-3D.cu", "gol_ref.cubin", [sync])]
    for D in (1, 2, 3, 4):
        # heat-3D.cu includes "../b2r_config.h": one shim folder per radius
        inc = os.path.join(refdir, "incg" if D == 1 else f"incg{D}")
        sub = os.path.join(inc, "sub")
        os.makedirs(sub, exist_ok=True)
        shim = os.path.join(inc, "b2r_config.h")
        text = f"#pragma once\n#define B2R_D {D}\ntypedef float CELL_DT;\n"
        if not os.path.exists(shim) or open(shim).read() != text:
            with open(shim, "w") as f:
                f.write(text)
        name = "heat_ref.cubin" if D == 1 else f"heat_ref_d{D}.cubin"
        jobs.append(("heat-3D.cu", name, [sync, "-I", sub]))
    for src, name, extra in jobs:
        path = os.path.join(REF_SRC, src)
        out = os.path.join(refdir, name)
        if force or not _newer(out, [path, os.path.join(REF_SRC, "b2r_config.h")]):
            subprocess.check_call([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                                   *extra, "-o", out, path])
        outs.append(out)
    return outs[0]


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
    print(build_ref_cubin(force=True))
