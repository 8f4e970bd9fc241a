"""Build libb2r.so in-tree for sm_103a (GB300).

Each translation unit of csrc/ is compiled by nvcc in parallel and linked
into b2r_gb300/libb2r.so; host/b2r_main.cpp (the simulation main over the C
ABI) is compiled by the host C++ compiler into b2r_gb300/b2r_main.  No
torch, no cmake.  Used by
__graft_entry__.build() on every machine (nvcc compiles without a GPU).
"""
import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libb2r.so")
MAIN_SRC = os.path.join(HERE, "host", "b2r_main.cpp")
MAIN = os.path.join(HERE, "b2r_main")
CXX = os.environ.get("CXX", "g++")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", os.path.join(HERE, "..", "include")] + os.environ.get("B2R_NVCC_FLAGS", "").split()


def _deps_newer(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if _deps_newer(obj, src):
        cmd = [NVCC, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose_ptxas=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    if force:
        for o in glob.glob(os.path.join(OBJ, "*.o")):
            os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-ldl", "-lpthread", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_main(force)
    return LIB


def build_main(force=False):
    """The C++ host program (b2r.cpp's main over the C ABI), linked to
    libb2r.so beside it."""
    if not force and os.path.exists(MAIN) and os.path.getmtime(MAIN) > max(
            os.path.getmtime(MAIN_SRC), os.path.getmtime(LIB)):
        return MAIN
    cmd = [CXX, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(HERE, "..", "include"), MAIN_SRC,
           "-L", HERE, "-lb2r", "-Wl,-rpath,$ORIGIN", "-o", MAIN]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"b2r_main build failed:\n{r.stdout}\n{r.stderr}")
    return MAIN


if __name__ == "__main__":
    import sys
    print(build(verbose_ptxas="-v" in sys.argv, force="-f" in sys.argv))
