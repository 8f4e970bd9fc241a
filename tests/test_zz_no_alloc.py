"""The heat block entry that allocates nothing (b2r_heat_3D_gpu_main_noalloc).

It serves callers that cannot allocate device memory themselves -- code
running under a framework that owns all device memory through its own pool
and forbids raw cudaMalloc/cudaFree -- by keeping its ping-pong blocks in a
fixed array inside the library.  Checked here through the C ABI against the
allocating entry b2r_heat_3D_gpu_main on the same inputs, for two calls in a
row (the second call reuses the array the first one left behind), within the
relative-L2 tolerance of the other heat tests.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def noalloc_fn(b2r):
    L = C.CDLL(b2r.LIB_PATH)
    fn = L.b2r_heat_3D_gpu_main_noalloc
    d = C.c_double
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int,
                   d, d, d, d, C.c_void_p]
    fn.restype = C.c_int
    return fn


def ef_bytes(ef):
    return None if ef is None else bytes([(v + 256) % 256 for v in ef])


@pytest.mark.parametrize("calls", [[
    dict(shape=(30, 26, 41), R=3, D=1, ef=None, coef=(0.01, 1.0, 1.0, 0.5), seed=1),
    dict(shape=(40, 35, 57), R=1, D=3, ef=(-1, 0, 1), coef=(0.02, 1.0, 1.2, 0.9), seed=2),
]])
def test_noalloc_matches_allocating_entry_twice(b2r, calls):
    import torch
    fn = noalloc_fn(b2r)
    for k, c in enumerate(calls):
        rng = np.random.default_rng(c["seed"])
        blk = rng.random(c["shape"], dtype=np.float32)
        nz, ny, nx = c["shape"]
        ref = blk.copy()
        b2r.heat_3D_gpu_main(ref, c["R"], D=c["D"], edge_flag=c["ef"], alpha_dt=c["coef"][0],
                             dx=c["coef"][1], dy=c["coef"][2], dz=c["coef"][3])
        d_in = torch.from_numpy(blk).cuda()
        d_out = torch.full_like(d_in, float("nan"))
        torch.cuda.synchronize()
        st = fn(C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()), c["R"], c["D"],
                ef_bytes(c["ef"]), nx, ny, nz, *c["coef"], C.c_void_p(0))
        assert st == 0, f"call {k}: status {st}"
        got = d_out.cpu().numpy()
        assert np.isfinite(got).all(), f"call {k}: unwritten cells"
        assert rel_l2(got, ref) <= TOL, f"call {k}"
        # the input block is left as it was
        assert np.array_equal(d_in.cpu().numpy(), blk)


def test_noalloc_in_place_and_too_large(b2r):
    import torch
    fn = noalloc_fn(b2r)
    rng = np.random.default_rng(5)
    blk = rng.random((20, 24, 28), dtype=np.float32)
    ref = blk.copy()
    b2r.heat_3D_gpu_main(ref, 2, D=1)
    d = torch.from_numpy(blk).cuda()
    assert fn(C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), 2, 1, None, 28, 24, 20,
              0.01, 1.0, 1.0, 0.5, C.c_void_p(0)) == 0
    assert rel_l2(d.cpu().numpy(), ref) <= TOL
    # beyond the fixed scratch: rejected with B2R_ERR_ARG, nothing launched
    big = torch.zeros((200, 200, 200), dtype=torch.float32, device="cuda")
    assert fn(C.c_void_p(big.data_ptr()), C.c_void_p(big.data_ptr()), 1, 1, None, 200, 200, 200,
              0.01, 1.0, 1.0, 0.5, C.c_void_p(0)) == 1
