"""The heat block entry that allocates nothing (b2r_heat_3D_gpu_main_noalloc).

It serves callers that cannot allocate device memory themselves -- code
running under a framework that owns all device memory through its own pool
and forbids raw cudaMalloc/cudaFree -- by keeping its ping-pong blocks in a
fixed array inside the library.  Checked here through the C ABI against the
allocating entry b2r_heat_3D_gpu_main and against the oracle's ping-pong of
the same sub-steps, on the same inputs, for calls in a row (each call reuses
the array the previous one left behind), within the relative-L2 tolerance of
the other heat tests.  Every stencil order is covered (orders 2 and 4 need
more than 48 KB of shared memory per CTA), and so is a block at the size
limit, whose last planes sit right against the status word.  This file is
collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5
CAP_CELLS = 4 << 20          # padded cells per ping-pong buffer


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


def padded_cells(nx, ny, nz, H):
    """The library's padded layout of one float block (rows of a multiple of
    32 cells, >= 4 cells of pad before x = 0 and >= 8 after the row)."""
    xoff = (H + 4 + 31) // 32 * 32 - H
    P = (xoff + nx + 8 + 31) // 32 * 32
    return P * ny * nz


def oracle_block(orc, blk, R, D, ef, coef):
    """heat-3D.cu:583 restated: R shrinking sub-steps ping-ponged on the
    block, planes [R*D, Ngz-R*D) of the result, the rest of the input."""
    edge = 0
    if ef:
        for a in range(3):
            edge |= (1 << (2 * a)) if ef[a] < 0 else 0
            edge |= (1 << (2 * a + 1)) if ef[a] > 0 else 0
    H = R * D
    a, b = blk.copy(), blk.copy()
    for i in range(R):
        orc.heat_substep(a, b, D, i, H, edge, *coef)
        a, b = b, a
    ref = blk.copy()
    ref[H:-H] = a[H:-H]
    return ref


CALLS = [
    dict(shape=(30, 26, 41), R=3, D=1, ef=None, coef=(0.01, 1.0, 1.0, 0.5), seed=1),
    dict(shape=(40, 35, 57), R=1, D=3, ef=(-1, 0, 1), coef=(0.02, 1.0, 1.2, 0.9), seed=2),
    dict(shape=(36, 33, 45), R=2, D=2, ef=(0, 1, -1), coef=(0.02, 1.0, 1.0, 1.0), seed=3),
    dict(shape=(44, 29, 70), R=1, D=4, ef=None, coef=(0.015, 1.1, 1.0, 1.0), seed=4),
    dict(shape=(41, 38, 33), R=2, D=4, ef=(1, -1, 0), coef=(0.01, 1.0, 1.0, 1.0), seed=5),
]


def test_noalloc_matches_allocating_entry_and_oracle(b2r, orc):
    """Five calls in a row, every stencil order: each matches the allocating
    entry and the oracle, and leaves its input as it was."""
    import torch
    fn = noalloc_fn(b2r)
    for k, c in enumerate(CALLS):
        rng = np.random.default_rng(c["seed"])
        blk = rng.random(c["shape"], dtype=np.float32)
        nz, ny, nx = c["shape"]
        ref = blk.copy()
        b2r.heat_3D_gpu_main(ref, c["R"], D=c["D"], edge_flag=c["ef"], alpha_dt=c["coef"][0],
                             dx=c["coef"][1], dy=c["coef"][2], dz=c["coef"][3])
        orc_ref = oracle_block(orc, blk, c["R"], c["D"], c["ef"], c["coef"])
        d_in = torch.from_numpy(blk).cuda()
        d_out = torch.full_like(d_in, float("nan"))
        torch.cuda.synchronize()
        st = fn(C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()), c["R"], c["D"],
                ef_bytes(c["ef"]), nx, ny, nz, *c["coef"], C.c_void_p(0))
        assert st == 0, f"call {k}: status {st}"
        got = d_out.cpu().numpy()
        assert np.isfinite(got).all(), f"call {k}: unwritten cells"
        assert rel_l2(got, ref) <= TOL, f"call {k}: against the allocating entry"
        assert rel_l2(got, orc_ref) <= TOL, f"call {k}: against the oracle"
        H = c["R"] * c["D"]
        assert np.array_equal(got[:H], blk[:H]) and np.array_equal(got[-H:], blk[-H:])
        assert np.array_equal(d_in.cpu().numpy(), blk)


def test_noalloc_at_the_size_limit(b2r, orc):
    """The largest cube the array holds at R*D = 1 (147^3) runs, twice in a
    row, and the next size up is refused; a small call after them still
    returns status 0 with the right result."""
    import torch
    fn = noalloc_fn(b2r)
    n = 147
    assert padded_cells(n, n, n, 1) <= CAP_CELLS < padded_cells(n + 1, n + 1, n + 1, 1)
    coef = (0.01, 1.0, 1.0, 0.5)
    rng = np.random.default_rng(7)
    blk = rng.random((n, n, n), dtype=np.float32)
    ref = blk.copy()
    b2r.heat_3D_gpu_main(ref, 1, D=1, alpha_dt=coef[0], dx=coef[1], dy=coef[2], dz=coef[3])
    d_in = torch.from_numpy(blk).cuda()
    for k in range(2):
        d_out = torch.full_like(d_in, float("nan"))
        torch.cuda.synchronize()
        assert fn(C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()), 1, 1, None, n, n, n,
                  *coef, C.c_void_p(0)) == 0, f"call {k}"
        got = d_out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_l2(got, ref) <= TOL
        # the last planes (next to the status word) are the result's
        assert rel_l2(got[-8:-1], ref[-8:-1]) <= TOL
    big = torch.zeros((n + 1, n + 1, n + 1), dtype=torch.float32, device="cuda")
    assert fn(C.c_void_p(big.data_ptr()), C.c_void_p(big.data_ptr()), 1, 1, None, n + 1, n + 1, n + 1,
              *coef, C.c_void_p(0)) == 1
    small = rng.random((20, 24, 28), dtype=np.float32)
    d = torch.from_numpy(small).cuda()
    assert fn(C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), 2, 1, None, 28, 24, 20,
              *coef, C.c_void_p(0)) == 0
    assert rel_l2(d.cpu().numpy(), oracle_block(orc, small, 2, 1, None, coef)) <= TOL


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
