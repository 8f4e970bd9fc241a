"""The heat model on the host cores (b2r_heat_3D_cpu_main, heat-3D.cpp:136)
and the block split between the host cores and the GPU
(b2r_heat_3D_hybrid_main, heat-3D.cpp:47,170).

CPU: the host entry against the oracle's ping-pong of the same sub-steps
(relative L2 <= 1e-5; the oracle weights in double as the reference does),
every stencil order, edge flags, R up to 3, and its argument checks.
GPU: the host entry and every split of the hybrid entry are bit-identical to
b2r_heat_3D_gpu_main (the host computes each cell with the GPU sweep's float
operations in the same order)."""
import numpy as np
import pytest

TOL = 1e-5
CASES = [((30, 26, 41), 1, 1, None), ((30, 26, 41), 3, 1, (-1, 0, 1)), ((28, 24, 33), 2, 2, (1, -1, 0)),
         ((27, 30, 25), 1, 3, (0, 1, -1)), ((34, 29, 31), 2, 4, None)]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_block(orc, blk, R, D, ef, coef):
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


@pytest.mark.parametrize("shape,R,D,ef", CASES)
def test_cpu_entry_matches_oracle(b2r, orc, shape, R, D, ef):
    coef = (0.02, 1.0, 1.1, 0.9)
    blk = np.random.default_rng(R * 10 + D).random(shape, dtype=np.float32)
    got = blk.copy()
    b2r.heat_3D_cpu_main(got, R, D=D, edge_flag=ef, alpha_dt=coef[0], dx=coef[1], dy=coef[2], dz=coef[3],
                         nthreads=3)
    ref = oracle_block(orc, blk, R, D, ef, coef)
    assert rel_l2(got, ref) <= TOL
    H = R * D
    assert np.array_equal(got[:H], blk[:H]) and np.array_equal(got[-H:], blk[-H:])
    # the thread count changes no bits
    one = blk.copy()
    b2r.heat_3D_cpu_main(one, R, D=D, edge_flag=ef, alpha_dt=coef[0], dx=coef[1], dy=coef[2], dz=coef[3],
                         nthreads=1)
    assert np.array_equal(one, got)


def test_cpu_entry_rejects_bad_args(b2r):
    a = np.zeros((6, 6, 6), np.float32)
    for kw in (dict(R=3, D=1), dict(R=1, D=5), dict(R=0, D=1)):
        with pytest.raises(b2r.B2RError) as ei:
            b2r.heat_3D_cpu_main(a, kw["R"], D=kw["D"])
        assert ei.value.status == 1
    with pytest.raises(ValueError):
        b2r.heat_3D_cpu_main(np.zeros((6, 6, 6), np.float64), 1)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,R,D,ef", CASES + [((40, 50, 70), 2, 1, (-1, 0, 1))])
def test_cpu_entry_bit_identical_to_gpu_entry(b2r, shape, R, D, ef):
    coef = (0.02, 1.0, 1.1, 0.9)
    blk = np.random.default_rng(R * 10 + D + 1).random(shape, dtype=np.float32)
    g = blk.copy()
    b2r.heat_3D_gpu_main(g, R, D=D, edge_flag=ef, alpha_dt=coef[0], dx=coef[1], dy=coef[2], dz=coef[3])
    c = blk.copy()
    b2r.heat_3D_cpu_main(c, R, D=D, edge_flag=ef, alpha_dt=coef[0], dx=coef[1], dy=coef[2], dz=coef[3])
    assert np.array_equal(c, g)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,R,D,ef", [((40, 50, 70), 3, 1, (-1, 0, 1)), ((44, 30, 36), 2, 2, (1, 1, 0)),
                                          ((37, 28, 33), 1, 4, (0, -1, 1)), ((36, 24, 20), 2, 1, None)])
def test_hybrid_split_bit_identical_to_gpu_entry(b2r, shape, R, D, ef):
    """Every cut: the GPU alone, one host plane, a few, half, and the host
    alone, with the cut face's deep halo on both sides."""
    coef = (0.02, 1.0, 1.0, 0.8)
    blk = np.random.default_rng(7 + R + D).random(shape, dtype=np.float32)
    g = blk.copy()
    b2r.heat_3D_gpu_main(g, R, D=D, edge_flag=ef, alpha_dt=coef[0], dx=coef[1], dy=coef[2], dz=coef[3])
    inner = shape[0] - 2 * R * D
    for cpu_planes in sorted({0, 1, 3, inner // 2, inner - 1, inner, inner + 5}):
        h = blk.copy()
        b2r.heat_3D_hybrid_main(h, R, cpu_planes, D=D, edge_flag=ef, alpha_dt=coef[0], dx=coef[1], dy=coef[2],
                                dz=coef[3], nthreads=4)
        assert np.array_equal(h, g), f"cpu_planes={cpu_planes}"


@pytest.mark.parametrize("shape,R,D,ef", [((40, 50, 70), 3, 1, (-1, 0, 1)), ((44, 30, 36), 2, 2, (1, 1, 0)),
                                          ((37, 28, 33), 1, 4, (0, -1, 1)), ((30, 20, 20), 2, 2, (0, 0, -1))])
def test_hybrid_split_model_on_the_host(b2r, shape, R, D, ef):
    """The split the hybrid entry makes, run with the host entry on both
    parts: the part below the cut with its high z face interior, the part
    above with its low z face interior, each with R*D planes of the other
    beyond the cut, and the rules that keep a deep halo off a fixed z face.
    Assembled, the parts equal the whole block bit for bit."""
    coef = (0.02, 1.0, 1.0, 0.8)
    blk = np.random.default_rng(7 + R + D).random(shape, dtype=np.float32)
    kw = dict(D=D, alpha_dt=coef[0], dx=coef[1], dy=coef[2], dz=coef[3])
    full = blk.copy()
    b2r.heat_3D_cpu_main(full, R, edge_flag=ef, **kw)
    H = R * D
    Ngz = shape[0]
    inner = Ngz - 2 * H
    for cp in sorted({1, 2, 3, 5, inner // 2, inner - 3, inner - 1}):
        if ef[2] == 1:
            cp = max(cp, H)
        if ef[2] == -1 and inner - cp < H:
            cp = inner
        if cp >= inner:
            continue
        cut = Ngz - H - cp
        lo = blk[:cut + H].copy()
        b2r.heat_3D_cpu_main(lo, R, edge_flag=(ef[0], ef[1], min(ef[2], 0)), **kw)
        hi = blk[cut - H:].copy()
        b2r.heat_3D_cpu_main(hi, R, edge_flag=(ef[0], ef[1], max(ef[2], 0)), **kw)
        out = blk.copy()
        out[H:cut] = lo[H:cut]
        out[cut:Ngz - H] = hi[H:-H]
        assert np.array_equal(out, full), f"cpu_planes={cp}"
