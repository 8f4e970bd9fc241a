"""GPU Game of Life: bit-exact against the oracle (integer work)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bernoulli(env, p, seed):
    rng = np.random.default_rng(seed)
    return (rng.random(env[::-1]) < p).astype(np.uint8)


@pytest.mark.parametrize("env,blocks,R", [((64, 64, 64), (2, 2, 2), 4), ((64, 48, 40), (1, 1, 1), 1),
                                          ((70, 36, 50), (2, 3, 1), 2), ((33, 17, 9), (1, 1, 1), 3)])
@pytest.mark.parametrize("tblock", [1, 2, 4])
def test_gol_periodic_bit_exact_every_period(b2r, orc, env, blocks, R, tblock):
    dom = bernoulli(env, 0.3, 2)
    ref = dom.copy()
    with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, D=1, boundary=b2r.BC_PERIODIC) as d:
        d.set_tuning(tblock=tblock)
        d.upload(dom)
        for period in range(3):
            d.step(R)
            orc.gol_run_periodic(ref, R)
            got = d.download()
            assert np.array_equal(got, ref), f"period {period}"
        d.synchronize()


def test_gol_invariant_in_R_and_blocks(b2r):
    env = (48, 48, 48)
    dom = bernoulli(env, 0.3, 4)
    outs = []
    for blocks, R in [((1, 1, 1), 1), ((2, 2, 2), 1), ((2, 2, 2), 2), ((2, 2, 2), 4), ((1, 2, 3), 4)]:
        with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, D=1, boundary=b2r.BC_PERIODIC) as d:
            d.upload(dom)
            d.step(12)
            outs.append(d.download())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_gol_fixed_shell(b2r, orc):
    env = (40, 30, 20)
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.uint8)
    dom[1:-1, 1:-1, 1:-1] = bernoulli(env, 0.35, 6)
    dom[0] = 1                                   # a live shell face stays live
    with b2r.Domain(b2r.MODEL_GOL, env, blocks=(2, 1, 2), R=2, D=1) as d:
        d.upload(dom)
        d.step(6)
        got = d.download()
    a, b = dom.copy(), dom.copy()
    for _ in range(6):
        orc.gol_substep(a, b, 0, 1, 63)
        a, b = b, a
    assert np.array_equal(got, a)


@pytest.mark.parametrize("R", [1, 2, 4])
def test_gol_3D_gpu_main_block_entry(b2r, orc, R):
    rng = np.random.default_rng(R)
    blk = (rng.random((21, 37, 45)) < 0.3).astype(np.uint8)
    got = blk.copy()
    b2r.gol_3D_gpu_main(got, R)
    a, b = blk.copy(), blk.copy()
    for i in range(R):
        orc.gol_substep(a, b, i, R, 0)
        a, b = b, a
    # the valid interior after R generations is bit-exact
    s = (slice(R, -R),) * 3
    assert np.array_equal(got[s], a[s])


@pytest.mark.parametrize("env,blocks,R,steps", [((300, 40, 30), (1, 1, 1), 1, 9), ((260, 70, 33), (2, 1, 1), 3, 7)])
def test_gol_multi_generation_pass(b2r, orc, env, blocks, R, steps):
    """Several generations per pass (wide rows split into x tiles, ragged
    tails) against one generation per pass and the oracle."""
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.uint8)
    dom[1:-1, 1:-1, 1:-1] = bernoulli(env, 0.3, 9)
    outs = []
    for tb in (1, 4):
        with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, D=1) as d:
            d.set_tuning(tblock=tb)
            d.upload(dom)
            d.step(steps)
            outs.append(d.download())
    assert np.array_equal(outs[0], outs[1])
    a, b = dom.copy(), dom.copy()
    for _ in range(steps):
        orc.gol_substep(a, b, 0, 1, 63)
        a, b = b, a
    assert np.array_equal(outs[1], a)


@pytest.mark.parametrize("env,blocks,R,periodic", [((64, 64, 64), (2, 2, 2), 4, True), ((300, 40, 30), (1, 1, 1), 1, False),
                                                   ((33, 17, 9), (1, 1, 1), 2, True), ((520, 35, 20), (2, 1, 1), 3, False),
                                                   ((70, 36, 50), (2, 3, 1), 2, True)])
def test_gol_bit_sliced_equals_byte_kernel(b2r, orc, env, blocks, R, periodic):
    """Bit-sliced cells (default) against four byte cells per word, on rows of
    1 to 9 words per thread and tails that cut words."""
    bc = b2r.BC_PERIODIC if periodic else b2r.BC_SHELL
    if periodic:
        dom = bernoulli(env, 0.3, 21)
    else:
        dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.uint8)
        dom[1:-1, 1:-1, 1:-1] = bernoulli(env, 0.3, 21)
    outs = []
    for gb in (1, 0):
        with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, D=1, boundary=bc) as d:
            d.set_tuning(gol_bytes=gb)
            d.upload(dom)
            d.step(2 * R + 1)
            outs.append(d.download())
    assert np.array_equal(outs[0], outs[1])
    if periodic:
        ref = dom.copy()
        orc.gol_run_periodic(ref, 2 * R + 1)
        assert np.array_equal(outs[1], ref)


@pytest.mark.parametrize("env,blocks,R", [((64, 64, 64), (2, 2, 2), 4), ((100, 52, 40), (2, 1, 1), 3)])
def test_gol_multi_generation_passes_agree(b2r, orc, env, blocks, R):
    """Several generations per pass with bit-sliced and with byte cells,
    against one generation per pass and the oracle (periodic)."""
    dom = bernoulli(env, 0.3, 31)
    outs = []
    for gb, tb in ((0, 4), (1, 4), (0, 1)):
        with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, D=1, boundary=b2r.BC_PERIODIC) as d:
            d.set_tuning(gol_bytes=gb, tblock=tb)
            d.upload(dom)
            d.step(2 * R)
            outs.append(d.download())
    ref = dom.copy()
    orc.gol_run_periodic(ref, 2 * R)
    for o in outs:
        assert np.array_equal(o, ref)


@pytest.mark.parametrize("env,blocks,R,periodic", [((64, 64, 64), (2, 2, 2), 4, True),
                                                   ((96, 32, 64), (3, 1, 2), 3, True),
                                                   ((64, 64, 32), (2, 2, 1), 4, False),
                                                   ((32, 32, 32), (1, 1, 1), 4, True),
                                                   ((64, 40, 48), (2, 1, 3), 2, True),
                                                   ((80, 36, 20), (2, 3, 1), 2, True)])
@pytest.mark.parametrize("graphs", [False, True])
def test_gol_halo_push_matches_gather(b2r, orc, env, blocks, R, periodic, graphs):
    """A pass that ends a period stores the next period's halos itself (no
    gather): the same bits as the gather, on tori and on shelled domains,
    direct and graph-replayed, and against the oracle."""
    import torch
    if periodic:
        dom = bernoulli(env, 0.3, 11)
        kw = dict(boundary=b2r.BC_PERIODIC)
    else:
        dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.uint8)
        dom[1:-1, 1:-1, 1:-1] = bernoulli(env, 0.3, 11)
        dom[:, 0] = 1
        kw = {}
    nsteps = 9 * R + 1
    outs = []
    for push in (1, 0):
        s = torch.cuda.Stream()
        with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, D=1, stream=s, **kw) as d:
            d.set_graphs(graphs)
            d.set_tuning(gol_push=push)
            assert d.get_tuning()["gol_push"] == push
            d.upload(dom)
            d.step(1)
            d.step(nsteps - 1)
            outs.append(d.download())
            d.synchronize()
    assert np.array_equal(outs[0], outs[1])
    ref = dom.copy()
    if periodic:
        orc.gol_run_periodic(ref, nsteps)
    else:
        a, b = dom.copy(), dom.copy()
        for _ in range(nsteps):
            orc.gol_substep(a, b, 0, 1, 63)
            a, b = b, a
        ref = a
    assert np.array_equal(outs[0], ref)


@pytest.mark.parametrize("env,blocks,R", [((80, 36, 20), (2, 3, 1), 2), ((64, 64, 64), (2, 2, 2), 4)])
def test_gol_halo_push_repeatable(b2r, orc, env, blocks, R):
    """Repeated runs with the halo fill requested give the oracle's bits
    every time (rows of 40 cells fall back to the gather: a word across the
    interior edge is stored whole and would race with the fill)."""
    import torch
    dom = bernoulli(env, 0.3, 12)
    nsteps = 6 * R
    ref = dom.copy()
    orc.gol_run_periodic(ref, nsteps)
    for _ in range(4):
        s = torch.cuda.Stream()
        with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, D=1, boundary=b2r.BC_PERIODIC, stream=s) as d:
            d.set_tuning(gol_push=1)
            d.upload(dom)
            d.step(nsteps)
            out = d.download()
            d.synchronize()
        assert np.array_equal(out, ref)


@pytest.mark.parametrize("env", [(30, 30, 40), (9, 7, 5), (65, 33, 17), (128, 20, 12)])
@pytest.mark.parametrize("R,tblock", [(1, 2), (2, 4), (5, 2), (3, 1)])
def test_gol_single_fixed_shell_block(b2r, orc, env, R, tblock):
    """One block with a one-cell fixed shell (no exchange, so a pass may take
    more generations than the shell is deep): every R and pass length
    against the oracle."""
    if R > min(env) // 2:
        pytest.skip("R*D <= min(B)/2 (b2r.cpp:54)")
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.uint8)
    dom[1:-1, 1:-1, 1:-1] = bernoulli(env, 0.35, 14)
    dom[:, :, 0] = 1
    nsteps = 11
    with b2r.Domain(b2r.MODEL_GOL, env, D=1, R=R) as d:
        d.set_tuning(tblock=tblock)
        d.upload(dom)
        d.step(nsteps)
        got = d.download()
        d.synchronize()
    a, b = dom.copy(), dom.copy()
    for _ in range(nsteps):
        orc.gol_substep(a, b, 0, 1, 63)
        a, b = b, a
    assert np.array_equal(got, a)


@pytest.mark.parametrize("env,blocks,R,periodic", [((64, 64, 64), (2, 2, 2), 4, True), ((70, 36, 50), (2, 3, 1), 2, True),
                                                   ((300, 40, 30), (1, 1, 1), 4, False), ((96, 130, 40), (1, 2, 1), 3, False)])
def test_gol_band_heights_bit_identical(b2r, orc, env, blocks, R, periodic):
    """The several-generation pass with bands of 7, 48 and a whole block of
    rows against the default 32 (and the oracle on the torus)."""
    bc = b2r.BC_PERIODIC if periodic else b2r.BC_SHELL
    if periodic:
        dom = bernoulli(env, 0.3, 23)
    else:
        dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.uint8)
        dom[1:-1, 1:-1, 1:-1] = bernoulli(env, 0.3, 23)
    outs = []
    for rows in (0, 7, 48, 1 << 20):
        with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, D=1, boundary=bc) as d:
            d.set_tuning(tblock=4, gol_bytes=0, gol_push=0, gol_rows=rows)
            assert d.get_tuning()["gol_rows"] == rows
            d.upload(dom)
            d.step(2 * R + 1)
            outs.append(d.download())
    for o in outs[1:]:
        assert np.array_equal(outs[0], o)
    if periodic:
        ref = dom.copy()
        orc.gol_run_periodic(ref, 2 * R + 1)
        assert np.array_equal(outs[0], ref)
