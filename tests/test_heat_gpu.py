"""GPU parity of the heat kernels (delta1-4) against the oracle.

Tolerance: FP32 on the GPU vs the oracle's FP32-storage restatement of the
reference arithmetic: relative L2 <= 1e-5 (the bound for FP32 work).  The
oracle itself is bit-exact to the reference's heat_3D_cpu_main (see
test_oracle.py), so the chain GPU ~ oracle == reference holds.  Each case also
reports the error against the FP64 run of the same scheme.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def shell_domain(env, D, seed):
    dom = np.zeros(tuple(e + 2 * D for e in env[::-1]), np.float32)
    rng = np.random.default_rng(seed)
    dom[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    return dom


def run_gpu(b2r, dom, env, D, nsteps, coef, blocks=(1, 1, 1), R=1):
    with b2r.Domain(b2r.MODEL_HEAT, env, blocks=blocks, R=R, D=D, alpha_dt=coef[0], dx=coef[1],
                    dy=coef[2], dz=coef[3]) as d:
        assert d.domain_shape == dom.shape
        d.upload(dom)
        d.step(nsteps)
        out = d.download()
        d.synchronize()
    return out


@pytest.mark.parametrize("D", [1, 2, 3, 4])
@pytest.mark.parametrize("env", [(64, 48, 40), (131, 37, 29), (257, 20, 12)])
def test_heat_domain_matches_oracle(b2r, orc, D, env):
    coef = (0.1, 1.0, 1.0, 1.0) if D == 1 else (0.02, 1.0, 1.3, 0.9)
    dom = shell_domain(env, D, 100 + D)
    got = run_gpu(b2r, dom, env, D, 12, coef)
    ref = dom.copy()
    orc.heat_run(ref, D, D, 12, *coef)
    ref64 = dom.astype(np.float64)
    orc.heat_run(ref64, D, D, 12, *coef)
    r32, r64 = rel_l2(got, ref), rel_l2(got, ref64)
    print(f"D={D} env={env}: rel-L2 vs oracle FP32 {r32:.2e}, vs FP64 {r64:.2e}")
    assert r32 <= TOL and r64 <= TOL
    # the fixed shell is never written
    s = np.ones(dom.shape, bool)
    s[D:-D, D:-D, D:-D] = False
    assert np.array_equal(got[s], dom[s])


def test_heat_matches_reference_fixture(b2r):
    g = np.load(os.path.join(GOLD, "heat_d1_small.npz"))
    dom = g["in_shell"]
    env = tuple(n - 2 for n in dom.shape[::-1])
    got = run_gpu(b2r, dom, env, 1, 10, (0.1 * 0.1, 1.0, 1.0, 0.5))
    assert rel_l2(got, g["out_r1x10"]) <= TOL


@pytest.mark.parametrize("coef", [(0.1 * 0.1, 1.0, 1.0, 0.5), (0.1, 1.0, 1.0, 1.0)])
def test_heat_128_config(b2r, orc, coef):
    """128^3 interior, 100 steps, R=1: the reference's constants and the
    isotropic alpha*dt/dx^2 = 0.1 of the benchmark configuration."""
    meta = json.load(open(os.path.join(GOLD, "heat_d1_cfg128.json")))
    dom = np.zeros((130, 130, 130), np.float32)
    rng = np.random.default_rng(meta["seed"])
    dom[1:-1, 1:-1, 1:-1] = rng.random((128, 128, 128), dtype=np.float32)
    got = run_gpu(b2r, dom, (128, 128, 128), 1, 100, coef)
    ref = dom.copy()
    orc.heat_run(ref, 1, 1, 100, *coef)
    r = rel_l2(got, ref)
    print(f"128^3 x100 coef={coef}: rel-L2 {r:.2e}")
    assert r <= TOL
    if coef[3] == 0.5:
        assert abs(got.astype(np.float64).sum() - meta["sum_out"]) / meta["sum_out"] < 1e-5


@pytest.mark.parametrize("D,R,blocks", [(1, 2, (2, 2, 2)), (1, 4, (4, 1, 2)), (2, 3, (2, 2, 1)),
                                        (3, 1, (1, 2, 2)), (4, 2, (2, 1, 1))])
def test_heat_invariant_in_R_and_blocks(b2r, D, R, blocks):
    env = (96, 48, 64)
    coef = (0.02, 1.0, 1.0, 0.8)
    dom = shell_domain(env, D, 5)
    one = run_gpu(b2r, dom, env, D, 11, coef)
    many = run_gpu(b2r, dom, env, D, 11, coef, blocks=blocks, R=R)
    # every cell is computed by the same instructions from the same inputs
    assert np.array_equal(one, many)


@pytest.mark.parametrize("R,ef", [(1, None), (3, None), (2, (-1, 0, 1)), (3, (1, -1, 0))])
def test_heat_3D_gpu_main_block_entry(b2r, orc, R, ef):
    """heat-3D.cu:583 semantics: R shrinking sub-steps on one padded block,
    planes [R*D, Ngz-R*D) copied back."""
    rng = np.random.default_rng(R)
    blk = rng.random((30, 26, 41), dtype=np.float32)
    got = blk.copy()
    b2r.heat_3D_gpu_main(got, R, D=1, edge_flag=ef)
    # oracle: same ping-pong, region and copy-back
    edge = 0
    if ef:
        for a in range(3):
            edge |= (1 << (2 * a)) if ef[a] < 0 else 0
            edge |= (1 << (2 * a + 1)) if ef[a] > 0 else 0
    a, b = blk.copy(), blk.copy()
    for i in range(R):
        orc.heat_substep(a, b, 1, i, R, edge, **orc.REF_HEAT)
        a, b = b, a
    ref = blk.copy()
    ref[R:-R] = a[R:-R]
    assert rel_l2(got, ref) <= TOL
    # untouched planes stay bit-identical
    assert np.array_equal(got[:R], blk[:R]) and np.array_equal(got[-R:], blk[-R:])


def test_run_host_roundtrip(b2r, orc):
    env = (40, 40, 40)
    dom = shell_domain(env, 1, 9)
    out = np.empty_like(dom)
    with b2r.Domain(b2r.MODEL_HEAT, env, D=1, alpha_dt=0.1) as d:
        d.run_host(dom, 5, out)
    ref = dom.copy()
    orc.heat_run(ref, 1, 1, 5, 0.1, 1.0, 1.0, 1.0)
    assert rel_l2(out, ref) <= TOL


@pytest.mark.parametrize("env,blocks,R,periodic", [((131, 37, 29), (1, 1, 1), 1, False),
                                                   ((250, 61, 47), (1, 1, 1), 3, False),
                                                   ((96, 48, 64), (2, 2, 2), 3, False),
                                                   ((64, 64, 48), (2, 1, 2), 4, True),
                                                   ((33, 17, 9), (1, 1, 1), 1, False),
                                                   ((121, 57, 70), (1, 1, 1), 1, False),
                                                   ((240, 52, 40), (2, 2, 1), 5, False),
                                                   ((96, 96, 96), (2, 2, 2), 8, True),
                                                   ((7, 130, 12), (1, 1, 1), 1, False)])
@pytest.mark.parametrize("tb,zc2,tb16,nar", [(2, 0, 0, 0), (2, 0, 1, 0), (2, 0, 1, 1), (3, 0, 0, 0), (3, 33, 0, 0),
                                            (3, 0, 0, 1), (3, 17, 0, 1), (4, 0, 0, 0), (4, 8, 0, 0), (4, 0, 0, 1)])
def test_several_step_sweeps_bit_identical(b2r, orc, env, blocks, R, periodic, tb, zc2, tb16, nar):
    """Two (8-warp and 16-warp kernels), three and four sub-steps per HBM
    pass (radius 1; tiles of 128 x 32 and 64 x 64 cells) against one step
    per launch: 11 steps, so every schedule also runs a shorter pass (four
    steps: 4 + 4 + 3; three: 3 + 3 + 3 + 2), and passes stop at period ends
    where the blocks exchange halos."""
    bc = b2r.BC_PERIODIC if periodic else b2r.BC_SHELL
    rng = np.random.default_rng(8)
    if periodic:
        dom = rng.random(env[::-1], dtype=np.float32)
    else:
        dom = shell_domain(env, 1, 8)
    outs = []
    for t, z, w, n in ((1, 0, 0, 0), (tb, zc2, tb16, nar)):
        with b2r.Domain(b2r.MODEL_HEAT, env, blocks=blocks, R=R, D=1, boundary=bc, alpha_dt=0.1) as d:
            d.set_tuning(tblock=t, zchunk2=z, tb16=w, tb_narrow=n)
            d.upload(dom)
            d.step(11)
            outs.append(d.download())
    assert np.array_equal(outs[0], outs[1])
    if not periodic:
        ref = dom.copy()
        orc.heat_run(ref, 1, 1, 11, 0.1, 1.0, 1.0, 1.0)
        assert rel_l2(outs[1], ref) <= TOL
    else:
        # the torus against a float64 restatement with wrapped neighbours
        assert rel_l2(outs[1], orc.heat_run_periodic(dom, 11, 0.1)) <= TOL


@pytest.mark.parametrize("env,blocks,R,periodic", [((131, 37, 29), (1, 1, 1), 1, False),
                                                   ((250, 61, 47), (1, 1, 1), 3, False),
                                                   ((96, 48, 64), (2, 2, 2), 3, False),
                                                   ((64, 64, 48), (2, 1, 2), 4, True),
                                                   ((33, 17, 9), (1, 1, 1), 1, False),
                                                   ((200, 130, 70), (1, 1, 1), 2, False),
                                                   ((240, 52, 40), (2, 2, 1), 5, False),
                                                   ((96, 96, 96), (2, 2, 2), 6, True),
                                                   ((7, 130, 12), (1, 1, 1), 1, False)])
@pytest.mark.parametrize("zc2", [0, 9, 64])
def test_radius2_two_step_sweep_bit_identical(b2r, orc, env, blocks, R, periodic, zc2):
    """Two sub-steps of radius 2 per HBM pass (heat_tb2.cu) against one step
    per launch: 11 steps, so runs end with a one-step pass, and passes stop
    at period ends where the blocks exchange halos (R = 1 and odd R leave
    one-step passes inside the run)."""
    bc = b2r.BC_PERIODIC if periodic else b2r.BC_SHELL
    rng = np.random.default_rng(9)
    dom = rng.random(env[::-1], dtype=np.float32) if periodic else shell_domain(env, 2, 9)
    outs = []
    for t in (1, 2):
        with b2r.Domain(b2r.MODEL_HEAT, env, blocks=blocks, R=R, D=2, boundary=bc, alpha_dt=0.03) as d:
            d.set_tuning(tblock=t, zchunk2=zc2, tb_r2=1)
            d.upload(dom)
            d.step(11)
            outs.append(d.download())
    assert np.array_equal(outs[0], outs[1])
    if not periodic:
        ref = dom.copy()
        orc.heat_run(ref, 2, 2, 11, 0.03, 1.0, 1.0, 1.0)
        assert rel_l2(outs[1], ref) <= TOL


@pytest.mark.parametrize("env", [(64, 2, 48), (2, 40, 33), (37, 29, 2), (3, 3, 3)])
@pytest.mark.parametrize("D", [1, 2])
def test_heat_thin_domains(b2r, orc, env, D):
    """Domains a few cells thick along one axis (TMA boxes larger than the
    block, windows of one or two cells) against the oracle."""
    if D > min(env) // 2:
        pytest.skip("R*D <= min(B)/2 (b2r.cpp:54)")
    rng = np.random.default_rng(15)
    dom = np.zeros(tuple(e + 2 * D for e in env[::-1]), np.float32)
    dom[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    with b2r.Domain(b2r.MODEL_HEAT, env, D=D, R=1, alpha_dt=0.05) as d:
        d.upload(dom)
        d.step(7)
        got = d.download()
        d.synchronize()
    ref = dom.copy()
    orc.heat_run(ref, D, D, 7, 0.05, 1.0, 1.0, 1.0)
    r = float(np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref))
    assert r <= 1e-5


@pytest.mark.parametrize("D", [1, 2, 3, 4])
def test_heat_periodic_matches_torus_oracle(b2r, orc, D):
    """Radius 1-4 on a torus split into 2 x 1 x 2 blocks (deep halo R = 2,
    exchanged across the wrap) against the float64 torus restatement."""
    env = (48, 40, 56)
    rng = np.random.default_rng(30 + D)
    dom = rng.random(env[::-1], dtype=np.float32)
    with b2r.Domain(b2r.MODEL_HEAT, env, blocks=(2, 1, 2), R=2, D=D, boundary=b2r.BC_PERIODIC,
                    alpha_dt=0.02, dx=1.0, dy=1.5, dz=0.75) as d:
        assert d.domain_shape == env[::-1]
        d.upload(dom)
        d.step(9)
        got = d.download()
    ref = orc.heat_run_periodic(dom, 9, 0.02, 1.0, 1.5, 0.75, D=D)
    assert rel_l2(got, ref) <= TOL
