"""Periods replayed from CUDA graphs give the same bits as direct launches;
handles driven from several host threads at once (first launches included)
give the bits of the same runs one after the other."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(b2r, model, env, blocks, R, D, dom, nsteps, graphs, **kw):
    import torch
    s = torch.cuda.Stream()
    with b2r.Domain(model, env, blocks=blocks, R=R, D=D, stream=s, **kw) as d:
        d.set_graphs(graphs)
        d.upload(dom)
        d.step(3)            # start mid-period, then whole periods, then a remainder
        d.step(nsteps)
        out = d.download()
        d.synchronize()
    return out


@pytest.mark.parametrize("blocks,R,D", [((1, 1, 1), 1, 1), ((2, 2, 2), 3, 1), ((2, 1, 2), 2, 4)])
def test_heat_graphs_bit_identical(b2r, blocks, R, D):
    env = (64, 48, 80)
    rng = np.random.default_rng(1)
    dom = np.zeros(tuple(e + 2 * D for e in env[::-1]), np.float32)
    dom[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    a = run(b2r, b2r.MODEL_HEAT, env, blocks, R, D, dom, 75, False, alpha_dt=0.02)
    b = run(b2r, b2r.MODEL_HEAT, env, blocks, R, D, dom, 75, True, alpha_dt=0.02)
    assert np.array_equal(a, b)


def test_gol_graphs_bit_identical(b2r, orc):
    env = (64, 64, 64)
    rng = np.random.default_rng(2)
    dom = (rng.random(env[::-1]) < 0.3).astype(np.uint8)
    a = run(b2r, b2r.MODEL_GOL, env, (2, 2, 2), 4, 1, dom, 70, True, boundary=b2r.BC_PERIODIC)
    ref = dom.copy()
    orc.gol_run_periodic(ref, 73)
    assert np.array_equal(a, ref)


def test_bounded_wait_reports_timeout_and_context_survives(b2r, orc):
    """The device failure path: a wait that nothing completes gives up after
    its limit and reports B2R_ERR_TIMEOUT; the next work on the GPU is right."""
    import time
    t0 = time.perf_counter()
    st = b2r.lib().b2r_selfcheck_bounded_wait(50.0, None)
    dt = time.perf_counter() - t0
    assert st == 4, st                      # B2R_ERR_TIMEOUT
    assert dt < 5.0
    env = (40, 36, 32)
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.float32)
    dom[1:-1, 1:-1, 1:-1] = np.random.default_rng(1).random(env[::-1], dtype=np.float32)
    with b2r.Domain(b2r.MODEL_HEAT, env, D=1, alpha_dt=0.1) as d:
        d.upload(dom)
        d.step(6)
        got = d.download()
    ref = dom.copy()
    orc.heat_run(ref, 1, 1, 6, 0.1, 1.0, 1.0, 1.0)
    assert np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref) <= 1e-5


def test_oom_is_reported_and_the_context_stays_usable(b2r, orc):
    """A domain larger than the GPU's memory is refused with B2R_ERR_OOM; the
    next handle works (the failed allocation leaves no error behind)."""
    with pytest.raises(b2r.B2RError) as ei:
        b2r.Domain(b2r.MODEL_HEAT, (4800, 4800, 4800), D=1)
    assert "B2R_ERR_OOM" in str(ei.value)
    env = (40, 32, 24)
    rng = np.random.default_rng(8)
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.float32)
    dom[1:-1, 1:-1, 1:-1] = rng.random(env[::-1], dtype=np.float32)
    with b2r.Domain(b2r.MODEL_HEAT, env, D=1, alpha_dt=0.1) as d:
        d.upload(dom)
        d.step(3)
        got = d.download()
        d.synchronize()
    ref = dom.copy()
    orc.heat_run(ref, 1, 1, 3, 0.1, 1.0, 1.0, 1.0)
    assert float(np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref)) <= 1e-5


def test_handles_on_two_host_threads(b2r):
    """One handle per host thread: heat and Game of Life stepped from two
    threads at once give the bits of the same runs one after the other."""
    import threading
    import torch
    rng = np.random.default_rng(13)
    henv, genv = (64, 48, 80), (64, 64, 64)
    hdom = np.zeros(tuple(e + 2 for e in henv[::-1]), np.float32)
    hdom[1:-1, 1:-1, 1:-1] = rng.random(henv[::-1], dtype=np.float32)
    gdom = (rng.random(genv[::-1]) < 0.3).astype(np.uint8)

    def heat(out):
        s = torch.cuda.Stream()
        with b2r.Domain(b2r.MODEL_HEAT, henv, blocks=(2, 1, 2), R=2, D=1, alpha_dt=0.05, stream=s) as d:
            d.upload(hdom)
            d.step(41)
            out.append(d.download())
            d.synchronize()

    def gol(out):
        s = torch.cuda.Stream()
        with b2r.Domain(b2r.MODEL_GOL, genv, blocks=(2, 2, 2), R=4, D=1, boundary=b2r.BC_PERIODIC,
                        stream=s) as d:
            d.upload(gdom)
            d.step(42)
            out.append(d.download())
            d.synchronize()

    ref_h, ref_g = [], []
    heat(ref_h)
    gol(ref_g)
    got_h, got_g = [], []
    threads = [threading.Thread(target=heat, args=(got_h,)), threading.Thread(target=gol, args=(got_g,))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert np.array_equal(got_h[0], ref_h[0])
    assert np.array_equal(got_g[0], ref_g[0])


FIRST_USE_SCRIPT = r"""
import sys, threading
import os

import numpy as np
sys.path.insert(0, sys.argv[1])
import b2r_gb300 as b2r
env = (48, 40, 32)
cases = [dict(D=1), dict(D=2), dict(D=4), dict(D=1, R=2, blocks=(2, 1, 1)), dict(D=2, R=2, blocks=(1, 2, 1))]

def start(c):
    rng = np.random.default_rng(c["D"])
    D = c["D"]
    dom = np.zeros(tuple(e + 2 * D for e in env[::-1]), np.float32)
    dom[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    return dom

def run(c, out, gate=None):
    with b2r.Domain(b2r.MODEL_HEAT, env, alpha_dt=0.02, **c) as d:
        d.upload(start(c))
        d.synchronize()
        if gate is not None:
            gate.wait()
        d.step(7)
        out.append(d.download())
        d.synchronize()

gate = threading.Barrier(len(cases))
outs = [[] for _ in cases]
ths = [threading.Thread(target=run, args=(c, o, gate)) for c, o in zip(cases, outs)]
for t in ths: t.start()
for t in ths: t.join()
for c, o in zip(cases, outs):
    ref = []
    run(c, ref)
    assert len(o) == 1 and np.array_equal(o[0], ref[0]), c
print("first-use threads ok")
"""


def test_first_launches_from_many_threads(b2r):
    """Kernel setup (shared-memory limit, occupancy) happens on a kernel's
    first launch: five threads of a fresh process making their first heat
    launches at once (the two-step and one-step sweeps, several radii) get
    the bits of the same runs made afterwards one at a time."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", FIRST_USE_SCRIPT, root], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "first-use threads ok" in r.stdout
