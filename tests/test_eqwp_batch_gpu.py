"""Batched staggered elastic-wave instances (one persistent launch over
several handles): every instance equal, bit for bit, to the same handle
stepped on its own with the two-pass step, over two runs in a row (the
second continuing from the first's time step and source samples), and the
batch's arguments checked."""
import numpy as np
import pytest

from test_eqwp_gpu import layered, ricker

pytestmark = pytest.mark.gpu
H = 10.0
DT = 0.5 * H / (4000 * np.sqrt(3) * (9 / 8 + 1 / 24))


def instances(n, seed):
    rng = np.random.default_rng(seed)
    edges = np.arange(16, 65, 8)
    out = []
    for i in range(n):
        env = tuple(int(v) for v in rng.choice(edges, 3))
        out.append(dict(env=env, nsteps=int(rng.integers(3, 14)), seed=100 + i,
                        src=tuple(int(rng.integers(2, e - 2)) for e in env)))
    return out


def make(b2r, it, stream=None, sync=True):
    d = b2r.Domain(b2r.MODEL_EQWP_STAG, it["env"], D=2, R=1, dt=DT, h=H, src=it["src"], stream=stream)
    mat = layered(it["env"], seed=it["seed"])
    for m, name in enumerate(["lambda", "mu", "buoy"]):
        d.upload(mat[m].astype(np.float32), field=name)
    rng = np.random.default_rng(it["seed"])
    shape = d.domain_shape
    for k in range(9):
        a = np.zeros(shape, np.float32)
        a[2:-2, 2:-2, 2:-2] = ((rng.random(tuple(s - 4 for s in shape)) - 0.5) * 1e-3).astype(np.float32)
        d.upload(a, field=k)
    d.set_source(ricker(64, DT, 10.0, 1e6 * DT).astype(np.float32))
    if sync:
        d.synchronize()
    return d


@pytest.mark.parametrize("graph,zchunk,own", [(True, 32, False), (False, 8, False), (True, 0, False),
                                              (True, 32, True)])
def test_eqwp_batch_matches_handles(b2r, graph, zchunk, own):
    """own: the domains on streams of their own, uploads not waited for --
    the run is ordered after them, and the downloads after the run, by
    events."""
    import torch
    items = instances(7, 5)
    s = torch.cuda.Stream()
    doms = [make(b2r, it, stream=None if own else s, sync=not own) for it in items]
    refs = [make(b2r, it) for it in items]
    try:
        with b2r.EqwpBatch(doms, [it["nsteps"] for it in items], stream=s) as bt:
            bt.set_zchunk(zchunk)
            assert bt.lups == sum(int(np.prod(it["env"])) * it["nsteps"] for it in items)
            for run in range(2):
                bt.run(graph=graph)
                bt.synchronize()
                for d, r, it in zip(doms, refs, items):
                    r.step(it["nsteps"])
                    assert d.time_step == r.time_step == (run + 1) * it["nsteps"]
                    for k in range(9):
                        got, want = d.download(field=k), r.download(field=k)
                        assert np.array_equal(got, want), (run, it, k)
        # the handles go on as usual after the batch
        doms[0].step(2)
        refs[0].step(2)
        assert np.array_equal(doms[0].download(field=3), refs[0].download(field=3))
    finally:
        for d in doms + refs:
            d.close()


def test_eqwp_batch_rejects_bad_instances(b2r):
    it = dict(env=(16, 16, 16), nsteps=2, seed=1, src=(8, 8, 8))
    d = make(b2r, it)
    with b2r.Domain(b2r.MODEL_HEAT, (16, 16, 16)) as heat, \
         b2r.Domain(b2r.MODEL_EQWP_STAG, (32, 16, 16), blocks=(2, 1, 1), D=2, R=1, dt=DT, h=H) as two:
        for bad, ns in (([heat], [2]), ([two], [2]), ([d, d], [1, 1]), ([d], [-1]),
                        ([d], [9_000_000])):          # 18 M rounds: more than a queue item names
            with pytest.raises(b2r.B2RError):
                b2r.EqwpBatch(bad, ns)
    d.close()


def test_eqwp_batch_long_instance(b2r):
    """An instance of 9000 steps (18000 rounds of the queue, once refused
    for the size of its schedule tables) beside a short one: both equal the
    same handles stepped alone."""
    import torch
    items = [dict(env=(16, 16, 16), nsteps=9000, seed=31, src=(8, 8, 8)),
             dict(env=(24, 16, 20), nsteps=5, seed=32, src=(12, 8, 10))]
    s = torch.cuda.Stream()
    doms = [make(b2r, it, stream=s) for it in items]
    refs = [make(b2r, it) for it in items]
    try:
        with b2r.EqwpBatch(doms, [it["nsteps"] for it in items], stream=s) as bt:
            bt.run(graph=False)
            bt.synchronize()
        for d, r, it in zip(doms, refs, items):
            r.step(it["nsteps"])
            for k in range(9):
                assert np.array_equal(d.download(field=k), r.download(field=k)), (it["env"], k)
    finally:
        for d in doms + refs:
            d.close()
