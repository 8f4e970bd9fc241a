"""Batched persistent launch: every instance matches its own plain run,
whatever tile shape each instance runs with."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def mix(n, seed, max_edge=96, max_steps=40):
    rng = np.random.default_rng(seed)
    edges = np.arange(32, max_edge + 1, 16)
    items = []
    for _ in range(n):
        items.append(dict(env=tuple(int(v) for v in rng.choice(edges, 3)), D=int(rng.integers(1, 5)),
                          nsteps=int(rng.integers(5, max_steps + 1)), alpha_dt=0.02, dx=1.0, dy=1.0,
                          dz=1.0))
    return items


def inputs(items, seed):
    rng = np.random.default_rng(seed)
    out = []
    for it in items:
        D = it["D"]
        a = np.zeros(tuple(e + 2 * D for e in it["env"][::-1]), np.float32)
        a[D:-D, D:-D, D:-D] = rng.random(it["env"][::-1], dtype=np.float32)
        out.append(a)
    return out


@pytest.mark.parametrize("graph,tile,steps", [(False, 0, 1), (True, 0, 1), (False, 128, 1), (True, 64, 1),
                                              (False, 32, 1), (False, 0, 2), (True, 32, 2)])
def test_batch_matches_plain_runs(b2r, orc, graph, tile, steps):
    """steps = 2: the radius-1 instances on two-step units (odd step counts
    end with a one-step unit), beside one-step instances of the other
    radii in the same launch."""
    import torch
    items = mix(12, 1)
    ins = inputs(items, 2)
    s = torch.cuda.Stream()
    with b2r.Batch(items, stream=s) as bt:
        bt.set_tile(tile)
        widths = bt.instance_tiles()
        assert set(widths) <= {128, 64, 32}
        if tile:
            assert bt.tile == tile and set(widths) == {tile}
        else:
            # each instance on its own fewest-cells shape: this mix holds
            # 64- and 32-cell-wide tiles in the one launch
            assert len(set(widths)) >= 2 and bt.tile == 0
        bt.set_pass_steps(steps)
        ps = bt.instance_pass_steps()
        assert ps == [steps if it["D"] == 1 else 1 for it in items]
        if steps == 2:
            d1 = [it["nsteps"] for it in items if it["D"] == 1]
            assert any(n % 2 for n in d1) and any(n % 2 == 0 for n in d1)
        for i, a in enumerate(ins):
            bt.upload(i, a)
        bt.run(graph=graph)
        bt.synchronize()
        got = [bt.download(i) for i in range(len(items))]
        # a second run from the same inputs gives the same bits
        for i, a in enumerate(ins):
            bt.upload(i, a)
        bt.run(graph=graph)
        bt.synchronize()
        again = [bt.download(i) for i in range(len(items))]
    for i, it in enumerate(items):
        with b2r.Domain(b2r.MODEL_HEAT, it["env"], D=it["D"], alpha_dt=0.02) as d:
            d.upload(ins[i])
            d.step(it["nsteps"])
            plain = d.download()
        assert np.array_equal(got[i], plain), i
        assert np.array_equal(again[i], plain), i
    # and the oracle agrees within the FP32 tolerance: on every instance (each
    # radius and size) with each instance's own tile shape, one step or two
    # per unit; on two of them otherwise
    for i in (range(len(items)) if not graph and not tile else (0, 5)):
        ref = ins[i].copy()
        it = items[i]
        orc.heat_run(ref, it["D"], it["D"], it["nsteps"], 0.02, 1.0, 1.0, 1.0)
        rel = np.linalg.norm(got[i].astype(np.float64) - ref) / np.linalg.norm(ref)
        assert rel <= 1e-5


def test_batch_autotune_keeps_inputs(b2r):
    import torch
    items = mix(6, 3, max_edge=64, max_steps=12)
    ins = inputs(items, 4)
    s = torch.cuda.Stream()
    with b2r.Batch(items, stream=s) as bt:
        for i, a in enumerate(ins):
            bt.upload(i, a)
        z, ms = bt.autotune()
        assert z in (8, 16, 32, 64, 0) and ms > 0
        assert set(bt.instance_tiles()) <= {128, 64, 32}
        assert set(bt.instance_pass_steps()) <= {1, 2}
        bt.run()
        bt.synchronize()
        got = [bt.download(i) for i in range(len(items))]
    for i, it in enumerate(items):
        with b2r.Domain(b2r.MODEL_HEAT, it["env"], D=it["D"], alpha_dt=0.02) as d:
            d.upload(ins[i])
            d.step(it["nsteps"])
            assert np.array_equal(got[i], d.download()), i


def test_batches_with_different_schedules_coexist(b2r):
    """A batch created after a larger one (longer schedule, more shared
    memory) does not lower the kernel's shared-memory limit under it: both
    run, concurrently, with their own results."""
    import torch
    big = mix(10, 7, max_steps=300)
    small = mix(3, 8, max_steps=8)
    ins_big, ins_small = inputs(big, 9), inputs(small, 10)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    res = []
    with b2r.Batch(big, stream=s1) as b1, b2r.Batch(small, stream=s2) as b2:
        for bt, ins in ((b1, ins_big), (b2, ins_small)):
            for i, a in enumerate(ins):
                bt.upload(i, a)
        b1.run()
        b2.run()
        b1.synchronize()
        b2.synchronize()
        res = [[b1.download(i) for i in range(len(big))], [b2.download(i) for i in range(len(small))]]
    for items, ins, outs in ((big, ins_big, res[0]), (small, ins_small, res[1])):
        for it, a, got in zip(items, ins, outs):
            with b2r.Domain(b2r.MODEL_HEAT, it["env"], D=it["D"], alpha_dt=it["alpha_dt"]) as d:
                d.upload(a)
                d.step(it["nsteps"])
                want = d.download()
            assert np.array_equal(got, want)


@pytest.mark.parametrize("steps", [1, 2])
def test_batch_tiny_and_thin_instances(b2r, steps):
    """Instances smaller than one tile, and a few cells thick, next to a
    larger one: each matches its own plain run (radius 1 on one-step or
    two-step units)."""
    import torch
    items = [dict(env=(5, 6, 7), D=1, nsteps=9), dict(env=(8, 8, 8), D=2, nsteps=4),
             dict(env=(16, 3, 40), D=1, nsteps=12), dict(env=(96, 80, 64), D=3, nsteps=6),
             dict(env=(2, 2, 2), D=1, nsteps=3)]
    for it in items:
        it.update(alpha_dt=0.03, dx=1.0, dy=1.0, dz=1.0)
    ins = inputs(items, 16)
    s = torch.cuda.Stream()
    with b2r.Batch(items, stream=s) as bt:
        bt.set_pass_steps(steps)
        for i, a in enumerate(ins):
            bt.upload(i, a)
        bt.run()
        bt.synchronize()
        outs = [bt.download(i) for i in range(len(items))]
    for it, a, got in zip(items, ins, outs):
        with b2r.Domain(b2r.MODEL_HEAT, it["env"], D=it["D"], alpha_dt=it["alpha_dt"]) as d:
            d.upload(a)
            d.step(it["nsteps"])
            want = d.download()
        assert np.array_equal(got, want), it


def test_batch_long_instance_beside_short_ones(b2r):
    """An instance of 30000 steps (a queue of 30000 rounds, once refused for
    the size of its schedule tables) beside short instances of every
    radius: each equals its own plain run."""
    import torch
    items = [dict(env=(16, 16, 16), D=1, nsteps=30000, alpha_dt=0.02, dx=1.0, dy=1.0, dz=1.0)]
    items += [dict(env=(24 + 8 * D, 20, 18), D=D, nsteps=3 + D, alpha_dt=0.02, dx=1.0, dy=1.0, dz=1.0)
              for D in (1, 2, 3, 4)]
    ins = inputs(items, 9)
    s = torch.cuda.Stream()
    with b2r.Batch(items, stream=s) as bt:
        assert bt.lups == sum(int(np.prod(it["env"])) * it["nsteps"] for it in items)
        for i, a in enumerate(ins):
            bt.upload(i, a)
        bt.run()
        bt.synchronize()
        got = [bt.download(i) for i in range(len(items))]
    for i, it in enumerate(items):
        with b2r.Domain(b2r.MODEL_HEAT, it["env"], D=it["D"], alpha_dt=0.02) as d:
            d.upload(ins[i])
            d.step(it["nsteps"])
            assert np.array_equal(got[i], d.download()), i


def test_batch_refuses_a_queue_it_cannot_name(b2r):
    """An instance of more than 2^24 rounds cannot be named by a queue item:
    creation is refused (before any queue is allocated) with B2R_ERR_ARG."""
    items = [dict(env=(16, 16, 16), D=1, nsteps=20_000_000, alpha_dt=0.02, dx=1.0, dy=1.0, dz=1.0)]
    with pytest.raises(b2r.B2RError) as ei:
        b2r.Batch(items)
    assert "split the batch" in str(ei.value)
