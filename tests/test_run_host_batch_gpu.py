"""Pipelined host runs (b2r_run_host_batch): the same bits as one
b2r_run_host per input (heat, Game of Life) or as per-field uploads and
downloads (the elastic wave, whose problem is the whole wavefield), with the
copies of the next input and the previous result overlapping the stepping."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(b2r, d, model, n, seed):
    rng = np.random.default_rng(seed)
    if model == b2r.MODEL_GOL:
        return [(rng.random(d.domain_shape) < 0.3).astype(np.uint8) for _ in range(n)]
    return [rng.random(d.domain_shape, dtype=np.float32) for _ in range(n)]


@pytest.mark.parametrize("model,env,blocks,R,kw", [
    (1, (64, 48, 40), (1, 1, 1), 1, dict(alpha_dt=0.1)),
    (1, (64, 64, 64), (2, 2, 1), 2, dict(alpha_dt=0.05, D=2)),
    (2, (64, 64, 64), (2, 2, 2), 4, dict(boundary=1)),
])
@pytest.mark.parametrize("count", [1, 2, 5])
def test_run_host_batch_matches_run_host(b2r, model, env, blocks, R, kw, count):
    import torch
    kw = dict(kw)
    D = kw.pop("D", 1)
    boundary = kw.pop("boundary", b2r.BC_SHELL)
    s = torch.cuda.Stream()
    with b2r.Domain(model, env, blocks=blocks, R=R, D=D, boundary=boundary, stream=s, **kw) as d:
        ins = _inputs(b2r, d, model, count, 7)
        pin_in = [torch.from_numpy(a).pin_memory() for a in ins]
        pin_out = [torch.empty_like(p).pin_memory() for p in pin_in]
        nsteps = 3 * R + 1
        d.run_host_batch(pin_in, nsteps, pin_out)
        ref = [np.empty_like(a) for a in ins]
        for a, r in zip(ins, ref):
            d.run_host(a, nsteps, r)
        d.synchronize()
        for k in range(count):
            assert np.array_equal(pin_out[k].numpy(), ref[k]), k
        # a second call reuses the buffers and streams
        d.run_host_batch(pin_in[::-1], nsteps, pin_out)
        d.synchronize()
        for k in range(count):
            assert np.array_equal(pin_out[k].numpy(), ref[count - 1 - k]), k


def test_run_host_batch_rejects_wrong_sizes(b2r):
    with b2r.Domain(b2r.MODEL_HEAT, (16, 16, 16)) as d:
        a = np.zeros(d.domain_shape, np.float32)
        with pytest.raises(ValueError):
            d.run_host_batch([a], 1, [np.zeros(10, np.float32)])


@pytest.mark.parametrize("model", ["ref", "stag"])
def test_run_host_batch_elastic_wave(b2r, model):
    """Elastic wave: a problem is every wavefield component back to back
    (ten with the displacement for the reference model); the material stays
    resident.  Same bits as uploading, stepping and downloading each field."""
    import torch
    rng = np.random.default_rng(11)
    s = torch.cuda.Stream()
    if model == "ref":
        m, env, kw = b2r.MODEL_EQWP_REF, (40, 24, 32), dict(R=1, D=2)
    else:
        m, env, kw = b2r.MODEL_EQWP_STAG, (64, 48, 40), dict(blocks=(2, 1, 1), R=2, D=2, dt=1e-3, h=10.0,
                                                             src=(30, 20, 18))
    with b2r.Domain(m, env, stream=s, **kw) as d:
        nf = d.nfields
        assert nf == (10 if model == "ref" else 9)
        if model == "stag":
            for name, v in (("lambda", 2e10), ("mu", 1e10), ("buoy", 1 / 2400.0)):
                d.upload(np.full(d.domain_shape, v, np.float32), field=name)
            d.set_source(np.sin(np.arange(64, dtype=np.float32)) * 1e3)
        shell = 2
        ins = []
        for _ in range(3):
            w = np.zeros((nf,) + d.domain_shape, np.float32)
            w[:, shell:-shell, shell:-shell, shell:-shell] = (
                (rng.random((nf,) + tuple(env[::-1]), dtype=np.float32) - 0.5) * 1e-2)
            ins.append(w)
        pin_in = [torch.from_numpy(a).pin_memory() for a in ins]
        pin_out = [torch.empty_like(p).pin_memory() for p in pin_in]
        nsteps = 5
        d.run_host_batch(pin_in, nsteps, pin_out)
        d.synchronize()
        for k, w in enumerate(ins):
            for f in range(nf):
                d.upload(w[f], field=f)
            d.step(nsteps)
            ref = np.stack([d.download(field=f) for f in range(nf)])
            d.synchronize()
            assert np.abs(ref).max() > 0
            assert np.array_equal(pin_out[k].numpy(), ref), k
        with pytest.raises(ValueError):
            d.run_host_batch([ins[0][0]], 1, [np.empty_like(ins[0][0])])
