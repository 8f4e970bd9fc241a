"""Pipelined host runs (b2r_run_host_batch): the same bits as one
b2r_run_host per input, for heat and Game of Life, with the copies of the
next input and the previous result overlapping the stepping."""
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
