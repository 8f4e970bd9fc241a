"""The heat autotuner: picks a launch schedule, keeps the state, changes no bits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_keeps_state_and_results(b2r):
    import torch
    env, D = (96, 64, 80), 2
    rng = np.random.default_rng(3)
    dom = np.zeros(tuple(e + 2 * D for e in env[::-1]), np.float32)
    dom[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    outs = []
    for tune in (False, True):
        s = torch.cuda.Stream()
        with b2r.Domain(b2r.MODEL_HEAT, env, blocks=(2, 1, 2), R=2, D=D, alpha_dt=0.02,
                        stream=s) as d:
            d.upload(dom)
            d.step(5)
            if tune:
                best, ms = d.autotune(2)
                assert best["zchunk"] in (0, 16, 32, 64, 128, 256)
                assert 0 <= best["ctas_per_sm"] <= 6 and best["pdl"] in (0, 1)
                assert d.time_step == 5
            d.step(9)
            outs.append(d.download())
            d.synchronize()
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("zchunk,cps,pdl", [(16, 0, 0), (7, 2, 1), (64, 1, 1), (0, 6, 0)])
def test_schedules_bit_identical(b2r, zchunk, cps, pdl):
    env, D = (130, 40, 70), 1
    rng = np.random.default_rng(4)
    dom = np.zeros(tuple(e + 2 * D for e in env[::-1]), np.float32)
    dom[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    res = []
    for t in (None, (zchunk, cps, pdl)):
        with b2r.Domain(b2r.MODEL_HEAT, env, D=D, alpha_dt=0.1) as d:
            if t:
                d.set_tuning(*t)
            d.upload(dom)
            d.step(6)
            res.append(d.download())
    assert np.array_equal(res[0], res[1])
