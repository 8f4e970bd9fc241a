"""The autotuners (heat schedules; Game-of-Life and staggered elastic-wave
kernel choices): each picks a launch schedule, keeps the state and changes
no bits."""
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


@pytest.mark.parametrize("model", ["gol", "stag"])
def test_knob_autotune_keeps_state_and_bits(b2r, model):
    """Game of Life and the staggered elastic wave: the autotuner times their
    kernel choices on the live fields, restores them and changes no bits."""
    import torch
    rng = np.random.default_rng(5)
    if model == "gol":
        env, kw = (64, 64, 64), dict(blocks=(2, 2, 2), R=4, D=1, boundary=b2r.BC_PERIODIC)
        m = b2r.MODEL_GOL
        init = {0: (rng.random(env[::-1]) < 0.3).astype(np.uint8)}
    else:
        env, kw = (64, 48, 40), dict(blocks=(2, 1, 1), R=2, D=2, dt=1e-3, h=10.0, src=(30, 20, 18))
        m = b2r.MODEL_EQWP_STAG
        shape = tuple(e + 4 for e in env[::-1])
        init = {"lambda": np.full(shape, 2e10, np.float32), "mu": np.full(shape, 1e10, np.float32),
                "buoy": np.full(shape, 1 / 2400.0, np.float32)}
        for k in range(9):
            a = np.zeros(shape, np.float32)
            a[2:-2, 2:-2, 2:-2] = ((rng.random(env[::-1]) - 0.5) * 1e-2).astype(np.float32)
            init[k] = a
    outs = []
    for tune in (False, True):
        s = torch.cuda.Stream()
        with b2r.Domain(m, env, stream=s, **kw) as d:
            for f, a in init.items():
                d.upload(a, field=f)
            d.step(4)
            if tune:
                best, ms = d.autotune(2)
                assert d.time_step == 4
                if model == "gol":
                    assert best["tblock"] in (1, 2, 4) and best["gol_bytes"] in (0, 1)
                else:
                    assert best["eqwp_fused"] in (0, 1)
            d.step(6)
            outs.append([d.download(field=f) for f in (range(9) if model == "stag" else [0])])
            d.synchronize()
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_every_knob_round_trips_and_unknown_keys_are_refused(b2r):
    """Each of the 15 knobs reads back what was set (boolean knobs as 0/1),
    on a handle of each model; keys outside 1..15 are refused through both
    entry points."""
    import ctypes as C
    values = dict(zchunk=24, ctas_per_sm=3, pdl=0, tblock=3, zchunk2=40, eqwp_fused=1, gol_bytes=1,
                  adj_fused=0, gol_push=1, tb16=1, tb_narrow=1, tb_r2=1, eqwp_tma=1, eqwp_overlap=1,
                  gol_rows=48)
    for model, kw in ((b2r.MODEL_HEAT, dict(D=1)), (b2r.MODEL_GOL, dict(D=1)),
                      (b2r.MODEL_EQWP_STAG, dict(D=2, dt=1e-4, h=10.0))):
        with b2r.Domain(model, (32, 32, 32), **kw) as d:
            d.set_tuning(**values)
            assert d.get_tuning() == values, model
            for key in (0, 16, -1):
                with pytest.raises(b2r.B2RError):
                    b2r._check(b2r.lib().b2r_set_tuning(d.h, key, 1), d.h)
                v = C.c_int()
                with pytest.raises(b2r.B2RError):
                    b2r._check(b2r.lib().b2r_get_tuning(d.h, key, C.byref(v)), d.h)
