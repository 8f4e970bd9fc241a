"""Parity at the benchmark's own sizes and launch schedules.

The bench times heat delta 1 at 512^3 with the schedule the autotuner picks
(two time steps per HBM pass, 64-plane units, programmatic dependent launch,
graph-replayed periods), Game of Life on the 256^3 torus as 2 x 2 x 2
subdomains at R = 4 for 400 generations, heat delta 4 at 512^3 and the
staggered elastic wave at 512 x 512 x 256 as 2 x 2 x 1 subdomains at R = 2.
These tests run those exact configurations, from the bench's seeded inputs,
against the oracle: FP32 work within relative L2 1e-5 of the oracle's FP32
restatement (its error against the FP64 restatement printed beside it),
Game of Life bit-exact at every R-th generation, the staggered elastic wave
bit-identical to the FP32 oracle (every operation rounded as the oracle
rounds it).
"""
import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def heat_domain(b2r, wl, stream):
    a, dx, dy, dz = wl["coef"]
    return b2r.Domain(b2r.MODEL_HEAT, wl["env"], blocks=wl["blocks"], R=wl["R"], D=wl["D"], alpha_dt=a,
                      dx=dx, dy=dy, dz=dz, stream=stream)


@pytest.mark.parametrize("workload,nsteps", [("heat1_512", 10), ("heat4_512", 6)])
def test_heat_512_bench_schedule_matches_oracle(b2r, orc, workload, nsteps):
    """heat1_512 with one, two (64-plane units), three and four time steps
    per HBM pass, graphs on, and with whatever the autotuner picks (the
    bench's schedule); heat4_512 with the autotuner's pick.  Every schedule
    gives the same bits."""
    import torch
    wl = bench.WORKLOADS[workload]
    D = wl["D"]
    shape = tuple(e + 2 * D for e in wl["env"][::-1])
    dom = bench.seeded_domain(wl, shape)
    stream = torch.cuda.Stream()
    results = {}
    with heat_domain(b2r, wl, stream) as d:
        schedules = {"autotuned": None}
        if D == 1:
            schedules = {"two-step": dict(tblock=2, zchunk2=64, pdl=1), "one-step": dict(tblock=1),
                         "two-step-16w": dict(tblock=2, zchunk2=0, tb16=1),
                         "three-step": dict(tblock=3, zchunk2=0), "four-step": dict(tblock=4, zchunk2=96),
                         "three-step-64x64": dict(tblock=3, zchunk2=0, tb_narrow=1),
                         **schedules}
        for name, knobs in schedules.items():
            d.upload(dom)
            if knobs is None:
                d.autotune(trial_steps=2)
                d.upload(dom)
            else:
                d.set_tuning(**knobs)
            d.step(nsteps)
            results[name] = d.download()
            d.synchronize()
    ref32 = dom.copy()
    orc.heat_run(ref32, D, D, nsteps, *wl["coef"])
    ref64 = dom.astype(np.float64)
    orc.heat_run(ref64, D, D, nsteps, *wl["coef"])
    first = next(iter(results.values()))
    for name, got in results.items():
        r32, r64 = rel_l2(got, ref32), rel_l2(got, ref64)
        print(f"{workload} x{nsteps} ({name}): rel-L2 vs oracle FP32 {r32:.2e}, vs FP64 {r64:.2e}")
        assert r32 <= TOL, name
        assert np.array_equal(got, first), name
        # the fixed shell is never written
        assert np.array_equal(got[:D], dom[:D]) and np.array_equal(got[-D:], dom[-D:])


def test_gol_256_torus_full_config_bit_exact(b2r, orc):
    """gol_256: 256^3 torus, 2 x 2 x 2 subdomains, R = 4, 400 generations
    from Bernoulli(0.3), with the autotuner's kernel choice; bit-exact
    against the oracle after every period (every 4th generation)."""
    import torch
    wl = bench.WORKLOADS["gol_256"]
    g = bench.seeded_domain(wl, wl["env"][::-1])
    stream = torch.cuda.Stream()
    ref = g.copy()
    with b2r.Domain(b2r.MODEL_GOL, wl["env"], blocks=wl["blocks"], R=wl["R"], D=1, boundary=b2r.BC_PERIODIC,
                    stream=stream) as d:
        d.upload(g)
        knobs, _ = d.autotune(trial_steps=4)
        d.upload(g)
        R = wl["R"]
        for period in range(wl["sub_steps"] // R):
            d.step(R)
            got = d.download()
            orc.gol_run_periodic(ref, R)
            assert np.array_equal(got, ref), f"generation {(period + 1) * R} ({knobs})"
    print(f"gol_256: bit-exact over {wl['sub_steps']} generations, live {float(ref.mean()):.3f}, {knobs}")


def test_eqwp_stag_512x512x256_matches_oracle(b2r, orc):
    """eqwp_stag: 512 x 512 x 256, 2 x 2 x 1 subdomains, R = 2, the bench's
    layered model and Ricker source, from a random wavefield, 8 steps, with
    the autotuner's choice of the one-pass or two-pass step: bit-identical to
    the FP32 oracle on the single domain."""
    import torch
    wl = bench.WORKLOADS["eqwp_stag"]
    nsteps = 8
    stream = torch.cuda.Stream()
    with bench.make_domain(b2r, wl, stream) as d:
        mat, amps = bench.stag_model(d.domain_shape, d.cfg.dt, nsteps)
        for name, arr in zip(("lambda", "mu", "buoy"), mat):
            d.upload(arr, field=name)
        rng = np.random.default_rng(12)
        init = []
        for k in range(9):
            f = np.zeros(d.domain_shape, np.float32)
            f[4:-4, 4:-4, 4:-4] = ((rng.random(tuple(s - 8 for s in f.shape), dtype=np.float32) - 0.5) *
                                   (1e-3 if k < 3 else 1e5))
            init.append(f)
            d.upload(f, field=k)
        d.set_source(amps)
        knobs, _ = d.autotune(trial_steps=2)
        for k in range(9):
            d.upload(init[k], field=k)
        d.step(nsteps)
        got = [d.download(field=k) for k in range(9)]
        d.synchronize()
        dt, h = d.cfg.dt, d.cfg.h
        src = tuple(int(s) + 2 for s in d.cfg.src)      # the domain array carries a 2-cell shell
    f32 = [a.copy() for a in init]
    for t in range(nsteps):
        orc.eqwp_stag_step(f32, mat, dt, h, 0, 2, 63, src, float(amps[t]))
    for k in range(9):
        assert np.array_equal(got[k], f32[k]), f"field {k} ({knobs})"
    # the FP32 scheme's distance from the FP64 one, for the record
    f64 = [a.astype(np.float64) for a in init]
    m64 = [m.astype(np.float64) for m in mat]
    for t in range(nsteps):
        orc.eqwp_stag_step(f64, m64, dt, h, 0, 2, 63, src, float(amps[t]))
    r64 = max(rel_l2(got[k], f64[k]) for k in range(9))
    print(f"eqwp_stag 512x512x256 x{nsteps} ({knobs}): bit-identical to FP32 oracle, max rel-L2 vs FP64 {r64:.2e}")
    assert r64 <= TOL
