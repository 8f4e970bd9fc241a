"""GPU elastic-wave models against the oracle (relative L2 <= 1e-5)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5
NAMES = ["vx", "vy", "vz", "sxx", "sxy", "sxz", "syy", "syz", "szz", "disp"]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def ref_force(env, shell=2):
    """Force patch of eqwp.cu:135,561-566 (reference block Ng = B+4, R = 1),
    in domain-array coordinates with a `shell`-deep shell."""
    ngx, ngz = env[0] + 4, env[2] + 4
    return dict(fy=shell + env[1] - 7, fx0=shell + ngx // 2 - 2, fx1=shell + ngx // 2 + ngx // 10 - 2,
                fz0=shell + ngz // 2 - 2, fz1=shell + ngz // 2 + ngz // 10 - 2, fval=-1e4, fsteps=50)


@pytest.mark.parametrize("env", [(40, 32, 24), (70, 20, 33)])
def test_eqwp_ref_matches_oracle(b2r, orc, env):
    nsteps = 30
    shape = tuple(e + 4 for e in env[::-1])
    rng = np.random.default_rng(3)
    init = [np.zeros(shape, np.float32) for _ in range(10)]
    for k in range(9):   # small random start so every term is exercised
        init[k][2:-2, 2:-2, 2:-2] = ((rng.random(env[::-1]) - 0.5) * 1e-2).astype(np.float32)
    with b2r.Domain(b2r.MODEL_EQWP_REF, env, D=2, R=1) as d:
        for k in range(10):
            d.upload(init[k], field=k)
        d.step(nsteps)
        got = [d.download(field=k) for k in range(10)]
        d.synchronize()
    ref = [a.copy() for a in init]
    ref64 = [a.astype(np.float64) for a in init]
    force = ref_force(env)
    for ts in range(nsteps):
        orc.eqwp_ref_substep(ref, 0, 2, 63, ts, force)
        orc.eqwp_ref_substep(ref64, 0, 2, 63, ts, force)
    for k in range(10):
        r32, r64 = rel_l2(got[k], ref[k]), rel_l2(got[k], ref64[k])
        print(f"{NAMES[k]}: rel-L2 vs oracle FP32 {r32:.2e}, vs FP64 {r64:.2e}")
        assert r32 <= TOL, NAMES[k]


def layered(env, seed=3, layers=8):
    """8 horizontal layers (along y): vp U[2000,4000], vs = vp/sqrt(3), rho U[2000,2600]."""
    rng = np.random.default_rng(seed)
    vp_l = rng.uniform(2000, 4000, layers)
    rho_l = rng.uniform(2000, 2600, layers)
    ny = env[1] + 4
    idx = np.minimum(np.arange(ny) * layers // ny, layers - 1)
    shape = tuple(e + 4 for e in env[::-1])
    vp = np.broadcast_to(vp_l[idx][None, :, None], shape)
    rho = np.broadcast_to(rho_l[idx][None, :, None], shape)
    vs = vp / np.sqrt(3.0)
    mu = rho * vs ** 2
    lam = rho * vp ** 2 - 2 * mu
    return [np.ascontiguousarray(m, np.float64) for m in (lam, mu, 1.0 / rho)]


def ricker(n, dt, f0, amp):
    t = np.arange(n) * dt - 1.2 / f0
    a = (np.pi * f0 * t) ** 2
    return amp * (1 - 2 * a) * np.exp(-a)


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("blocks,R", [((1, 1, 1), 1), ((2, 2, 1), 2), ((2, 1, 2), 1)])
def test_eqwp_stag_matches_oracle(b2r, orc, blocks, R, fused):
    env = (48, 40, 32)
    nsteps = 40
    h = 10.0
    mat = layered(env)
    dt = 0.5 * h / (4000 * np.sqrt(3) * (9 / 8 + 1 / 24))
    src = (env[0] // 2, env[1] // 2, env[2] // 2)
    amps = ricker(nsteps, dt, 10.0, 1e6 * dt).astype(np.float32)
    with b2r.Domain(b2r.MODEL_EQWP_STAG, env, blocks=blocks, R=R, D=2, dt=dt, h=h, src=src) as d:
        d.set_tuning(eqwp_fused=fused)
        for m, name in enumerate(["lambda", "mu", "buoy"]):
            d.upload(mat[m].astype(np.float32), field=name)
        zero = np.zeros(d.domain_shape, np.float32)
        for k in range(9):
            d.upload(zero, field=k)
        d.set_source(amps)
        d.step(nsteps)
        got = [d.download(field=k) for k in range(9)]
        d.synchronize()
    f = [np.zeros(zero.shape, np.float32) for _ in range(9)]
    f64 = [np.zeros(zero.shape, np.float64) for _ in range(9)]
    m32 = [np.ascontiguousarray(m.astype(np.float32)) for m in mat]
    sc = tuple(s + 2 for s in src)
    for t in range(nsteps):
        orc.eqwp_stag_step(f, m32, dt, h, 0, 2, 63, sc, float(amps[t]))
        orc.eqwp_stag_step(f64, mat, dt, h, 0, 2, 63, sc, float(amps[t]))
    for k in range(9):
        r32, r64 = rel_l2(got[k], f[k]), rel_l2(got[k], f64[k])
        print(f"{NAMES[k]} blocks={blocks} R={R}: vs FP32 {r32:.2e}, vs FP64 {r64:.2e}")
        assert r32 <= TOL, NAMES[k]
        # every operation is rounded as the FP32 oracle rounds it
        assert np.array_equal(got[k], f[k]), NAMES[k]


@pytest.mark.parametrize("env,blocks,R", [((150, 90, 70), (3, 2, 1), 2), ((97, 61, 131), (1, 1, 1), 1),
                                          ((64, 64, 64), (2, 2, 2), 3), ((260, 33, 17), (2, 1, 1), 1),
                                          ((40, 120, 90), (1, 2, 3), 2)])
def test_eqwp_stag_tma_stress_equals_plain(b2r, env, blocks, R):
    """The stress stage with TMA-streamed inputs against the plain-load
    stage (two-pass step both), on sizes that leave ragged tiles, short z
    chunks and several blocks, with the source switched on."""
    nsteps = 2 * R + 1
    h = 10.0
    mat = layered(env)
    dt = 0.5 * h / (4000 * np.sqrt(3) * (9 / 8 + 1 / 24))
    src = (env[0] // 3, env[1] // 2, env[2] // 2)
    amps = ricker(nsteps, dt, 10.0, 1e6 * dt).astype(np.float32)
    outs = []
    for tma in (0, 1):
        with b2r.Domain(b2r.MODEL_EQWP_STAG, env, blocks=blocks, R=R, D=2, dt=dt, h=h, src=src) as d:
            d.set_tuning(eqwp_fused=0, eqwp_tma=tma)
            for m, name in enumerate(["lambda", "mu", "buoy"]):
                d.upload(mat[m].astype(np.float32), field=name)
            rng = np.random.default_rng(12)
            for k in range(9):
                d.upload(rng.standard_normal(d.domain_shape).astype(np.float32), field=k)
            d.set_source(amps)
            d.step(nsteps)
            outs.append([d.download(field=k) for k in range(9)])
            d.synchronize()
    for k in range(9):
        assert np.array_equal(outs[0][k], outs[1][k]), NAMES[k]


@pytest.mark.parametrize("env,blocks,R", [((150, 90, 70), (3, 2, 1), 2), ((97, 61, 131), (1, 1, 1), 1),
                                          ((64, 64, 64), (2, 2, 2), 3)])
def test_eqwp_stag_one_pass_equals_two_pass(b2r, env, blocks, R):
    """The one-pass step against the two stage kernels, on sizes that leave
    ragged tiles and z chunks; both round every operation the same way."""
    nsteps = 2 * R + 1
    h = 10.0
    mat = layered(env)
    dt = 0.5 * h / (4000 * np.sqrt(3) * (9 / 8 + 1 / 24))
    src = (env[0] // 3, env[1] // 2, env[2] // 2)
    amps = ricker(nsteps, dt, 10.0, 1e6 * dt).astype(np.float32)
    rng = np.random.default_rng(11)
    outs = []
    for fused in (False, True):
        with b2r.Domain(b2r.MODEL_EQWP_STAG, env, blocks=blocks, R=R, D=2, dt=dt, h=h, src=src) as d:
            d.set_tuning(eqwp_fused=fused)
            for m, name in enumerate(["lambda", "mu", "buoy"]):
                d.upload(mat[m].astype(np.float32), field=name)
            rng = np.random.default_rng(11)
            for k in range(9):
                d.upload(rng.standard_normal(d.domain_shape).astype(np.float32), field=k)
            d.set_source(amps)
            d.step(nsteps)
            outs.append([d.download(field=k) for k in range(9)])
            d.synchronize()
    for k in range(9):
        assert np.array_equal(outs[0][k], outs[1][k]), NAMES[k]


@pytest.mark.parametrize("env,blocks,R", [((150, 90, 70), (3, 2, 1), 2), ((64, 64, 64), (2, 2, 2), 3),
                                          ((96, 40, 120), (2, 1, 3), 1), ((40, 120, 90), (1, 2, 3), 2)])
def test_eqwp_stag_overlapped_exchange_bit_identical(b2r, orc, env, blocks, R):
    """The next period's halo exchange issued inside the period's last
    stress stage (band tiles first, the exchange on a second stream, the
    other tiles meanwhile) against the exchange at the period start: the
    same bits, stepping whole runs and in pieces that split periods, with an
    upload in between (whose scatter fills the halos itself)."""
    h = 10.0
    mat = layered(env)
    dt = 0.5 * h / (4000 * np.sqrt(3) * (9 / 8 + 1 / 24))
    src = (env[0] // 3, env[1] // 2, env[2] // 2)
    nsteps = 4 * R + 1
    amps = ricker(2 * nsteps, dt, 10.0, 1e6 * dt).astype(np.float32)
    outs = []
    for overlap in (0, 1):
        with b2r.Domain(b2r.MODEL_EQWP_STAG, env, blocks=blocks, R=R, D=2, dt=dt, h=h, src=src) as d:
            d.set_tuning(eqwp_fused=0, eqwp_tma=0, eqwp_overlap=overlap)
            assert d.get_tuning()["eqwp_overlap"] == overlap
            for m, name in enumerate(["lambda", "mu", "buoy"]):
                d.upload(mat[m].astype(np.float32), field=name)
            rng = np.random.default_rng(21)
            for k in range(9):
                d.upload(rng.standard_normal(d.domain_shape).astype(np.float32), field=k)
            d.set_source(amps)
            d.step(nsteps)
            mid = d.download(field=4)
            d.upload(mid, field=4)
            for n in (1, R, 2, 1):
                d.step(n)
            outs.append([d.download(field=k) for k in range(9)])
            d.synchronize()
    for k in range(9):
        assert np.array_equal(outs[0][k], outs[1][k]), NAMES[k]


@pytest.mark.parametrize("env,blocks,R,overlap", [((48, 40, 32), (1, 1, 1), 1, 0), ((48, 40, 32), (2, 2, 1), 2, 0),
                                                  ((48, 40, 32), (2, 2, 1), 2, 1), ((64, 48, 40), (2, 1, 2), 1, 1)])
def test_eqwp_stag_periodic_matches_torus_oracle(b2r, orc, env, blocks, R, overlap):
    """The staggered model on a torus (every axis wraps; one block exchanges
    with itself) against the float64 torus restatement of the scheme, with
    the exchange at the period start or overlapped with the last stress
    stage."""
    nsteps = 12
    h = 10.0
    # the layered model without its shell: a periodic domain has none
    mat = [np.ascontiguousarray(m[2:-2, 2:-2, 2:-2]) for m in layered(env)]
    dt = 0.5 * h / (4000 * np.sqrt(3) * (9 / 8 + 1 / 24))
    src = (env[0] // 3, env[1] // 2, env[2] // 2)
    amps = ricker(nsteps, dt, 10.0, 1e6 * dt).astype(np.float32)
    rng = np.random.default_rng(41)
    init = [(rng.standard_normal(env[::-1]) * 1e-3).astype(np.float32) for _ in range(9)]
    with b2r.Domain(b2r.MODEL_EQWP_STAG, env, blocks=blocks, R=R, D=2, dt=dt, h=h, src=src,
                    boundary=b2r.BC_PERIODIC) as d:
        d.set_tuning(eqwp_fused=0, eqwp_tma=0, eqwp_overlap=overlap)
        assert d.domain_shape == env[::-1]
        for m, name in enumerate(["lambda", "mu", "buoy"]):
            d.upload(mat[m].astype(np.float32), field=name)
        for k in range(9):
            d.upload(init[k], field=k)
        d.set_source(amps)
        d.step(nsteps)
        got = [d.download(field=k) for k in range(9)]
        d.synchronize()
    ref = orc.eqwp_stag_run_periodic(init, [m.astype(np.float32) for m in mat], float(np.float32(dt)),
                                     float(np.float32(h)), [float(a) for a in amps], src)
    for k in range(9):
        r = rel_l2(got[k], ref[k])
        print(f"{NAMES[k]} periodic blocks={blocks} R={R} overlap={overlap}: vs FP64 torus {r:.2e}")
        assert r <= TOL, NAMES[k]
