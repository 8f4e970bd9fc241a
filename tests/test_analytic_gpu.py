"""Analytic checks of the schemes on the GPU: the decay of a discrete
Fourier mode under the delta-1 heat step, and bounded energy of the
staggered elastic wave at half the CFL limit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("env,blocks,R", [((40, 30, 50), (1, 1, 1), 1), ((48, 32, 40), (2, 2, 2), 3)])
def test_heat_fourier_mode_decays_at_the_discrete_rate(b2r, env, blocks, R):
    """u = prod_a sin(pi x_a / (N_a + 1)) is an eigenvector of the delta-1
    step with the zero shell: each step multiplies it by
    1 + c sum_a (2 cos(pi / (N_a + 1)) - 2)."""
    c, nsteps = 0.1, 60
    axes = []
    for n in env:
        x = np.arange(n + 2, dtype=np.float64)
        axes.append(np.sin(np.pi * x / (n + 1)))
    u0 = axes[2][:, None, None] * axes[1][None, :, None] * axes[0][None, None, :]
    u0[0] = u0[-1] = 0.0
    u0[:, 0] = u0[:, -1] = 0.0
    u0[:, :, 0] = u0[:, :, -1] = 0.0
    lam = 1.0 + c * sum(2.0 * np.cos(np.pi / (n + 1)) - 2.0 for n in env)
    with b2r.Domain(b2r.MODEL_HEAT, env, blocks=blocks, R=R, D=1, alpha_dt=c) as d:
        d.upload(u0.astype(np.float32))
        d.step(nsteps)
        got = d.download().astype(np.float64)
        d.synchronize()
    want = lam ** nsteps * u0
    r = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    print(f"mode decay {lam ** nsteps:.6f} after {nsteps} steps: rel-L2 {r:.2e}")
    assert r <= 1e-5


def test_staggered_energy_bounded_at_half_cfl(b2r):
    """Random wavefield, homogeneous medium, rigid (zero) shell, no source:
    over 600 steps at half the CFL limit the energy stays within a constant
    of its start and nothing overflows."""
    env, h = (48, 40, 44), 10.0
    vp, rho = 3000.0, 2400.0
    mu = rho * (vp / np.sqrt(3.0)) ** 2
    lam = rho * vp ** 2 - 2 * mu
    dt = 0.5 * h / (vp * np.sqrt(3.0) * (9 / 8 + 1 / 24))
    rng = np.random.default_rng(17)
    with b2r.Domain(b2r.MODEL_EQWP_STAG, env, D=2, R=1, dt=dt, h=h, src=(24, 20, 22)) as d:
        shape = d.domain_shape
        for name, v in (("lambda", lam), ("mu", mu), ("buoy", 1 / rho)):
            d.upload(np.full(shape, v, np.float32), field=name)
        init = []
        for k in range(9):
            a = np.zeros(shape, np.float32)
            scale = 1e-3 if k < 3 else 1e5
            a[2:-2, 2:-2, 2:-2] = ((rng.random(env[::-1]) - 0.5) * scale).astype(np.float32)
            d.upload(a, field=k)
            init.append(a.astype(np.float64))

        def energy(f):
            kin = 0.5 * rho * sum(float(np.sum(f[k] ** 2)) for k in range(3))
            pot = 0.5 * sum(float(np.sum(f[k] ** 2)) for k in range(3, 9)) / (lam + 2 * mu)
            return kin + pot

        e0 = energy(init)
        worst = 1.0
        for _ in range(6):
            d.step(100)
            f = [d.download(field=k).astype(np.float64) for k in range(9)]
            assert all(np.isfinite(a).all() for a in f)
            worst = max(worst, energy(f) / e0)
        d.synchronize()
    print(f"largest energy ratio over 600 steps: {worst:.3f}")
    assert worst <= 2.0
