"""CPU checks of the oracle's heat adjoint (FP64): dot-product test of the
transposed stencil and central finite differences of the conductivity
gradient."""
import numpy as np
import pytest


def setup(D, env=(14, 12, 10), nsteps=9, nrec=6, seed=5):
    rng = np.random.default_rng(seed)
    shape = tuple(e + 2 * D for e in env[::-1])
    u0 = np.zeros(shape)
    u0[D:-D, D:-D, D:-D] = rng.random(env[::-1])
    kappa = 1.0 + 0.3 * rng.random(shape)
    rec = [(int(rng.integers(D, env[0] + D)), int(rng.integers(D, env[1] + D)), int(rng.integers(D, env[2] + D)))
           for _ in range(nrec)]
    return u0, kappa, rec, nsteps


@pytest.mark.parametrize("D", [1, 3])
def test_heat_adjoint_dot_product(orc, D):
    u0, kappa, rec, nsteps = setup(D)
    w = orc.heat_lap_weights(D, 0.05, 1.0, 1.0, 1.0)
    rng = np.random.default_rng(2)
    x = np.zeros(u0.shape)
    x[D:-D, D:-D, D:-D] = rng.standard_normal(x[D:-D, D:-D, D:-D].shape)
    _, d = orc.heat_kappa_record(x, kappa, D, w, rec, nsteps)
    # the recording is linear in u^0: <d(x), y> = <x, adjoint(y)>
    yv = rng.standard_normal(d.shape)
    _, _, _, lam = orc.heat_kappa_gradient(x, kappa, D, w, rec, nsteps, d - yv)
    lhs = float(np.sum(d * yv))
    rhs = float(np.sum(x[D:-D, D:-D, D:-D] * lam[D:-D, D:-D, D:-D]))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


@pytest.mark.parametrize("D", [1, 4])
def test_heat_kappa_gradient_finite_differences(orc, D):
    u0, kappa, rec, nsteps = setup(D)
    w = orc.heat_lap_weights(D, 0.05, 1.0, 1.0, 1.0)
    _, d_true = orc.heat_kappa_record(u0, kappa * 1.1, D, w, rec, nsteps)
    J, g, _, _ = orc.heat_kappa_gradient(u0, kappa, D, w, rec, nsteps, d_true)
    rng = np.random.default_rng(3)
    for _ in range(4):
        v = np.zeros(kappa.shape)
        v[D:-D, D:-D, D:-D] = rng.standard_normal(v[D:-D, D:-D, D:-D].shape)
        eps = 1e-5
        Jp = 0.5 * np.sum((orc.heat_kappa_record(u0, kappa + eps * v, D, w, rec, nsteps)[1] - d_true) ** 2)
        Jm = 0.5 * np.sum((orc.heat_kappa_record(u0, kappa - eps * v, D, w, rec, nsteps)[1] - d_true) ** 2)
        fd = (Jp - Jm) / (2 * eps)
        an = float(np.sum(g * v))
        assert abs(fd - an) <= 1e-7 * abs(an)
