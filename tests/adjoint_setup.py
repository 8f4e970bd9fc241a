"""Shared set-up of the adjoint tests: a small layered elastic model with a
Gaussian anomaly, an explosive Ricker source and receivers on the top plane
(the shape of the differentiated-eqwp benchmark case, scaled down)."""
import numpy as np

H = 4          # halo / fixed-shell depth of a single block with R = 1


def layered(env, seed=3, layers=8, anomaly=0.0, sigma=None):
    """lambda, mu, buoyancy on the padded block (z, y, x), FP64."""
    rng = np.random.default_rng(seed)
    vp_l = rng.uniform(2000, 4000, layers)
    rho_l = rng.uniform(2000, 2600, layers)
    shape = tuple(e + 2 * H for e in env[::-1])
    ny = shape[1]
    idx = np.minimum(np.arange(ny) * layers // ny, layers - 1)
    vp = np.broadcast_to(vp_l[idx][None, :, None], shape).copy()
    rho = np.broadcast_to(rho_l[idx][None, :, None], shape).copy()
    if anomaly:
        z, y, x = np.meshgrid(*[np.arange(s, dtype=np.float64) for s in shape], indexing="ij")
        c = [s / 2 for s in shape]
        sg = sigma or min(env) / 6
        gauss = np.exp(-((z - c[0]) ** 2 + (y - c[1]) ** 2 + (x - c[2]) ** 2) / (2 * sg * sg))
        vp *= 1 + anomaly * gauss
    vs = vp / np.sqrt(3.0)
    mu = rho * vs ** 2
    lam = rho * vp ** 2 - 2 * mu
    return [np.ascontiguousarray(lam), np.ascontiguousarray(mu), np.ascontiguousarray(1.0 / rho)]


def problem(env=(24, 20, 22), nsteps=40, nrec=12, f0=12.0, h=10.0, seed=7):
    dt = 0.5 * h / (4400 * np.sqrt(3) * (9 / 8 + 1 / 24))
    src = (env[0] // 2, env[1] // 2, env[2] // 2)              # global interior coordinates
    rng = np.random.default_rng(seed)
    rec = np.stack([rng.integers(2, env[0] - 2, nrec), np.full(nrec, 2),
                    rng.integers(2, env[2] - 2, nrec)], axis=1).astype(np.int32)
    t = np.arange(nsteps) * dt - 1.2 / f0
    a = (np.pi * f0 * t) ** 2
    amps = 1e7 * dt * (1 - 2 * a) * np.exp(-a)
    return dict(env=env, nsteps=nsteps, dt=dt, h=h, src=src, rec=rec, amps=amps.astype(np.float32))
