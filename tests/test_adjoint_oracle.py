"""CPU checks of the oracle's discrete adjoint (FP64): dot-product test of the
transposed stencils and a central finite-difference check of the gradient."""
import numpy as np

from adjoint_setup import H, layered, problem


def blk(P, rec):
    return [(int(x) + H, int(y) + H, int(z) + H) for x, y, z in rec]


def test_adjoint_dot_product(orc):
    P = problem(env=(20, 18, 16), nsteps=12)
    mat = layered(P["env"])
    shape = mat[0].shape
    rng = np.random.default_rng(1)
    x = [np.zeros(shape) for _ in range(9)]
    for f in x:
        f[H:-H, H:-H, H:-H] = rng.standard_normal(f[H:-H, H:-H, H:-H].shape)
    rec = blk(P, P["rec"])
    zero_amps = np.zeros(P["nsteps"])
    _, d = orc.eqwp_stag_record(x, mat, P["dt"], P["h"], H, (0, 0, 0), zero_amps, rec, P["nsteps"])
    y = rng.standard_normal(d.shape)
    # adjoint of the recording: inject y, run the reverse steps (d_obs = d - y
    # makes the residual exactly y)
    J, g, _, tmp = orc.eqwp_stag_gradient(x, mat, P["dt"], P["h"], H, (0, 0, 0), zero_amps, rec,
                                          P["nsteps"], d - y)
    lhs = float(np.sum(d * y))
    order = [0, 1, 2, 3, 4, 5, 6, 7, 8]   # tmp: vb(3), sb(xx xy xz yy yz zz) = field order
    rhs = sum(float(np.sum(x[k] * tmp[k])) for k in order)
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), 1e-30), (lhs, rhs)


def test_adjoint_gradient_finite_differences(orc):
    P = problem(env=(16, 16, 14), nsteps=25, nrec=8)
    mat = layered(P["env"])
    obs_mat = layered(P["env"], anomaly=0.05)
    shape = mat[0].shape
    zero = [np.zeros(shape) for _ in range(9)]
    rec = blk(P, P["rec"])
    src = tuple(s + H for s in P["src"])
    _, d_obs = orc.eqwp_stag_record(zero, obs_mat, P["dt"], P["h"], H, src, P["amps"], rec, P["nsteps"])
    J, g, _, _ = orc.eqwp_stag_gradient(zero, mat, P["dt"], P["h"], H, src, P["amps"], rec,
                                        P["nsteps"], d_obs)
    rng = np.random.default_rng(5)
    inner = (slice(H, -H),) * 3
    for trial in range(3):
        dm = [np.zeros(shape) for _ in range(3)]
        for k in range(3):
            dm[k][inner] = rng.standard_normal(dm[k][inner].shape)
        # perturb lambda, mu and rho (buoyancy = 1/rho)
        scale = [mat[0][inner].mean(), mat[1][inner].mean(), 1.0 / mat[2][inner].mean()]
        eps = 1e-5
        def J_at(sgn):
            rho = 1.0 / mat[2] + sgn * eps * scale[2] * dm[2]
            m2 = [mat[0] + sgn * eps * scale[0] * dm[0], mat[1] + sgn * eps * scale[1] * dm[1], 1.0 / rho]
            return orc.eqwp_stag_gradient(zero, m2, P["dt"], P["h"], H, src, P["amps"], rec,
                                          P["nsteps"], d_obs)[0]
        fd = (J_at(1) - J_at(-1)) / (2 * eps)
        an = sum(float(np.sum(g[k] * scale[k] * dm[k])) for k in range(3))
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-30), (trial, fd, an)
