"""GPU adjoint of the staggered elastic wave: FP64 oracle gradient, finite
differences through the torch.autograd wrapper, checkpointing invariance."""
import numpy as np
import pytest

from adjoint_setup import H, layered, problem

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def gpu_domain(b2r, P, mat):
    d = b2r.Domain(b2r.MODEL_EQWP_STAG, P["env"], D=2, R=1, dt=P["dt"], h=P["h"], src=P["src"])
    s = 2                               # domain arrays carry a 2-deep shell
    for name, m in zip(("lambda", "mu", "buoy"), mat):
        d.upload(np.ascontiguousarray(m[H - s:m.shape[0] - H + s, H - s:m.shape[1] - H + s,
                                        H - s:m.shape[2] - H + s], np.float32), field=name)
    zero = np.zeros(d.domain_shape, np.float32)
    for k in range(9):
        d.upload(zero, field=k)
    d.set_source(P["amps"])
    return d


def observed(b2r, P):
    with gpu_domain(b2r, P, layered(P["env"], anomaly=0.05)) as d:
        return d.eqwp_record(P["nsteps"], P["rec"])


def test_gradient_matches_fp64_oracle(b2r, orc):
    P = problem(env=(24, 20, 22), nsteps=40)
    d_obs = observed(b2r, P)
    mat = layered(P["env"])
    with gpu_domain(b2r, P, mat) as d:
        J, g, syn = d.eqwp_misfit_gradient(P["nsteps"], P["rec"], d_obs, ckpt_every=9)
    # the oracle in FP64 on the same (float32-rounded) material and data
    m64 = [m.astype(np.float32).astype(np.float64) for m in mat]
    zero = [np.zeros(mat[0].shape) for _ in range(9)]
    rec = [(int(x) + H, int(y) + H, int(z) + H) for x, y, z in P["rec"]]
    src = tuple(c + H for c in P["src"])
    J64, g64, syn64, _ = orc.eqwp_stag_gradient(zero, m64, P["dt"], P["h"], H, src,
                                                P["amps"].astype(np.float64), rec, P["nsteps"],
                                                d_obs.astype(np.float64))
    inner = (slice(H, -H),) * 3
    print(f"J gpu {J:.6e} fp64 {J64:.6e}; synthetic rel {rel_l2(syn, syn64):.2e}")
    assert abs(J - J64) <= 1e-4 * abs(J64)
    assert rel_l2(syn, syn64) <= 1e-5
    for k, name in enumerate(("lambda", "mu", "rho")):
        r = rel_l2(g[k], g64[k][inner])
        print(f"grad {name}: rel-L2 vs FP64 oracle {r:.2e}")
        assert r <= 1e-5, name


def test_gradient_matches_fp64_oracle_64(b2r, orc):
    """The FP64 reference gradient at 64^3 (the differentiated-eqwp check size)."""
    # source at the centre, 64 receivers on the top plane, long enough for
    # the Ricker peak (1.2 / f0 = 178 steps) to reach them
    P = problem(env=(64, 64, 64), nsteps=240, nrec=64)
    d_obs = observed(b2r, P)
    mat = layered(P["env"])
    with gpu_domain(b2r, P, mat) as d:
        J, g, syn = d.eqwp_misfit_gradient(P["nsteps"], P["rec"], d_obs, ckpt_every=50)
    m64 = [m.astype(np.float32).astype(np.float64) for m in mat]
    zero = [np.zeros(m64[0].shape) for _ in range(9)]
    src = tuple(s + H for s in P["src"])
    rec = [(int(x) + H, int(y) + H, int(z) + H) for x, y, z in P["rec"]]
    J64, g64, syn64, _ = orc.eqwp_stag_gradient(zero, m64, P["dt"], P["h"], H, src,
                                                P["amps"].astype(np.float64), rec, P["nsteps"],
                                                d_obs.astype(np.float64))
    inner = (slice(H, -H),) * 3
    print(f"64^3: J gpu {J:.6e} fp64 {J64:.6e}; synthetic rel-L2 {rel_l2(syn, syn64):.2e}")
    assert abs(J - J64) <= 1e-4 * abs(J64)
    assert rel_l2(syn, syn64) <= 1e-5
    for k, name in enumerate(("lambda", "mu", "rho")):
        r = rel_l2(g[k], g64[k][inner])
        print(f"64^3 grad {name}: rel-L2 vs FP64 oracle {r:.2e}")
        assert r <= 1e-5, name


def test_checkpoint_interval_changes_no_bits(b2r):
    P = problem(env=(20, 16, 18), nsteps=30)
    d_obs = observed(b2r, P)
    mat = layered(P["env"])
    res = []
    for k in (0, 7, 30):
        with gpu_domain(b2r, P, mat) as d:
            res.append(d.eqwp_misfit_gradient(P["nsteps"], P["rec"], d_obs, ckpt_every=k))
    for r in res[1:]:
        assert r[0] == res[0][0]
        for a, b in zip(r[1], res[0][1]):
            assert np.array_equal(a, b)


def test_autograd_matches_central_differences(b2r):
    import torch
    from b2r_gb300.autograd import EqwpMisfit
    P = problem(env=(20, 18, 16), nsteps=30)
    P["d_obs"] = observed(b2r, P)
    mat = layered(P["env"])
    inner = (slice(H, -H),) * 3
    lam = torch.tensor(mat[0][inner], requires_grad=True)
    mu = torch.tensor(mat[1][inner], requires_grad=True)
    rho = torch.tensor(1.0 / mat[2][inner], requires_grad=True)
    J = EqwpMisfit.apply(lam, mu, rho, P)
    J.backward()
    rng = np.random.default_rng(11)
    for trial in range(16):
        dirs = [torch.from_numpy(rng.standard_normal(lam.shape)) for _ in range(3)]
        scale = [float(lam.mean()), float(mu.mean()), float(rho.mean())]
        eps = 2e-3
        def J_at(s):
            with torch.no_grad():
                return float(EqwpMisfit.apply(lam + s * eps * scale[0] * dirs[0],
                                              mu + s * eps * scale[1] * dirs[1],
                                              rho + s * eps * scale[2] * dirs[2], P))
        fd = (J_at(1) - J_at(-1)) / (2 * eps)
        an = float(sum((g * sc * dd).sum() for g, sc, dd in
                       zip((lam.grad, mu.grad, rho.grad), scale, dirs)))
        print(f"direction {trial}: FD {fd:.6e} adjoint {an:.6e}")
        # relative to the typical size of a random directional derivative
        gnorm = float(sum(((g * sc) ** 2).sum() for g, sc in
                          zip((lam.grad, mu.grad, rho.grad), scale)) ** 0.5)
        assert abs(fd - an) <= 1e-3 * max(abs(an), gnorm), trial


def test_fused_stress_gradient_sweep_changes_no_bits(b2r):
    """The stress adjoint with the lambda / mu gradients in one sweep and as
    two kernels give the same bits."""
    P = problem(env=(22, 18, 20), nsteps=24)
    d_obs = observed(b2r, P)
    mat = layered(P["env"])
    res = []
    for fused in (1, 0):
        with gpu_domain(b2r, P, mat) as d:
            d.set_tuning(adj_fused=fused)
            assert d.get_tuning()["adj_fused"] == fused
            res.append(d.eqwp_misfit_gradient(P["nsteps"], P["rec"], d_obs, ckpt_every=8))
    assert res[0][0] == res[1][0]
    for a, b in zip(res[0][1], res[1][1]):
        assert np.array_equal(a, b)
