"""GPU adjoint of the conductivity-scaled heat scheme: the FP64 oracle
gradient, checkpoint-interval invariance and central finite differences along
16 random directions (through the torch.autograd wrapper)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
COEF = (0.05, 1.0, 1.0, 1.0)


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def problem(D, env=(40, 36, 32), nsteps=30, nrec=16, seed=4):
    rng = np.random.default_rng(seed)
    shape = tuple(e + 2 * D for e in env[::-1])
    u0 = np.zeros(shape, np.float32)
    u0[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    kappa = (1.0 + 0.3 * rng.random(shape)).astype(np.float32)
    rec = np.stack([rng.integers(0, env[0], nrec), rng.integers(0, env[1], nrec),
                    rng.integers(0, env[2], nrec)], axis=1).astype(np.int32)
    return dict(D=D, env=env, nsteps=nsteps, coef=COEF, u0=u0, kappa=kappa, rec=rec)


def domain(b2r, P, kappa):
    a, dx, dy, dz = P["coef"]
    d = b2r.Domain(b2r.MODEL_HEAT, P["env"], D=P["D"], R=1, alpha_dt=a, dx=dx, dy=dy, dz=dz)
    d.upload(np.ascontiguousarray(kappa, np.float32), field="kappa")
    d.upload(P["u0"])
    return d


def observed(b2r, P):
    with domain(b2r, P, P["kappa"] * np.float32(1.1)) as d:
        return d.heat_record(P["nsteps"], P["rec"])


@pytest.mark.parametrize("D", [1, 2, 4])
def test_heat_gradient_matches_fp64_oracle(b2r, orc, D):
    P = problem(D)
    d_obs = observed(b2r, P)
    with domain(b2r, P, P["kappa"]) as d:
        J, g, syn = d.heat_misfit_gradient(P["nsteps"], P["rec"], d_obs, ckpt_every=7)
    w = orc.heat_lap_weights(D, *COEF)
    rec_blk = [(int(x) + D, int(y) + D, int(z) + D) for x, y, z in P["rec"]]
    J64, g64, syn64, _ = orc.heat_kappa_gradient(P["u0"].astype(np.float64), P["kappa"].astype(np.float64), D, w,
                                                 rec_blk, P["nsteps"], d_obs.astype(np.float64))
    inner = (slice(D, -D),) * 3
    r_syn, r_g = rel_l2(syn, syn64), rel_l2(g, g64[inner])
    print(f"D={D}: J gpu {J:.6e} fp64 {J64:.6e}; synthetic rel-L2 {r_syn:.2e}; gradient rel-L2 {r_g:.2e}")
    assert abs(J - J64) <= 1e-4 * abs(J64)
    assert r_syn <= 1e-5
    assert r_g <= 1e-5


def test_heat_checkpoint_interval_changes_no_bits(b2r):
    P = problem(2, env=(24, 20, 18), nsteps=25)
    d_obs = observed(b2r, P)
    out = []
    for k in (0, 4, 25):
        with domain(b2r, P, P["kappa"]) as d:
            out.append(d.heat_misfit_gradient(P["nsteps"], P["rec"], d_obs, ckpt_every=k))
    for r in out[1:]:
        assert r[0] == out[0][0]
        assert np.array_equal(r[1], out[0][1])


def test_heat_autograd_matches_central_differences(b2r):
    import torch
    from b2r_gb300.autograd import HeatMisfit
    D = 1
    P = problem(D, env=(20, 18, 16), nsteps=20)
    P["d_obs"] = observed(b2r, P)
    inner = (slice(D, -D),) * 3
    kappa = torch.tensor(P["kappa"][inner].astype(np.float64), requires_grad=True)
    J = HeatMisfit.apply(kappa, P)
    J.backward()
    rng = np.random.default_rng(12)
    for trial in range(16):
        v = torch.from_numpy(rng.standard_normal(kappa.shape))
        eps = 1e-3
        with torch.no_grad():
            fd = (float(HeatMisfit.apply(kappa + eps * v, P)) - float(HeatMisfit.apply(kappa - eps * v, P))) / (2 * eps)
        an = float((kappa.grad * v).sum())
        print(f"direction {trial}: FD {fd:.6e} adjoint {an:.6e}")
        # relative to the typical size of a random directional derivative
        # (|g|), so that a direction nearly orthogonal to g is not judged on
        # the FP32 noise of the two forward runs alone
        scale = max(abs(an), float(kappa.grad.norm()))
        assert abs(fd - an) <= 1e-3 * scale, trial
