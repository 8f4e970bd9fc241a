"""The reference model of the elastic wave against the reference's own CUDA
kernels (eqwp.cu:60-477, compiled unmodified into oracle/_ref/eqwp_ref.cubin
and run through the driver API), inside their envelope: R = 1, one block of
at most 16 rows in y.  Relative L2 <= 1e-5 per field, as for the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
NAMES = ["vx", "vy", "vz", "sxx", "sxy", "sxz", "syy", "syz", "szz", "disp"]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("env,nsteps", [((40, 12, 24), 60), ((27, 11, 30), 20)])
def test_ref_model_matches_reference_kernels(b2r, env, nsteps):
    from oracle import refgpu
    if not refgpu.available():
        pytest.skip("oracle/_ref/eqwp_ref.cubin not built (the reference source tree was absent at build time)")
    shape = tuple(e + 4 for e in env[::-1])          # the reference block Ng = B + 2*B2R_D*R
    assert shape[1] <= refgpu.TILE
    rng = np.random.default_rng(21)
    init = [np.zeros(shape, np.float32) for _ in range(10)]
    for k in range(9):
        init[k][2:-2, 2:-2, 2:-2] = ((rng.random(env[::-1]) - 0.5) * 1e-2).astype(np.float32)
    ref = refgpu.run_reference(init, nsteps)
    with b2r.Domain(b2r.MODEL_EQWP_REF, env, D=2, R=1) as d:
        for k in range(10):
            d.upload(init[k], field=k)
        d.step(nsteps)
        got = [d.download(field=k) for k in range(10)]
        d.synchronize()
    worst = 0.0
    for k in range(10):
        r = rel_l2(got[k], ref[k])
        same = float(np.mean(got[k] == ref[k]))
        print(f"{NAMES[k]}: rel-L2 vs the reference kernels {r:.2e}, identical cells {100 * same:.1f} %")
        worst = max(worst, r)
        assert np.abs(ref[k]).max() > 0
    assert worst <= 1e-5


def test_oracle_restatement_matches_reference_kernels(orc):
    """The oracle's FP32 restatement of the reference model (used by every
    other elastic-wave test) against the reference's own kernels."""
    from oracle import refgpu
    if not refgpu.available():
        pytest.skip("oracle/_ref/eqwp_ref.cubin not built (the reference source tree was absent at build time)")
    env, nsteps = (27, 11, 30), 20
    shape = tuple(e + 4 for e in env[::-1])
    rng = np.random.default_rng(22)
    init = [np.zeros(shape, np.float32) for _ in range(10)]
    for k in range(9):
        init[k][2:-2, 2:-2, 2:-2] = ((rng.random(env[::-1]) - 0.5) * 1e-2).astype(np.float32)
    ref = refgpu.run_reference(init, nsteps)
    ngx, ngz = shape[2], shape[0]
    force = dict(fy=shape[1] - 7 - 2, fx0=ngx // 2, fx1=ngx // 2 + ngx // 10, fz0=ngz // 2,
                 fz1=ngz // 2 + ngz // 10, fval=-1e4, fsteps=50)   # eqwp.cu:131,561-566 in block coordinates
    o = [a.copy() for a in init]
    for ts in range(nsteps):
        orc.eqwp_ref_substep(o, 0, 2, 63, ts, force)
    for k in range(10):
        r = rel_l2(o[k], ref[k])
        print(f"{NAMES[k]}: oracle vs the reference kernels rel-L2 {r:.2e}")
        assert r <= 1e-5, NAMES[k]

