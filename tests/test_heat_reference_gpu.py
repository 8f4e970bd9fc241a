"""Heat delta 1 against the reference's own CUDA kernel
(fdm_heat_diffuse_delta1, heat-3D.cu:173-235, compiled unmodified into
oracle/_ref/heat_ref.cubin): several 32 x 32 tiles, R = 1, the reference's
constants.  FP32 work: relative L2 <= 1e-5 (the kernel weights in double)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("env,nsteps", [((70, 50, 40), 30), ((128, 128, 128), 100)])
def test_heat_matches_reference_kernel(b2r, env, nsteps):
    from oracle import refgpu
    if not refgpu.heat_available():
        pytest.skip("oracle/_ref/heat_ref.cubin not built (the reference source tree was absent at build time)")
    rng = np.random.default_rng(41)
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.float32)
    dom[1:-1, 1:-1, 1:-1] = rng.random(env[::-1], dtype=np.float32)
    ref = refgpu.run_reference_heat(dom, nsteps)
    with b2r.Domain(b2r.MODEL_HEAT, env, D=1, R=1, alpha_dt=0.01, dx=1.0, dy=1.0, dz=0.5) as d:
        d.upload(dom)
        d.step(nsteps)
        got = d.download()
        d.synchronize()
    r = float(np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref.astype(np.float64)))
    same = float(np.mean(got == ref))
    print(f"heat {env} x{nsteps}: rel-L2 vs the reference kernel {r:.2e}, identical cells {100 * same:.1f} %")
    assert r <= 1e-5
