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


@pytest.mark.parametrize("D,env,nsteps", [(2, (86, 24, 20), 25), (3, (84, 22, 18), 25), (4, (82, 24, 20), 25),
                                          (2, (28, 26, 40), 40), (4, (120, 22, 24), 15)])
def test_heat_high_order_matches_reference_kernels(b2r, D, env, nsteps):
    """fdm_heat_diffuse_delta2..4 (heat-3D.cu:250-521, compiled at B2R_D = D)
    inside their envelope: R = 1, one 32-row tile in y, x tiles whose left
    halo loads all happen.  The library's order-D sweep and the oracle's
    restatement both match them."""
    from oracle import orc, refgpu
    if not refgpu.heat_d_available(D):
        pytest.skip(f"oracle/_ref/heat_ref_d{D}.cubin not built (the reference source tree was absent)")
    rng = np.random.default_rng(50 + D)
    dom = np.zeros(tuple(e + 2 * D for e in env[::-1]), np.float32)
    dom[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    assert refgpu.heat_d_envelope(dom.shape, D)
    ref = refgpu.run_reference_heat_d(dom, D, nsteps)
    with b2r.Domain(b2r.MODEL_HEAT, env, D=D, R=1, alpha_dt=0.01, dx=1.0, dy=1.0, dz=0.5) as d:
        d.upload(dom)
        d.step(nsteps)
        got = d.download()
        d.synchronize()
    o = dom.copy()
    orc.heat_run(o, D, D, nsteps, 0.01, 1.0, 1.0, 0.5)
    r = float(np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref.astype(np.float64)))
    ro = float(np.linalg.norm(o.astype(np.float64) - ref) / np.linalg.norm(ref.astype(np.float64)))
    print(f"delta{D} {env} x{nsteps}: library {r:.2e}, oracle {ro:.2e} rel-L2 vs the reference kernel")
    assert r <= 1e-5 and ro <= 1e-5


@pytest.mark.parametrize("shape,R,ef", [((40, 50, 70), 3, (-1, 0, 1)), ((36, 45, 66), 2, (1, -1, 0)),
                                        ((34, 70, 100), 4, (-1, 1, -1)), ((30, 40, 50), 1, (0, 0, 0))])
def test_heat_edge_flags_match_reference_verify_kernel(b2r, shape, R, ef):
    """fdm_heat_diffuse_delta1_verify (heat-3D.cu:57-158), the reference's
    edge-flag kernel, driven as heat_3D_gpu_main (heat-3D.cu:583-637) with
    b2r_i = 0..R-1, against b2r_heat_3D_gpu_main with the same flags: the
    fixed-shell semantics of the library are the reference's own."""
    from oracle import refgpu
    if not refgpu.heat_available():
        pytest.skip("oracle/_ref/heat_ref.cubin not built (the reference source tree was absent)")
    blk = np.random.default_rng(60 + R).random(shape, dtype=np.float32)
    ref = refgpu.run_reference_heat_verify(blk, R, ef)
    got = blk.copy()
    b2r.heat_3D_gpu_main(got, R, D=1, edge_flag=ef)
    r = float(np.linalg.norm(got.astype(np.float64) - ref) / np.linalg.norm(ref.astype(np.float64)))
    print(f"verify {shape} R={R} ef={ef}: rel-L2 {r:.2e}")
    assert r <= 1e-5
    assert np.array_equal(got[:R], blk[:R]) and np.array_equal(got[-R:], blk[-R:])
