"""Game of Life against the reference's own CUDA kernel (gol_3d_kernel,
gol-3D.cu:30-102, compiled unmodified into oracle/_ref/gol_ref.cubin) inside
its envelope: one 32 x 32 tile in x and y, one generation per launch, a
fixed shell.  Integer work: bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("env,ngen", [((30, 30, 40), 12), ((17, 25, 9), 7), ((30, 8, 64), 20)])
def test_gol_matches_reference_kernel(b2r, orc, env, ngen):
    from oracle import refgpu
    if not refgpu.gol_available():
        pytest.skip("oracle/_ref/gol_ref.cubin not built (the reference source tree was absent at build time)")
    rng = np.random.default_rng(31)
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.uint8)
    dom[1:-1, 1:-1, 1:-1] = (rng.random(env[::-1]) < 0.3).astype(np.uint8)
    dom[0] = 1                                  # a live shell face
    ref = refgpu.run_reference_gol(dom, ngen)
    with b2r.Domain(b2r.MODEL_GOL, env, D=1, R=1) as d:
        d.upload(dom)
        d.step(ngen)
        got = d.download()
        d.synchronize()
    assert np.array_equal(got, ref)
    a, b = dom.copy(), dom.copy()
    for _ in range(ngen):
        orc.gol_substep(a, b, 0, 1, 63)
        a, b = b, a
    assert np.array_equal(a, ref)
