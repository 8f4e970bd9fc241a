"""GPU B2R boundary update between resident subdomains vs the numpy oracle
of the X->Y->Z exchange (b2r_halo_sync.cu)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model,env,blocks,R,D,periodic", [
    (1, (48, 40, 56), (2, 2, 2), 2, 1, False),
    (1, (48, 40, 56), (3, 2, 1), 1, 3, True),
    (2, (40, 40, 60), (2, 2, 3), 4, 1, True),
    (2, (36, 24, 24), (3, 1, 2), 2, 1, False),
])
@pytest.mark.parametrize("staged", [False, True])
def test_boundary_updating_matches_oracle(b2r, orc, model, env, blocks, R, D, periodic, staged):
    bc = b2r.BC_PERIODIC if periodic else b2r.BC_SHELL
    with b2r.Domain(model, env, blocks=blocks, R=R, D=D, boundary=bc, alpha_dt=0.05) as d:
        rng = np.random.default_rng(1)
        if d.dtype == np.uint8:
            dom = (rng.random(d.domain_shape) < 0.4).astype(np.uint8)
        else:
            dom = rng.random(d.domain_shape, dtype=np.float32)
        d.upload(dom)
        d.step(R)                       # one period: halos are now stale
        before = d.download_blocks()
        if staged:
            d.boundary_updating(R, 0)
        else:
            d.boundary_updating_direct(R, 0)
        after = d.download_blocks()
        d.synchronize()
    ref = {k: v.copy() for k, v in before.items()}
    orc.halo_exchange(ref, blocks, d.halo, periodic=periodic)
    for k in ref:
        assert np.array_equal(after[k], ref[k]), k


def test_upload_fills_halos_like_exchange(b2r, orc):
    env, blocks, R = (32, 24, 40), (2, 2, 2), 3
    rng = np.random.default_rng(4)
    dom = (rng.random(env[::-1]) < 0.5).astype(np.uint8)
    with b2r.Domain(b2r.MODEL_GOL, env, blocks=blocks, R=R, boundary=b2r.BC_PERIODIC) as d:
        d.upload(dom)
        got = d.download_blocks()
    ref = orc.split_blocks(dom, blocks, R, periodic=True)
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("model,env,blocks,R,D,periodic", [
    (1, (24, 16, 20), (2, 2, 2), 4, 1, False),    # R*D = min(B)/2 = 4
    (1, (32, 16, 24), (2, 2, 2), 2, 2, True),     # R*D = 4 = 8/2
    (2, (32, 32, 32), (2, 2, 2), 8, 1, True),     # R = 8 = 16/2
])
def test_boundary_updating_at_the_halo_limit(b2r, orc, model, env, blocks, R, D, periodic):
    """Halos as deep as b2r.cpp:54 allows (R*D = min(B)/2), non-cubic."""
    bc = b2r.BC_PERIODIC if periodic else b2r.BC_SHELL
    with b2r.Domain(model, env, blocks=blocks, R=R, D=D, boundary=bc, alpha_dt=0.05) as d:
        rng = np.random.default_rng(2)
        if d.dtype == np.uint8:
            dom = (rng.random(d.domain_shape) < 0.4).astype(np.uint8)
        else:
            dom = rng.random(d.domain_shape, dtype=np.float32)
        d.upload(dom)
        d.step(R)
        before = d.download_blocks()
        d.boundary_updating_direct(R, 0)
        after = d.download_blocks()
        d.synchronize()
    ref = {k: v.copy() for k, v in before.items()}
    orc.halo_exchange(ref, blocks, d.halo, periodic=periodic)
    for k in ref:
        assert np.array_equal(after[k], ref[k]), k
