"""CPU tests of the oracle: pinned to the reference, then used as the reference
for the GPU tests.

* bit-exact against the golden fixtures produced by the reference's own
  heat_3D_cpu_main (tests/golden/gen_golden.py);
* bit-exact against the compiled reference where its source tree is present;
* the B2R restructuring (subdomains + X->Y->Z halo exchange + shrinking
  windows) reproduces the single-domain result bit for bit;
* Game of Life known-answer cases built from the rule text of gol-3D.cu:104-117.
"""
import hashlib
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_oracle_matches_reference_small_fixture(orc):
    g = np.load(os.path.join(GOLD, "heat_d1_small.npz"))
    a = g["in_shell"].copy()
    for _ in range(10):
        orc.heat_cpu_main(a, 1, 1, **orc.REF_HEAT)
    assert np.array_equal(a, g["out_r1x10"])
    for R, key in ((2, "out_r2"), (3, "out_r3")):
        b = g["in_rand"].copy()
        orc.heat_cpu_main(b, R, 1, **orc.REF_HEAT)
        assert np.array_equal(b, g[key]), f"R={R}"


def test_oracle_matches_reference_128_checksum(orc):
    meta = json.load(open(os.path.join(GOLD, "heat_d1_cfg128.json")))
    n = meta["storage"]
    a = np.zeros(n[::-1], np.float32)
    rng = np.random.default_rng(meta["seed"])
    a[1:-1, 1:-1, 1:-1] = rng.random((n[2] - 2, n[1] - 2, n[0] - 2), dtype=np.float32)
    assert hashlib.sha256(a.tobytes()).hexdigest() == meta["sha256_in"]
    orc.heat_run(a, 1, 1, meta["steps"], meta["alpha_dt"], meta["dx"], meta["dy"], meta["dz"])
    assert hashlib.sha256(a.tobytes()).hexdigest() == meta["sha256_out"]
    for k, v in meta["samples"].items():
        z, y, x = map(int, k.split(","))
        assert float(a[z, y, x]) == v


@pytest.mark.parametrize("shape,R", [((17, 23, 31), 1), ((20, 16, 12), 2), ((26, 22, 18), 4)])
def test_oracle_matches_compiled_reference(orc, shape, R):
    if orc.ref_lib() is None:
        pytest.skip("reference source tree not present on this host")
    rng = np.random.default_rng(sum(shape) + R)
    a = rng.random(shape, dtype=np.float32)
    b = a.copy()
    orc.ref_heat_cpu_main(a, R, 2)
    orc.heat_cpu_main(b, R, 1, **orc.REF_HEAT, nthreads=2)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("D", [1, 2, 3, 4])
def test_heat_fp32_scheme_close_to_fp64(orc, D):
    rng = np.random.default_rng(D)
    n = (24 + 2 * D, 20 + 2 * D, 18 + 2 * D)
    f = np.zeros(n[::-1], np.float64)
    f[D:-D, D:-D, D:-D] = rng.random((n[2] - 2 * D, n[1] - 2 * D, n[0] - 2 * D))
    f32 = f.astype(np.float32)
    orc.heat_run(f, D, D, 20, 0.1, 1.0, 1.0, 1.0)
    orc.heat_run(f32, D, D, 20, 0.1, 1.0, 1.0, 1.0)
    rel = np.linalg.norm(f32 - f) / np.linalg.norm(f)
    assert rel < 1e-6


def _b2r_heat(orc, dom, nb, R, D, nsteps, coef):
    """Run heat through B2R blocks in the oracle: exchange, then R sub-steps."""
    H = R * D
    # domain with a D-deep shell -> pad to an H-deep shell (zeros beyond D)
    pad = H - D
    big = np.pad(dom, pad) if pad else dom.copy()
    blocks = orc.split_blocks(big, nb, H)
    tmp = {k: v.copy() for k, v in blocks.items()}
    cur, nxt = blocks, tmp
    for s in range(nsteps):
        i = s % R
        if i == 0 and s > 0:
            orc.halo_exchange(cur, nb, H)
        for k in cur:
            edge = orc.edge_mask(k, nb)
            nxt[k][...] = cur[k]
            orc.heat_substep(cur[k], nxt[k], D, i, H, edge, *coef)
        cur, nxt = nxt, cur
    out = orc.join_blocks(cur, nb, H, shell=big)
    return out[pad:out.shape[0] - pad, pad:out.shape[1] - pad, pad:out.shape[2] - pad] if pad else out


@pytest.mark.parametrize("D,R,nb", [(1, 1, (2, 2, 2)), (1, 3, (2, 1, 2)), (2, 2, (2, 2, 1)),
                                    (4, 1, (1, 2, 2))])
def test_b2r_blocks_reproduce_single_domain(orc, D, R, nb):
    env = (24, 16, 16)
    rng = np.random.default_rng(7)
    dom = np.zeros(tuple(e + 2 * D for e in env[::-1]), np.float32)
    dom[D:-D, D:-D, D:-D] = rng.random(env[::-1], dtype=np.float32)
    coef = (0.02, 1.0, 1.0, 0.7)
    ref = dom.copy()
    orc.heat_run(ref, D, D, 7, *coef)
    got = _b2r_heat(orc, dom, nb, R, D, 7, coef)
    assert np.array_equal(got, ref)


def test_halo_exchange_is_global_wrap(orc):
    rng = np.random.default_rng(3)
    env, nb, H = (12, 8, 10), (3, 2, 2), 2
    dom = rng.integers(0, 255, env[::-1]).astype(np.uint8)
    blocks = orc.split_blocks(dom, nb, H, periodic=True)
    # scramble halos, exchange, compare with the wrapped padding
    for b in blocks.values():
        inner = b[H:-H, H:-H, H:-H].copy()
        b[...] = 0
        b[H:-H, H:-H, H:-H] = inner
    orc.halo_exchange(blocks, nb, H, periodic=True)
    ref = orc.split_blocks(dom, nb, H, periodic=True)
    for k in blocks:
        assert np.array_equal(blocks[k], ref[k]), k


def _gol_center(orc, cube3, center):
    """State of the centre cell after one generation, neighbours given as 3x3x3."""
    g = np.zeros((5, 5, 5), np.uint8)
    g[1:4, 1:4, 1:4] = cube3
    g[2, 2, 2] = center
    out = g.copy()
    orc.gol_substep(g, out, 0, 1, 63)
    return int(out[2, 2, 2])


@pytest.mark.parametrize("n", range(0, 27))
def test_gol_rule_known_answers(orc, n):
    rng = np.random.default_rng(n)
    cube = np.zeros(27, np.uint8)
    idx = [i for i in range(27) if i != 13]
    cube[rng.choice(idx, n, replace=False)] = 1
    cube = cube.reshape(3, 3, 3)
    # gol-3D.cu:104-117: live dies with <=1 or >=8, dead is born with exactly 5
    assert _gol_center(orc, cube, 1) == (0 if (n <= 1 or n >= 8) else 1)
    assert _gol_center(orc, cube, 0) == (1 if n == 5 else 0)


def test_gol_blocks_reproduce_torus(orc):
    rng = np.random.default_rng(2)
    env, nb, R = (16, 12, 20), (2, 2, 2), 3
    dom = (rng.random(env[::-1]) < 0.3).astype(np.uint8)
    ref = dom.copy()
    orc.gol_run_periodic(ref, 7)
    blocks = orc.split_blocks(dom, nb, R, periodic=True)
    tmp = {k: v.copy() for k, v in blocks.items()}
    cur, nxt = blocks, tmp
    for s in range(7):
        i = s % R
        if i == 0 and s > 0:
            orc.halo_exchange(cur, nb, R, periodic=True)
        for k in cur:
            nxt[k][...] = cur[k]
            orc.gol_substep(cur[k], nxt[k], i, R, 0)
        cur, nxt = nxt, cur
    assert np.array_equal(orc.join_blocks(cur, nb, R), ref)


def _eqwp_fields(n, dtype, seed=5):
    rng = np.random.default_rng(seed)
    f = [np.zeros(n[::-1], dtype) for _ in range(10)]
    for k in range(9):
        f[k][4:-4, 4:-4, 4:-4] = (rng.random((n[2] - 8, n[1] - 8, n[0] - 8)) - 0.5) * 1e-3
    return f


def test_eqwp_ref_fp32_close_to_fp64(orc):
    n = (28, 24, 20)
    f64 = _eqwp_fields(n, np.float64)
    f32 = [a.astype(np.float32) for a in f64]
    force = dict(fy=14, fx0=10, fx1=13, fz0=8, fz1=11, fval=-1e4, fsteps=50)
    for ts in range(6):
        orc.eqwp_ref_substep(f64, 0, 4, 63, ts, force)
        orc.eqwp_ref_substep(f32, 0, 4, 63, ts, force)
    for k in range(10):
        rel = np.linalg.norm(f32[k] - f64[k]) / max(np.linalg.norm(f64[k]), 1e-30)
        assert rel < 1e-5, (k, rel)


def test_eqwp_stag_fp32_close_to_fp64(orc):
    n = (26, 22, 20)
    rng = np.random.default_rng(9)
    f64 = _eqwp_fields(n, np.float64, 11)[:9]
    vp = 2000 + 2000 * rng.random(n[::-1])
    vs = vp / np.sqrt(3.0)
    rho = 2000 + 600 * rng.random(n[::-1])
    mu = rho * vs ** 2
    lam = rho * vp ** 2 - 2 * mu
    m64 = [lam, mu, 1.0 / rho]
    f32 = [a.astype(np.float32) for a in f64]
    m32 = [np.ascontiguousarray(m.astype(np.float32)) for m in m64]
    dt = 0.5 * 10.0 / (4000 * np.sqrt(3) * (9 / 8 + 1 / 24))
    for t in range(8):
        orc.eqwp_stag_step(f64, m64, dt, 10.0, 0, 4, 63, (13, 11, 10), 1e3 * (t + 1))
        orc.eqwp_stag_step(f32, m32, dt, 10.0, 0, 4, 63, (13, 11, 10), 1e3 * (t + 1))
    for k in range(9):
        rel = np.linalg.norm(f32[k] - f64[k]) / max(np.linalg.norm(f64[k]), 1e-30)
        assert rel < 1e-5, (k, rel)


def test_periodic_heat_oracle_against_explicit_loop(orc):
    """The torus restatement (numpy, float64) against an explicit loop with
    wrapped indices on a small ragged grid; the total heat is conserved."""
    rng = np.random.default_rng(1)
    a = rng.random((5, 4, 6)).astype(np.float32)
    got = orc.heat_run_periodic(a, 3, 0.1, 1.0, 2.0, 0.5)
    u = a.astype(np.float64)
    nz, ny, nx = u.shape
    for _ in range(3):
        n = u.copy()
        for z in range(nz):
            for y in range(ny):
                for x in range(nx):
                    lx = u[z, y, (x - 1) % nx] - 2 * u[z, y, x] + u[z, y, (x + 1) % nx]
                    ly = u[z, (y - 1) % ny, x] - 2 * u[z, y, x] + u[z, (y + 1) % ny, x]
                    lz = u[(z - 1) % nz, y, x] - 2 * u[z, y, x] + u[(z + 1) % nz, y, x]
                    n[z, y, x] = u[z, y, x] + 0.1 * (lx / 1.0 + ly / 4.0 + lz / 0.25)
        u = n
    assert np.abs(got - u).max() < 1e-13
    assert abs(got.sum() - a.astype(np.float64).sum()) < 1e-9


def test_periodic_staggered_oracle_against_c_oracle_inside(orc):
    """The torus restatement of the staggered step (numpy, float64) against
    the C oracle (fixed shell) on the cells the wrap cannot reach yet: a
    disturbance confined to the middle, 3 steps (4 cells of reach per step)."""
    env = (40, 36, 44)
    rng = np.random.default_rng(3)
    shape = env[::-1]
    f = [np.zeros(shape) for _ in range(9)]
    for k in range(9):
        f[k][16:28, 14:22, 16:24] = rng.standard_normal((12, 8, 8)) * 1e-3
    mat = [np.full(shape, 4.0e9), np.full(shape, 3.0e9), np.full(shape, 1.0 / 2300.0)]
    mat[0][: shape[0] // 2] *= 1.2
    dt, h = 1e-4, 10.0
    amps = [0.5, -0.25, 0.125]
    got = orc.eqwp_stag_run_periodic(f, mat, dt, h, amps, (20, 18, 22))
    ref = [a.copy() for a in f]
    for t, amp in enumerate(amps):
        orc.eqwp_stag_step(ref, mat, dt, h, 0, 2, 63, (20, 18, 22), amp)
    for k in range(9):
        inner = (slice(4, -4), slice(4, -4), slice(4, -4))
        assert np.allclose(got[k][inner], ref[k][inner], rtol=1e-12, atol=1e-18), k
        assert np.abs(got[k]).max() > 0


@pytest.mark.parametrize("D", [2, 3, 4])
def test_periodic_heat_oracle_inside_matches_c_oracle(orc, D):
    """Radius 2-4 on the torus (numpy, float64) against the C oracle's
    fixed-shell float64 steps on the cells the wrap cannot reach: a
    disturbance confined to the middle, 2 steps."""
    n = 40
    rng = np.random.default_rng(D)
    a = np.zeros((n, n, n))
    a[14:26, 14:26, 14:26] = rng.random((12, 12, 12))
    got = orc.heat_run_periodic(a, 2, 0.02, 1.0, 1.5, 0.75, D=D)
    ref = a.copy()
    orc.heat_run(ref, D, D, 2, 0.02, 1.0, 1.5, 0.75)
    inner = (slice(3 * D, -3 * D),) * 3
    assert np.allclose(got[inner], ref[inner], rtol=1e-12, atol=1e-15)
