"""The oracle (CPU) and the library (GPU) against golden outputs of the
reference's own CUDA kernels (tests/golden/gen_ref_kernel_golden.py made
them on the GPU from the unmodified eqwp.cu, gol-3D.cu and heat-3D.cu)."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import gen_ref_kernel_golden as G  # noqa: E402

META = json.load(open(os.path.join(HERE, "golden", "ref_kernels.json")))
NPZ = np.load(os.path.join(HERE, "golden", "ref_kernels.npz"))
NAMES = ["vx", "vy", "vz", "sxx", "sxy", "sxz", "syy", "syz", "szz", "disp"]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def eqwp_force(shape):
    ngz, ngy, ngx = shape
    return dict(fy=ngy - 7 - 2, fx0=ngx // 2, fx1=ngx // 2 + ngx // 10, fz0=ngz // 2,
                fz1=ngz // 2 + ngz // 10, fval=-1e4, fsteps=50)   # eqwp.cu:131,561-566


def test_oracle_eqwp_matches_reference_kernels(orc):
    f = G.eqwp_inputs()
    force = eqwp_force(f[0].shape)
    for ts in range(G.EQWP["nsteps"]):
        orc.eqwp_ref_substep(f, 0, 2, 63, ts, force)
    for k in range(10):
        assert rel_l2(f[k], NPZ[f"eqwp{k}"]) <= 1e-5, NAMES[k]


def test_oracle_gol_matches_reference_kernel(orc):
    a = G.gol_input()
    b = a.copy()
    for _ in range(G.GOL["ngen"]):
        orc.gol_substep(a, b, 0, 1, 63)
        a, b = b, a
    assert hashlib.sha256(a.tobytes()).hexdigest() == META["gol"]["sha256_out"]


def test_oracle_heat_matches_reference_kernel(orc):
    u = G.heat_input()
    orc.heat_run(u, 1, 1, G.HEAT["nsteps"], 0.01, 1.0, 1.0, 0.5)
    assert rel_l2(u, NPZ["heat"]) <= 1e-5


@pytest.mark.gpu
def test_library_matches_reference_kernels(b2r):
    init = G.eqwp_inputs()
    with b2r.Domain(b2r.MODEL_EQWP_REF, G.EQWP["env"], D=2, R=1) as d:
        for k in range(10):
            d.upload(init[k], field=k)
        d.step(G.EQWP["nsteps"])
        got = [d.download(field=k) for k in range(10)]
    for k in range(10):
        assert rel_l2(got[k], NPZ[f"eqwp{k}"]) <= 1e-5, NAMES[k]
    with b2r.Domain(b2r.MODEL_GOL, G.GOL["env"], D=1, R=1) as d:
        d.upload(G.gol_input())
        d.step(G.GOL["ngen"])
        g = d.download()
    assert hashlib.sha256(g.tobytes()).hexdigest() == META["gol"]["sha256_out"]
    with b2r.Domain(b2r.MODEL_HEAT, G.HEAT["env"], D=1, R=1, alpha_dt=0.01, dx=1.0, dy=1.0, dz=0.5) as d:
        d.upload(G.heat_input())
        d.step(G.HEAT["nsteps"])
        h = d.download()
    assert rel_l2(h, NPZ["heat"]) <= 1e-5


HEAT_NPZ = np.load(os.path.join(HERE, "golden", "ref_heat_kernels.npz"))


def verify_edge(ef):
    e = 0
    for a in range(3):
        e |= (1 << (2 * a)) if ef[a] < 0 else 0
        e |= (1 << (2 * a + 1)) if ef[a] > 0 else 0
    return e


@pytest.mark.parametrize("D", [2, 3, 4])
def test_oracle_heat_high_order_matches_reference_kernels(orc, D):
    """The oracle's order-D restatement against fdm_heat_diffuse_delta<D>
    (heat-3D.cu:250-521) inside its envelope: R = 1, one y tile."""
    u = G.heat_d_input(D)
    orc.heat_run(u, D, D, G.HEAT_D[D]["nsteps"], 0.01, 1.0, 1.0, 0.5)
    assert rel_l2(u, HEAT_NPZ[f"heat_d{D}"]) <= 1e-5


@pytest.mark.parametrize("k", [0, 1])
def test_oracle_heat_edge_flags_match_reference_verify_kernel(orc, k):
    """The oracle's fixed-shell window against fdm_heat_diffuse_delta1_verify
    (heat-3D.cu:57-158) driven as heat_3D_gpu_main, R = 2 and 3."""
    c = G.HEAT_VERIFY[k]
    blk = G.heat_verify_input(k)
    R = c["R"]
    a, b = blk.copy(), blk.copy()
    for i in range(R):
        orc.heat_substep(a, b, 1, i, R, verify_edge(c["ef"]), **orc.REF_HEAT)
        a, b = b, a
    ref = blk.copy()
    ref[R:-R] = a[R:-R]
    assert rel_l2(ref, HEAT_NPZ[f"heat_verify{k}"]) <= 1e-5


@pytest.mark.gpu
def test_library_matches_reference_heat_kernels(b2r):
    for D, c in G.HEAT_D.items():
        with b2r.Domain(b2r.MODEL_HEAT, c["env"], D=D, R=1, alpha_dt=0.01, dx=1.0, dy=1.0, dz=0.5) as d:
            d.upload(G.heat_d_input(D))
            d.step(c["nsteps"])
            h = d.download()
        assert rel_l2(h, HEAT_NPZ[f"heat_d{D}"]) <= 1e-5, f"delta{D}"
    for k, c in enumerate(G.HEAT_VERIFY):
        blk = G.heat_verify_input(k)
        b2r.heat_3D_gpu_main(blk, c["R"], D=1, edge_flag=c["ef"])
        assert rel_l2(blk, HEAT_NPZ[f"heat_verify{k}"]) <= 1e-5, f"edge flags {c['ef']}"
