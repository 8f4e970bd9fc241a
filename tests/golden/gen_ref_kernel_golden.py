"""Golden outputs of the reference's own CUDA kernels, for tests that run
without them.

Run on a machine with the GPU, where oracle/_ref holds the cubins that
oracle/build.py compiles from the reference's eqwp.cu, gol-3D.cu and
heat-3D.cu:

    python tests/golden/gen_ref_kernel_golden.py [out_dir]

It drives the kernels through oracle/refgpu.py inside their correct
envelope (R = 1; the elastic wave within one 16-row tile in y; Game of Life
within one 32 x 32 tile, one generation per launch with the shell restored;
heat delta 2-4 within one 32-row tile in y; the edge-flag delta-1 kernel at
any R) on seeded inputs and writes ref_kernels.npz (the elastic-wave and
delta-1 heat outputs), ref_heat_kernels.npz (delta 2-4 and the edge-flag
kernel) and ref_kernels.json (the cases, and the SHA-256 of the Game of Life
output, which is integer work).

Cases (inputs re-created from numpy default_rng seeds by the tests):
* eqwp: interior 12 x 8 x 10 (16 x 12 x 14 reference block), the nine
  wavefield components U[-5e-3, 5e-3) from seed 21 in that order, zero
  displacement, 60 steps (the body force on for the first 50).
* gol: interior 30 x 30 x 40 with a one-cell shell, Bernoulli(0.3) from
  seed 31, the z = 0 shell plane live, 12 generations.
* heat: interior 30 x 20 x 16 with a zero shell, U[0, 1) from seed 41, 30
  steps with the kernel's constants (alpha*dt = 0.01, dx = dy = 1, dz = 0.5).
* heat delta D = 2, 3, 4 (fdm_heat_diffuse_delta<D>, heat-3D.cu:250,337,432):
  interiors 86 x 24 x 20, 84 x 22 x 18 and 82 x 24 x 20 with a zero D-cell
  shell (90 cells in x: three x tiles whose last one keeps its left halo
  loads), U[0, 1) from seeds 42, 43, 44, 20 steps, the kernels' constants.
* heat edge flags (fdm_heat_diffuse_delta1_verify, heat-3D.cu:57, driven as
  heat_3D_gpu_main, heat-3D.cu:583): padded blocks 70 x 50 x 40 with R = 3
  and flags (-1, 0, 1), and 66 x 45 x 36 with R = 2 and flags (1, -1, 0),
  every cell U[0, 1) from seeds 45, 46.
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

EQWP = dict(env=(12, 8, 10), seed=21, nsteps=60)
GOL = dict(env=(30, 30, 40), seed=31, ngen=12)
HEAT = dict(env=(30, 20, 16), seed=41, nsteps=30)
HEAT_D = {2: dict(env=(86, 24, 20), seed=42, nsteps=20), 3: dict(env=(84, 22, 18), seed=43, nsteps=20),
          4: dict(env=(82, 24, 20), seed=44, nsteps=20)}
HEAT_VERIFY = [dict(shape=(40, 50, 70), R=3, ef=(-1, 0, 1), seed=45),
               dict(shape=(36, 45, 66), R=2, ef=(1, -1, 0), seed=46)]


def eqwp_inputs():
    env = EQWP["env"]
    shape = tuple(e + 4 for e in env[::-1])
    rng = np.random.default_rng(EQWP["seed"])
    init = [np.zeros(shape, np.float32) for _ in range(10)]
    for k in range(9):
        init[k][2:-2, 2:-2, 2:-2] = ((rng.random(env[::-1]) - 0.5) * 1e-2).astype(np.float32)
    return init


def gol_input():
    env = GOL["env"]
    rng = np.random.default_rng(GOL["seed"])
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.uint8)
    dom[1:-1, 1:-1, 1:-1] = (rng.random(env[::-1]) < 0.3).astype(np.uint8)
    dom[0] = 1
    return dom


def heat_input():
    env = HEAT["env"]
    rng = np.random.default_rng(HEAT["seed"])
    dom = np.zeros(tuple(e + 2 for e in env[::-1]), np.float32)
    dom[1:-1, 1:-1, 1:-1] = rng.random(env[::-1], dtype=np.float32)
    return dom


def heat_d_input(D):
    c = HEAT_D[D]
    rng = np.random.default_rng(c["seed"])
    dom = np.zeros(tuple(e + 2 * D for e in c["env"][::-1]), np.float32)
    dom[D:-D, D:-D, D:-D] = rng.random(c["env"][::-1], dtype=np.float32)
    return dom


def heat_verify_input(k):
    c = HEAT_VERIFY[k]
    return np.random.default_rng(c["seed"]).random(c["shape"], dtype=np.float32)


def main(out_dir):
    from oracle import refgpu
    eq = refgpu.run_reference(eqwp_inputs(), EQWP["nsteps"])
    gol = refgpu.run_reference_gol(gol_input(), GOL["ngen"])
    heat = refgpu.run_reference_heat(heat_input(), HEAT["nsteps"])
    heat_d = {D: refgpu.run_reference_heat_d(heat_d_input(D), D, HEAT_D[D]["nsteps"]) for D in HEAT_D}
    heat_v = [refgpu.run_reference_heat_verify(heat_verify_input(k), c["R"], c["ef"])
              for k, c in enumerate(HEAT_VERIFY)]
    os.makedirs(out_dir, exist_ok=True)
    np.savez_compressed(os.path.join(out_dir, "ref_kernels.npz"), heat=heat,
                        **{f"eqwp{k}": a for k, a in enumerate(eq)})
    np.savez_compressed(os.path.join(out_dir, "ref_heat_kernels.npz"),
                        **{f"heat_d{D}": a for D, a in heat_d.items()},
                        **{f"heat_verify{k}": a for k, a in enumerate(heat_v)})
    meta = dict(eqwp=EQWP, gol=dict(GOL, sha256_out=hashlib.sha256(gol.tobytes()).hexdigest()), heat=HEAT,
                heat_d={str(D): c for D, c in HEAT_D.items()}, heat_verify=HEAT_VERIFY,
                kernels="eqwp.cu eqwp_fd4_stress/vx/vy/vz, gol-3D.cu gol_3d_kernel, "
                        "heat-3D.cu fdm_heat_diffuse_delta1 / delta1_verify and (built at B2R_D = 2, 3, 4) "
                        "fdm_heat_diffuse_delta2/3/4, compiled unmodified for sm_103a")
    with open(os.path.join(out_dir, "ref_kernels.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", out_dir)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
