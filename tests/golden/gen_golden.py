"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in the container that holds the reference source tree:

    python tests/golden/gen_golden.py

It compiles the reference's heat-3D.cpp (oracle/build.py), runs its
heat_3D_cpu_main (heat-3D.cpp:136) on seeded inputs and stores inputs and
outputs.  The reference's CPU heat path is delta1 only (its delta2-4 CPU
loops read out of bounds and delta3/4 use the delta2 coefficients,
heat-3D.cpp:67-132), and its constants are fixed (Alpha*Dt = 0.01, Dx = Dy
= 1, Dz = 0.5, heat-3D.cpp:19-23), so every fixture uses them.

Files:
* heat_d1_small.npz   -- 26x22x18 block, shell 0, interior U[0,1) seed 11:
                         10 calls with R=1; and one call each with R=2, R=3
                         on a block that is random everywhere (seed 12).
* heat_d1_cfg128.json -- the 128^3 case (130^3 storage, shell 0, interior
                         U[0,1) from numpy default_rng(1), 100 calls with
                         R=1): sha256 of input and output bytes, sums and
                         sample values.
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build as obuild  # noqa: E402
from oracle import orc  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def shell_field(n, seed, dtype=np.float32):
    """(nz,ny,nx) storage with a 1-deep zero shell and U[0,1) interior."""
    nx, ny, nz = n
    a = np.zeros((nz, ny, nx), dtype)
    rng = np.random.default_rng(seed)
    a[1:-1, 1:-1, 1:-1] = rng.random((nz - 2, ny - 2, nx - 2), dtype=np.float32)
    return a


def main():
    if obuild.build_ref(force=True) is None:
        raise SystemExit("reference source tree not found")
    # small block
    a = shell_field((26, 22, 18), 11)
    out10 = a.copy()
    for _ in range(10):
        orc.ref_heat_cpu_main(out10, 1, 4)
    rng = np.random.default_rng(12)
    b = rng.random((18, 22, 26), dtype=np.float32)
    out_r2 = b.copy()
    orc.ref_heat_cpu_main(out_r2, 2, 4)
    out_r3 = b.copy()
    orc.ref_heat_cpu_main(out_r3, 3, 4)
    np.savez_compressed(os.path.join(OUT, "heat_d1_small.npz"), in_shell=a, out_r1x10=out10,
                        in_rand=b, out_r2=out_r2, out_r3=out_r3)
    # config-1 size, checksums only
    c = shell_field((130, 130, 130), 1)
    hin = hashlib.sha256(c.tobytes()).hexdigest()
    for _ in range(100):
        orc.ref_heat_cpu_main(c, 1, 8)
    meta = {
        "storage": [130, 130, 130], "shell": 1, "seed": 1, "steps": 100, "R": 1,
        "alpha_dt": 0.1 * 0.1, "dx": 1.0, "dy": 1.0, "dz": 0.5,
        "sha256_in": hin, "sha256_out": hashlib.sha256(c.tobytes()).hexdigest(),
        "sum_out": float(c.astype(np.float64).sum()),
        "samples": {f"{z},{y},{x}": float(c[z, y, x]) for (z, y, x) in
                    [(1, 1, 1), (64, 64, 64), (128, 1, 77), (65, 128, 3), (100, 31, 128)]},
        "generator": "tests/golden/gen_golden.py via the reference heat_3D_cpu_main",
    }
    with open(os.path.join(OUT, "heat_d1_cfg128.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote fixtures")


if __name__ == "__main__":
    main()
