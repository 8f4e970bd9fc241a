"""CPU check of the second oracle's loader: the kernel names it asks the
driver for are the C++ (Itanium) manglings of the reference kernels'
signatures (eqwp.cu:60,154,249,341; gol-3D.cu:30; heat-3D.cu:57,173,250,337,432), as g++
mangles the same declarations."""
import os
import shutil
import subprocess

import pytest

SIGS = {
    "stress": "void eqwp_fd4_stress(int, int, int, float*, float*, float*, float*, float*, float*, float*, "
              "float*, float*, int) {}",
    "vx": "void eqwp_fd4_vx(int, int, int, float*, float*, float*, float*, float3*, int, int, int) {}",
    "vy": "void eqwp_fd4_vy(int, int, int, float*, float*, float*, float*, float3*, float*, int, int, int) {}",
    "vz": "void eqwp_fd4_vz(int, int, int, float*, float*, float*, float*, float3*, int, int, int) {}",
    "gol": "void gol_3d_kernel(unsigned char*, unsigned char*, int, int, int, int) {}",
    "heat": "void fdm_heat_diffuse_delta1(float*, float*, int, int, int, int) {}",
    "heat_verify": "void fdm_heat_diffuse_delta1_verify(float*, float*, int, int, int, int, int, int, int, "
                   "int) {}",
    "heat2": "void fdm_heat_diffuse_delta2(float*, float*, int, int, int, int) {}",
    "heat3": "void fdm_heat_diffuse_delta3(float*, float*, int, int, int, int) {}",
    "heat4": "void fdm_heat_diffuse_delta4(float*, float*, int, int, int, int) {}",
}


def test_mangled_names_match_signatures(tmp_path):
    if not (shutil.which("g++") and shutil.which("nm")):
        pytest.skip("g++ / nm not available")
    from oracle import refgpu
    src = tmp_path / "sigs.cpp"
    src.write_text("struct float3 { float x, y, z; };\n" + "\n".join(SIGS.values()) + "\n")
    obj = tmp_path / "sigs.o"
    subprocess.check_call(["g++", "-c", str(src), "-o", str(obj)])
    names = set(line.split()[-1] for line in subprocess.check_output(["nm", str(obj)], text=True).splitlines())
    want = dict(refgpu._NAMES)
    want["gol"] = refgpu._GOL_NAME
    want["heat"] = refgpu._HEAT_NAME
    want["heat_verify"] = refgpu._HEAT_VERIFY_NAME
    for D, name in refgpu._HEAT_D_NAMES.items():
        want[f"heat{D}"] = name
    for k, name in want.items():
        assert name in names, (k, name)
