"""CPU tests of the C ABI: the library builds, loads, exports every declared
entry point, and rejects invalid configurations before touching a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if hdr.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", hdr)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(b2r_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(b2r):
    names = declared_symbols()
    assert len(names) >= 15
    L = C.CDLL(b2r.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


@pytest.mark.parametrize("kw,frag", [
    (dict(model=1, env=(100, 64, 64), blocks=(3, 1, 1)), "divisible"),
    (dict(model=1, env=(64, 64, 64), blocks=(2, 2, 2), R=9, D=2), "R*D"),
    (dict(model=1, env=(64, 64, 64), D=5), "radius"),
    (dict(model=2, env=(64, 64, 64), D=2), "radius D = 1"),
    (dict(model=3, env=(64, 64, 64), D=1), "D = 2"),
    (dict(model=7, env=(64, 64, 64)), "unknown model"),
    (dict(model=1, env=(64, 64, 64), R=0), "R must be"),
])
def test_create_rejects_bad_config(b2r, kw, frag):
    with pytest.raises(b2r.B2RError) as ei:
        b2r.Domain(**kw)
    assert ei.value.status == 1 and frag in str(ei.value)


def test_per_block_entry_rejects_bad_args(b2r):
    import numpy as np
    a = np.zeros((6, 6, 6), np.float32)
    with pytest.raises(b2r.B2RError) as ei:
        b2r.heat_3D_gpu_main(a, R=3, D=1)      # 6 - 2*3 = 0 interior cells
    assert ei.value.status == 1
    with pytest.raises(b2r.B2RError):
        b2r.heat_3D_gpu_main(a, R=1, D=7)
