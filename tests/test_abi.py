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


def test_wrapper_checks_host_buffers(b2r):
    """The library trusts a host pointer for a fixed number of bytes, so the
    Python face refuses arrays of another size, element size or layout
    before any copy."""
    import numpy as np
    from b2r_gb300 import _ptr, _ef, _traces
    a = np.zeros((4, 5, 6), np.float32)
    assert _ptr(a, a.nbytes, 4)[1] == 0
    with pytest.raises(ValueError, match="must hold"):
        _ptr(a, a.nbytes + 4, 4)
    with pytest.raises(ValueError, match="cells of 4 bytes"):
        _ptr(a.astype(np.float64), a.nbytes * 2, 4)
    with pytest.raises(ValueError, match="C-contiguous"):
        _ptr(a[:, :, ::2])
    with pytest.raises(TypeError):
        _ptr([0.0] * 8)
    assert _ef((-1, 0, 1)) == bytes([255, 0, 1])
    for bad in ((0, 0), (0, 2, 0), (1, 1, 1, 1)):
        with pytest.raises(ValueError, match="edge_flag"):
            _ef(bad)
    assert _traces(np.zeros((7, 3)), 7, 3).dtype == np.float32
    with pytest.raises(ValueError, match="d_obs"):
        _traces(np.zeros((7, 2)), 7, 3)


def test_per_block_entries_check_the_block(b2r):
    import numpy as np
    for bad in (np.zeros((6, 6, 6), np.float64), np.zeros((6, 6), np.float32),
                np.zeros((6, 6, 12), np.float32)[:, :, ::2]):
        with pytest.raises(ValueError, match="numpy block"):
            b2r.heat_3D_gpu_main(bad, R=1)
    with pytest.raises(ValueError, match="numpy block"):
        b2r.gol_3D_gpu_main(np.zeros((6, 6, 6), np.float32), R=1)
    with pytest.raises(ValueError, match="edge_flag"):
        b2r.heat_3D_gpu_main(np.zeros((8, 8, 8), np.float32), R=1, edge_flag=(0, 0))
