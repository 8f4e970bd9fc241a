"""Block data files in the reference's format (eqwp.cu:616-651): an int32[3]
{Ngx, Ngy, Ngz} header and the padded block's float cells (x fastest), or
comma-separated text with one line per row."""
import os

import numpy as np
import pytest


def test_read_block_data_bin_roundtrip(tmp_path):
    """Reader against a file written here by hand (no GPU)."""
    import b2r_gb300
    rng = np.random.default_rng(0)
    cells = rng.random((5, 4, 3), dtype=np.float32)
    p = tmp_path / "displacement-7.bin"
    with open(p, "wb") as f:
        f.write(np.array([3, 4, 5], np.int32).tobytes())
        f.write(cells.tobytes())
    np.testing.assert_array_equal(b2r_gb300.read_block_data_bin(str(p)), cells)
    with open(p, "ab") as f:
        f.write(b"\0\0\0\0")
    with pytest.raises(ValueError):
        b2r_gb300.read_block_data_bin(str(p))


@pytest.mark.gpu
def test_displacement_file_matches_block(b2r, tmp_path):
    env = (24, 20, 16)
    rng = np.random.default_rng(5)
    shape = tuple(e + 4 for e in env[::-1])
    with b2r.Domain(b2r.MODEL_EQWP_REF, env, D=2, R=1) as d:
        for k in range(9):
            a = np.zeros(shape, np.float32)
            a[2:-2, 2:-2, 2:-2] = ((rng.random(env[::-1]) - 0.5) * 1e-2).astype(np.float32)
            d.upload(a, field=k)
        d.step(12)
        blk = d.download_blocks(field="disp")[(0, 0, 0)]
        p = d.write_block_data(field="disp", directory=str(tmp_path))
        pt = d.write_block_data(field="disp", directory=str(tmp_path), text=True)
        pv = d.write_block_data(field="vy", time_step=3, directory=str(tmp_path))
        vy = d.download_blocks(field="vy")[(0, 0, 0)]
        d.synchronize()
    assert os.path.basename(p) == "displacement-12.bin"
    assert os.path.basename(pt) == "displacement-12.txt"
    assert os.path.basename(pv) == "vy-3.bin"
    got = b2r.read_block_data_bin(p)
    assert got.shape == blk.shape
    np.testing.assert_array_equal(got, blk)
    np.testing.assert_array_equal(b2r.read_block_data_bin(pv), vy)
    assert np.abs(blk).max() > 0
    lines = open(pt).read().splitlines()
    assert len(lines) == blk.shape[0] * blk.shape[1]
    row = [float(v) for v in lines[-3].rstrip(",").split(",")]
    assert len(row) == blk.shape[2]
    np.testing.assert_allclose(row, blk.reshape(-1, blk.shape[2])[-3], rtol=1e-5, atol=1e-12)


@pytest.mark.gpu
def test_block_data_per_block_names_and_errors(b2r, tmp_path):
    env = (32, 32, 32)
    rng = np.random.default_rng(6)
    u = rng.random(env[::-1], dtype=np.float32)
    with b2r.Domain(b2r.MODEL_HEAT, env, D=1, R=2, blocks=(2, 1, 1)) as d:
        d.upload(np.pad(u, 1))
        d.step(2)
        blocks = d.download_blocks()
        p1 = d.write_block_data(block=1, directory=str(tmp_path))
        d.synchronize()
        assert os.path.basename(p1) == "u-b1-2.bin"
        np.testing.assert_array_equal(b2r.read_block_data_bin(p1), blocks[(1, 0, 0)])
        with pytest.raises(b2r.B2RError):
            d.write_block_data(block=2, directory=str(tmp_path))
        with pytest.raises(b2r.B2RError):
            d.write_block_data(field="lambda", directory=str(tmp_path))
