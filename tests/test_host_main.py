"""The C++ host program b2r_main (b2r.cpp's main over the C ABI): argument
checks as the reference makes them (CPU), and full runs of every model on
the GPU, whose snapshot matches the library driven from Python."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAIN = os.path.join(ROOT, "b2r_gb300", "b2r_main")


def run(*args, cwd=None):
    if not os.path.exists(MAIN):
        pytest.fail("b2r_main is missing: build() compiles it")
    return subprocess.run([MAIN, *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=600)


def test_usage_without_four_arguments(b2r):
    r = run(1, 2, 2)
    assert r.returncode == 1
    assert "please set parameter B2R_B_R, BLOCK_DIM_(X,Y,Z)" in r.stdout


def test_env_must_divide_by_blocks(b2r):
    r = run(1, 3, 1, 1, "--env", 64, 64, 64)
    assert r.returncode == 1
    assert "perfectly divisible" in r.stdout


def test_halo_must_fit_the_block(b2r):
    r = run(40, 1, 1, 1, "--env", 64, 64, 64)
    assert r.returncode == 1
    assert "R*D" in r.stdout


def test_unknown_model(b2r):
    r = run(1, 1, 1, 1, "--model", "nope")
    assert r.returncode == 1 and "unknown model" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("model,R,blocks,env,extra", [
    ("eqwp", 2, (2, 1, 2), (48, 32, 40), []),
    ("eqwp", 1, (1, 1, 1), (40, 24, 32), ["--direct"]),
    ("heat", 3, (2, 2, 1), (48, 48, 32), []),
    ("gol", 4, (2, 2, 2), (64, 64, 64), []),
    ("stag", 2, (2, 2, 1), (64, 64, 32), []),
])
def test_main_runs_every_model(b2r, tmp_path, model, R, blocks, env, extra):
    r = run(R, *blocks, "--model", model, "--env", *env, "--iters", 13, "--snapshot", tmp_path, *extra)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "13 Iterations with B2R_R=%d took" % R in r.stdout
    assert "device computation took" in r.stdout
    files = sorted(os.listdir(tmp_path))
    assert len(files) == (0 if model == "gol" else blocks[0] * blocks[1] * blocks[2])


@pytest.mark.gpu
def test_main_matches_library(b2r, tmp_path):
    """The program's heat run (exchange of the field by boundary_updating,
    then R steps, per period) gives the bits of Domain.step."""
    env, R, blocks, iters = (48, 40, 32), 2, (2, 1, 1), 9
    r = run(R, *blocks, "--model", "heat", "--env", *env, "--iters", iters, "--D", 1, "--snapshot", tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    # the program's seeded start, from a zero-step run of it
    (tmp_path / "start").mkdir()
    r0 = run(R, *blocks, "--model", "heat", "--env", *env, "--iters", 0, "--D", 1,
             "--snapshot", tmp_path / "start")
    assert r0.returncode == 0, r0.stdout + r0.stderr
    with b2r.Domain(b2r.MODEL_HEAT, env, blocks=blocks, R=R, D=1, alpha_dt=0.1) as d:
        start = [b2r.read_block_data_bin(str(tmp_path / "start" / n))
                 for n in ("u-0.bin", "u-b1-0.bin")]
        # rebuild the domain array from the two padded blocks (halo H = 2)
        H, B = 2, env[0] // 2
        dom = np.zeros(d.domain_shape, np.float32)
        dom[:, :, : B + 1] = start[0][H - 1:-(H - 1), H - 1:-(H - 1), H - 1:H + B]
        dom[:, :, B + 1:] = start[1][H - 1:-(H - 1), H - 1:-(H - 1), H:H + B + 1]
        d.upload(dom)
        d.step(iters)
        blocks_now = d.download_blocks()
        d.synchronize()
    for k, n in enumerate(("u-%d.bin" % iters, "u-b1-%d.bin" % iters)):
        got = b2r.read_block_data_bin(str(tmp_path / n))
        want = blocks_now[(k, 0, 0)]
        s = (slice(H, -H),) * 3
        assert np.array_equal(got[s], want[s]), n
