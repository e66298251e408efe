"""The restated MagicHat stream (pngf_gb300/csrc/hat_rng.h), which the
device-resident DBS loop draws from, against this C++ library's
std::mt19937 and std::uniform_int_distribution<int> (what MagicHat uses,
pngf-opt/magichat.hpp:53-107): engine words, bounded draws over many ranges
and whole hat passes must agree exactly."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def check_exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("hat_rng") / "hat_rng_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "pngf_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "hat_rng_check.cpp"), "-o", exe], check=True)
    return exe


def test_restated_hat_stream_matches_std(check_exe):
    out = subprocess.run([check_exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")


def _oracle_sequence(tx, ty, sym, seed, evals):
    """The reference's candidate order under the same accept rule, from the
    oracle's MagicHat and draw loop (main.cpp:343-392)."""
    from oracle.dbs import hat_size, initial_design, next_candidate
    from oracle.geometry import Geometry
    from oracle.magichat import MagicHat
    geo = Geometry(tx, ty)
    hat = MagicHat(seed, 0, hat_size(geo, sym))
    initial_design(geo, hat, sym, True)
    seq, last = [], -1
    while len(seq) < evals:
        c = next_candidate(geo, hat, sym, last)
        if c is None:
            break
        li, tiles, last = c
        seq.append([li] + list(tiles))
        if (len(seq) - 1) % 7 == 3:
            hat.reset()
    return seq


@pytest.mark.parametrize("tx,sym,seed,batch,evals", [(7, 1, 1, 5, 60), (9, 1, 3, 16, 120), (11, 0, 2, 16, 400),
                                                     (11, 0, 2, 1, 150)])
def test_device_replay_matches_oracle_order(check_exe, tx, sym, seed, batch, evals):
    """The device loop's draws (restated stream, shared skip rules, speculative
    batches replayed by engine-output counts) give the oracle's candidate
    order under a fixed accept rule."""
    q = (tx + 1) // 2
    binary_draws = q * q if sym else tx * tx  # the initial design's rand_binary draws
    out = subprocess.run([check_exe, "seq", str(tx), str(tx), str(sym), str(seed), str(binary_draws), str(batch),
                          str(evals)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    got = [[int(v) for v in line.split()] for line in out.stdout.strip().splitlines()]
    assert got == _oracle_sequence(tx, tx, bool(sym), seed, evals)
