"""Failure detection without a GPU fault: a bounded mbarrier wait that nothing
completes gives up after its time limit, records an error code (as the
tensor-core update kernels do, which the library reports as
PNGF_ERR_TIMEOUT), and the context stays usable."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_survives(tmp_path):
    exe = str(tmp_path / "wait_timeout")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                    os.path.join(ROOT, "tests", "cpp", "wait_timeout.cu"), "-o", exe], check=True)
    r = subprocess.run([exe, "20000"], capture_output=True, text=True, timeout=120)  # 20 ms limit
    assert r.returncode == 0, r.stdout + r.stderr
    assert "wait status 77, after 1234" in r.stdout
    waited_us = int(r.stdout.split("waited_us")[1].split(",")[0])
    assert 20000 <= waited_us < 20000 + 1000000, r.stdout  # gave up at the limit, not long after
