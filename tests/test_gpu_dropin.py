"""Code written for the reference's optimizer class runs on the library.

tests/cpp/dropin_main.cpp follows pngf-opt/main.cpp's call sequence on
PNGF_Optimizer objects (one per frequency) from include/pngf_optimizer.hpp.
It is compiled with g++ against libpngf_gb300.so, fed acmefdfd-layout G files
and must reproduce the reference's golden log."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, case_G, golden_log

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dropin_exe(tmp_path_factory, built_lib):
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_main")
    lib_dir = os.path.join(ROOT, "pngf_gb300")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp"), "-L" + lib_dir, "-lpngf_gb300",
                    "-Wl,-rpath," + lib_dir, "-o", out], check=True)
    return out


@pytest.mark.parametrize("name", ["sym_7x7_f1_seed1", "single_7x7_f2_seed1"])
def test_reference_style_program_matches_golden(name, cases, dropin_exe, tmp_path, built_lib):
    from oracle.dbs import parse_ref_log
    from pngf_gb300 import lib
    c = cases[name]
    Gs, gobj = case_G(c, built_lib)
    cmd = [dropin_exe, "--tiles", str(c["tiles"]), str(c["tiles"]), "--freq",
           ",".join(repr(float(f)) for f in c["freqs"]), "--seed", str(c["seed"]), "--init", c["init"],
           "--mode", c["mode"], "--log", str(tmp_path / "log.txt")]
    for i, G in enumerate(Gs):
        p = str(tmp_path / ("G%d.bin" % i))
        lib.write_G_file(p, G, gobj[i])
        cmd += ["--gfile", p]
    subprocess.run(cmd, check=True)
    got = parse_ref_log(str(tmp_path / "log.txt"))
    ref = golden_log(name)
    assert got["init_map"] == ref["init_map"]
    assert len(got["rows"]) == len(ref["rows"])
    for a, b in zip(got["rows"], ref["rows"]):
        assert a[1] == b[1] and a[2] == b[2]
        assert abs(a[3] - b[3]) <= 1e-10 * abs(b[3])
        np.testing.assert_allclose(a[5], b[5], rtol=1e-10, atol=1e-12)
    assert got["final_map"] == ref["final_map"]
