"""The reference's own driver compiles against the drop-in class.

pngf-opt/main.cpp, unmodified except that its two includes of the optimizer
("linalg.hpp", "pngfopt.hpp", main.cpp:111-112) become one include of
include/pngf_optimizer.hpp, is compiled syntax-only with g++ (Eigen and CBLAS
come from the oracle's shims, oracle/shim/, as in the oracle's own build of
the reference). Needs the reference tree: set PNGF_REFERENCE to it; without
it the test is skipped (the tree does not travel with this repository)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_main_compiles_against_dropin(tmp_path):
    ref = os.environ.get("PNGF_REFERENCE", "")
    main = os.path.join(ref, "pngf-opt", "main.cpp")
    if not ref or not os.path.exists(main):
        pytest.skip("set PNGF_REFERENCE to the reference tree")
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    src = open(main).read()
    assert src.count('#include "linalg.hpp"') == 1 and src.count('#include "pngfopt.hpp"') == 1
    src = src.replace('#include "linalg.hpp"', '#include "pngf_optimizer.hpp"').replace('#include "pngfopt.hpp"', "")
    (tmp_path / "main.cpp").write_text(src)
    (tmp_path / "Eigen").write_text('#include "eigen_subset.hpp"\n')  # main.cpp includes <Eigen>
    cmd = ["g++", "-std=c++17", "-fopenmp", "-fsyntax-only", "-I" + str(tmp_path),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle", "shim"),
           "-I" + os.path.join(ref, "pngf-opt"), str(tmp_path / "main.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
