import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def built_lib():
    """The in-tree shared library, built once if it is missing."""
    from pngf_gb300 import build, lib
    if not os.path.exists(lib.LIB_PATH):
        build.build()
    return lib.load()


@pytest.fixture(scope="session")
def cases():
    with open(os.path.join(GOLDEN, "cases.json")) as fh:
        return {c["name"]: c for c in json.load(fh)}


_G_CACHE = {}


def case_G(case, built_lib=None):
    """(Gs, gobj_rows) for a golden case: the inputs the reference ran on, from
    the oracle's generator (oracle/synth.c) -- G per frequency and the two
    synthetic NF2FF rows (zero rows for a case recorded without them)."""
    from oracle import synth
    key = case["name"]
    if key not in _G_CACHE:
        Gs = [synth.synth_G(case["tiles"], case["tiles"], f, seed=case["g_seed"]) for f in case["freqs"]]
        n = Gs[0].shape[0]
        if case.get("gobj") == "synth":
            rows = synth.synth_gobj(case["tiles"], case["tiles"], seed=case["g_seed"])
        else:
            rows = np.zeros((2, n), dtype=np.complex128)
        _G_CACHE[key] = (Gs, [rows for _ in Gs])
    return _G_CACHE[key]


def golden_log(name):
    from oracle.dbs import parse_ref_log
    return parse_ref_log(os.path.join(GOLDEN, name + ".log"))
