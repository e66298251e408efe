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


def force_port_tiles(tm, tiles_x, tiles_y):
    """The tiles pngf-opt/main.cpp:209-218 forces around the lumped port at the
    map centre (source tile and the tiles above and below it empty, the tiles
    left and right of it metal); DBS never flips them. Random test designs
    get the same, so that the port is not shorted (|S11| = 1, an objective
    with a 0/0 directivity)."""
    mx, my = (tiles_x - 1) // 2, (tiles_y - 1) // 2
    tm = [int(v) for v in tm]
    tm[my * tiles_x + mx - 1] = 1
    tm[my * tiles_x + mx + 1] = 1
    tm[my * tiles_x + mx] = 0
    tm[(my - 1) * tiles_x + mx] = 0
    tm[(my + 1) * tiles_x + mx] = 0
    return tm


def free_tiles(tiles_x, tiles_y):
    """Tiles a DBS candidate may flip: all but the source tile and its two
    forced metal neighbours (main.cpp:358-359)."""
    mx, my = (tiles_x - 1) // 2, (tiles_y - 1) // 2
    return [t for t in range(tiles_x * tiles_y) if not (t // tiles_x == my and t % tiles_x in (mx - 1, mx, mx + 1))]
