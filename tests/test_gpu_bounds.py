"""The bounds-checked build (libpngf_gb300_bc.so, -DPNGF_BOUNDS_CHECK) on
golden cases: every data-dependent gather checks its index on the device and
records a violation instead of reading out of range. The DBS runs here --
the host driver (candidate kernels of both shapes, FP64 accepts on the
tensor cores including 96-edge accepts in pieces, the FP64 triangular-solve
W), the device-resident loop and the complex64 forms, immediate and deferred
(dense pending blocks, pending-factor appends, flushes) -- must record no
violation and still reproduce the reference's golden logs. This is the check
that stands in for compute-sanitizer. It runs in a child process, which loads
the checked library instead of the default one."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
import ctypes as C
from conftest import case_G, golden_log
from pngf_gb300 import lib
assert lib.LIB_PATH.endswith("_bc.so")
L = lib.load()
cases = {c["name"]: c for c in json.load(open(sys.argv[1] + "/tests/golden/cases.json"))}
out = []
for name, prec, dev_loop, simt, defer in (("sym_9x9_f2_seed3", lib.PREC_FP64, False, False, 0),
                                          ("sym_9x9_f2_seed3", lib.PREC_FP64, False, True, 0),
                                          ("single_7x7_f2_seed1", lib.PREC_FP64, True, False, 0),
                                          ("single_11x11_f3_seed2", lib.PREC_C64, False, False, 0),
                                          ("single_11x11_f3_seed2", lib.PREC_C64, False, False, 48)):
    c = cases[name]
    Gs, gobj = case_G(c)
    kw = {"fp64_update": lib.F64_SIMT} if simt else {}
    if defer:
        kw["defer_rank"] = defer
    h = lib.Handle(c["tiles"], c["tiles"], c["freqs"], precision=prec,
                   max_flips=4 if c["mode"] == "sym" else 1, **kw)
    for f, G in enumerate(Gs):
        h.load_G(f, G, gobj[f])
    d = lib.Dbs(h, mode=lib.DBS_SYMMETRIC if c["mode"] == "sym" else lib.DBS_SINGLE,
                init=lib.INIT_RANDOM if c["init"] == "random" else lib.INIT_EMPTY, seed=c["seed"],
                max_evals=c["max_evals"], batch=-4, device_loop=dev_loop)
    s = d.run()
    lg = d.log()
    ref = golden_log(name)
    same = [int(t) for t in lg["tile"]] == [r[1] for r in ref["rows"]] and \
           [int(a) for a in lg["accept"]] == [r[2] for r in ref["rows"]]
    v = C.c_longlong(-1)
    first = (C.c_longlong * 3)()
    rc = L.pngf_bounds_check_report(C.byref(v), first, 1)
    out.append(dict(name=name, prec=prec, device_loop=dev_loop, simt=simt, defer=defer, rc=rc, violations=v.value,
                    first=list(first), sequence_matches=bool(same) if prec == lib.PREC_FP64 else None,
                    evals=s.evals))
    d.close()
    h.close()
print("RESULT " + json.dumps(out))
'''


def test_bounds_checked_build_records_no_violation():
    from pngf_gb300 import build
    if not os.path.exists(build.LIB_BC):
        build.build(bounds_check=True)
    env = dict(os.environ, PNGF_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("RESULT ")][-1]
    res = json.loads(line[len("RESULT "):])
    assert len(res) == 5
    for x in res:
        assert x["rc"] == 0, x
        assert x["violations"] == 0, x
        assert x["evals"] > 0
        if x["sequence_matches"] is not None:
            assert x["sequence_matches"], x
