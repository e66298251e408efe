"""Regenerates the golden DBS logs in this directory from the reference itself.

Builds the reference optimizer from its own sources (oracle/Makefile target
``ref``, which compiles pngf-opt/{pngfopt,linalg,magichat,acmetime}.hpp in
place from the reference tree), writes synthetic G files in the acmefdfd
layout with the library's generator, runs the reference DBS on each case and
copies its log here. ``cases.json`` records each case and checksums of the G
matrices it used, so that a test can confirm the generator reproduces them.

Usage: python tests/golden/make_golden.py [--ref /path/to/reference]
Needs the built libpngf_gb300.so (only its CPU-side G generator is used).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from pngf_gb300 import lib  # noqa: E402

FREQS_REF = [25.0e9, 27.5e9, 30.0e9, 32.5e9, 35.0e9]

CASES = [
    # The CPU-runnable plain case: 7x7 tiles, one frequency at 30 GHz, 50%-fill
    # random start from seed 1, the reference's mirror-symmetric hat, to convergence.
    dict(name="sym_7x7_f1_seed1", tiles=7, freqs=[30e9], seed=1, init="random", mode="sym", max_evals=0),
    # The reference's own defaults (empty start, its RNG seed, its five
    # frequencies) at 7x7.
    dict(name="sym_7x7_f5_empty", tiles=7, freqs=FREQS_REF, seed=-514213645, init="empty", mode="sym",
         max_evals=0),
    # Single-tile candidates, two frequencies.
    dict(name="single_7x7_f2_seed1", tiles=7, freqs=[28e9, 32e9], seed=1, init="random", mode="single",
         max_evals=0),
    dict(name="sym_9x9_f2_seed3", tiles=9, freqs=[27e9, 33e9], seed=3, init="random", mode="sym", max_evals=0),
    # A longer single-tile prefix at 11x11 with three frequencies.
    dict(name="single_11x11_f3_seed2", tiles=11, freqs=[28e9, 30e9, 32e9], seed=2, init="random",
         mode="single", max_evals=300),
]


def g_checksum(G):
    return dict(sum_re=float(G.real.sum()), sum_im=float(G.imag.sum()), sumsq=float((abs(G) ** 2).sum()),
                g00=[float(G[0, 0].real), float(G[0, 0].imag)],
                g_last0=[float(G[-1, 0].real), float(G[-1, 0].imag)])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    a = ap.parse_args()
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + a.ref], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "pngf_ref")
    meta = []
    with tempfile.TemporaryDirectory() as tmp:
        for c in CASES:
            gfiles, sums = [], []
            for i, f in enumerate(c["freqs"]):
                G = lib.synth_G(c["tiles"], c["tiles"], f, seed=1)
                p = os.path.join(tmp, "%s_%d.bin" % (c["name"], i))
                lib.write_G_file(p, G)
                gfiles.append(p)
                sums.append(g_checksum(G))
            cmd = [exe, "--tiles", str(c["tiles"]), str(c["tiles"]), "--freq",
                   ",".join(repr(float(f)) for f in c["freqs"]), "--seed", str(c["seed"]), "--init", c["init"],
                   "--mode", c["mode"], "--max-evals", str(c["max_evals"]),
                   "--log", os.path.join(HERE, c["name"] + ".log")]
            for p in gfiles:
                cmd += ["--gfile", p]
            env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "4"))
            out = subprocess.run(cmd, check=True, capture_output=True, text=True, env=env).stdout
            print(c["name"], out.strip().splitlines()[-1])
            meta.append(dict(c, g_seed=1, eps_r=2.25, g_checksums=sums))
    with open(os.path.join(HERE, "cases.json"), "w") as fh:
        json.dump(meta, fh, indent=1)


if __name__ == "__main__":
    main()
