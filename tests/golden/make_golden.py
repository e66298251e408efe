"""Regenerates the golden DBS logs in this directory from the reference itself.

Builds the reference optimizer from its own sources (oracle/Makefile target
``ref``, which compiles pngf-opt/{pngfopt,linalg,magichat,acmetime}.hpp in
place from the reference tree), writes synthetic G files in the acmefdfd
layout with the oracle's generator (oracle/synth.c: G plus the two NF2FF
rows, so that the directivity half of the objective and the far-field rows of
R are exercised), runs the reference DBS on each case and copies its log here.
``cases.json`` records each case and checksums of the G matrices and NF2FF
rows it used, so that a test can confirm the generators reproduce them.

Usage: python tests/golden/make_golden.py --ref <reference tree> [--only NAME ...]
(or set PNGF_REFERENCE). The 21x21 x 5-frequency case needs about 15 GB of
host memory and a few minutes of the reference's OpenBLAS time.
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

from oracle import synth  # noqa: E402

FREQS_REF = [25.0e9, 27.5e9, 30.0e9, 32.5e9, 35.0e9]
FREQS_WIDE = [27.0e9, 28.5e9, 30.0e9, 31.5e9, 33.0e9]

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
    # The benchmarked wideband workload itself: 21x21 tiles (N = 8064), five
    # frequencies 27-33 GHz, single-tile hat, 50%-fill start from seed 1; the
    # first 120 evaluations.
    dict(name="single_21x21_f5_seed1", tiles=21, freqs=FREQS_WIDE, seed=1, init="random", mode="single",
         max_evals=120),
    # The same size in the reference's default candidate set (4-fold mirror
    # hat: flips of 1, 2 or 4 tiles, up to 96 edges): the first 40 evaluations.
    dict(name="sym_21x21_f5_seed1", tiles=21, freqs=FREQS_WIDE, seed=1, init="random", mode="sym", max_evals=40),
]


def g_checksum(G):
    return dict(sum_re=float(G.real.sum()), sum_im=float(G.imag.sum()), sumsq=float((abs(G) ** 2).sum()),
                g00=[float(G[0, 0].real), float(G[0, 0].imag)],
                g_last0=[float(G[-1, 0].real), float(G[-1, 0].imag)])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PNGF_REFERENCE"),
                    help="the reference tree (default: $PNGF_REFERENCE)")
    ap.add_argument("--only", nargs="*", help="regenerate only these cases (cases.json keeps the others)")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref <reference tree> or set PNGF_REFERENCE")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "synth", "REF=" + a.ref], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "pngf_ref")
    meta_path = os.path.join(HERE, "cases.json")
    old = {}
    if a.only and os.path.exists(meta_path):
        old = {c["name"]: c for c in json.load(open(meta_path))}
    meta = []
    for c in CASES:
        if a.only and c["name"] not in a.only:
            if c["name"] in old:
                meta.append(old[c["name"]])
            continue
        with tempfile.TemporaryDirectory() as tmp:
            gfiles, sums = [], []
            rows = synth.synth_gobj(c["tiles"], c["tiles"], seed=1)
            for i, f in enumerate(c["freqs"]):
                G = synth.synth_G(c["tiles"], c["tiles"], f, seed=1)
                p = os.path.join(tmp, "%s_%d.bin" % (c["name"], i))
                synth.write_G_file(p, G, rows)
                gfiles.append(p)
                sums.append(g_checksum(G))
                del G
            cmd = [exe, "--tiles", str(c["tiles"]), str(c["tiles"]), "--freq",
                   ",".join(repr(float(f)) for f in c["freqs"]), "--seed", str(c["seed"]), "--init", c["init"],
                   "--mode", c["mode"], "--max-evals", str(c["max_evals"]),
                   "--log", os.path.join(HERE, c["name"] + ".log")]
            for p in gfiles:
                cmd += ["--gfile", p]
            env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "4"))
            out = subprocess.run(cmd, check=True, capture_output=True, text=True, env=env).stdout
            print(c["name"], out.strip().splitlines()[-1], flush=True)
        meta.append(dict(c, g_seed=1, eps_r=2.25, gobj="synth", g_checksums=sums,
                         gobj_checksum=g_checksum(rows)))
    with open(meta_path, "w") as fh:
        json.dump(meta, fh, indent=1)


if __name__ == "__main__":
    main()
