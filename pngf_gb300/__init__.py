"""pngf_gb300 — GB300 (sm_103a) implementation of the PNGF direct-binary-search
hot path (Woodbury tile-flip evaluation and rank-k accept update over a
numerical Green's function matrix), behind a C ABI (include/pngf_gb300.h).

This Python package is a thin ctypes binding used for tests and
benchmarks; the product is libpngf_gb300.so built from ``csrc/``.
"""
from .lib import (DBS_SINGLE, DBS_SYMMETRIC, INIT_EMPTY, INIT_RANDOM, PREC_C64, PREC_FP64, Dbs, Handle,  # noqa: F401
                  PngfError, load, num_edges, synth_G, write_G_file)

FREQS_REF = (25.0e9, 27.5e9, 30.0e9, 32.5e9, 35.0e9)   # pngf-opt/main.cpp:117
FREQS_WIDEBAND = (27.0e9, 28.5e9, 30.0e9, 31.5e9, 33.0e9)
