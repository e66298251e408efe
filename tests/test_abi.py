"""The C-ABI library: it loads, exports every function the public header
declares, and fails cleanly (status codes, no crash) without a GPU or on bad
arguments. No compute call needs a GPU here."""
import ctypes as C

import pytest
import torch

from pngf_gb300 import lib


def test_exports_every_header_symbol(built_lib):
    names = lib.header_symbols()
    assert len(names) >= 29
    for n in names:
        assert hasattr(built_lib, n), n


def test_config_default_matches_reference_constants(built_lib):
    cfg = lib.Config()
    fr = (C.c_double * 16)(25e9, 27.5e9, 30e9, 32.5e9, 35e9)
    built_lib.pngf_config_default(C.byref(cfg), 21, 21, 5, fr)
    assert (cfg.cells_x, cfg.cells_y, cfg.num_eobj, cfg.max_flips) == (3, 3, 3, 4)
    assert cfg.dx == 0.01 / 60.0 and cfg.dz == 0.01 / 180.0
    assert lib.num_edges(21, 21) == 8064 and lib.num_edges(7, 7) == 924 and lib.num_edges(41, 41) == 30504


def test_create_rejects_bad_config(built_lib):
    cfg = lib.Config()
    built_lib.pngf_config_default(C.byref(cfg), 21, 21, 1, None)
    h = C.c_void_p()
    bad = lib.Config.from_buffer_copy(cfg)
    bad.num_freq = 0
    assert built_lib.pngf_create(C.byref(bad), C.byref(h)) == 1
    bad = lib.Config.from_buffer_copy(cfg)
    bad.tiles_x = 2
    assert built_lib.pngf_create(C.byref(bad), C.byref(h)) == 1
    assert built_lib.pngf_create(None, C.byref(h)) == 1


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU path")
def test_create_without_gpu_reports_no_device(built_lib):
    with pytest.raises(lib.PngfError) as e:
        lib.Handle(7, 7, [30e9])
    assert e.value.code == 9


def test_null_handle_calls_are_errors(built_lib):
    assert built_lib.pngf_prepare(None) == 1
    assert built_lib.pngf_accept(None, 0) == 1
    assert built_lib.pngf_destroy(None) == 0


def test_struct_layouts_match_header(tmp_path):
    """Every public struct's ctypes mirror has the size and field offsets the
    C compiler gives the header's declaration (fields appended to a struct
    keep callers compiled against it in step with the library)."""
    import os
    import shutil
    import subprocess

    from conftest import ROOT
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not found")
    structs = {"pngf_config": lib.Config, "pngf_dbs_params": lib.DbsParams, "pngf_dbs_stats": lib.DbsStats,
               "pngf_timing": lib.Timing, "pngf_tune": lib.Tune, "pngf_group_stats": lib.GroupStats}
    src = ['#include <stddef.h>', '#include <stdio.h>', '#include "pngf_gb300.h"', "int main(void) {"]
    for cname, cls in structs.items():
        src.append('  printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in cls._fields_:
            src.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    src += ["  return 0;", "}"]
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.run([gcc, "-std=c11", "-I" + os.path.join(ROOT, "include"), str(c), "-o", exe], check=True)
    got = dict(line.split() for line in subprocess.run([exe], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for cname, cls in structs.items():
        assert int(got[cname]) == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got["%s.%s" % (cname, fname)]) == getattr(cls, fname).offset, (cname, fname)
