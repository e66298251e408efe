"""pngf_load_G_file streams an acmefdfd G file to the device in pinned panels
(no host copy of the whole matrix). The state it builds must equal, bit for
bit, the state built from the same G and NF2FF rows passed from host memory
with pngf_load_G; a truncated file must fail with PNGF_ERR_IO and leave the
handle usable."""
import os

import numpy as np
import pytest

from conftest import case_G

pytestmark = pytest.mark.gpu


def test_streamed_file_load_equals_host_load(tmp_path, cases, built_lib):
    from oracle import synth
    from pngf_gb300 import lib
    c = cases["single_11x11_f3_seed2"]
    Gs, gobj = case_G(c, built_lib)
    a = c["tiles"]
    paths = []
    for i, G in enumerate(Gs):
        p = str(tmp_path / ("g%d.bin" % i))
        synth.write_G_file(p, G, gobj[i])
        paths.append(p)
    rng = np.random.default_rng(4)
    tm = [int(v) for v in rng.integers(0, 2, a * a)]
    states = []
    for from_file in (True, False):
        h = lib.Handle(a, a, c["freqs"], max_flips=1)
        for f, G in enumerate(Gs):
            if from_file:
                h.load_G_file(f, paths[f])
            else:
                h.load_G(f, G, gobj[f])
        h.set_tile_map(tm)
        h.set_source_port(a // 2, a // 2, 1, 2)
        h.prepare()
        states.append(([h.get_M(f)[0] for f in range(len(Gs))], h.objective()))
        h.close()
    (Ma, Fa), (Mb, Fb) = states
    assert Fa == Fb
    for x, y in zip(Ma, Mb):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64))


def test_truncated_file_is_io_error(tmp_path, cases, built_lib):
    from oracle import synth
    from pngf_gb300 import lib
    c = cases["sym_7x7_f1_seed1"]
    Gs, gobj = case_G(c, built_lib)
    p = str(tmp_path / "g.bin")
    synth.write_G_file(p, Gs[0], gobj[0])
    n = Gs[0].shape[0]
    with open(p, "r+b") as fh:
        fh.truncate(16 * (n + 2) * (n - 3))
    h = lib.Handle(7, 7, c["freqs"], max_flips=4)
    with pytest.raises(lib.PngfError) as e:
        h.load_G_file(0, p)
    assert e.value.code == 4
    with pytest.raises(lib.PngfError):
        h.load_G_file(0, str(tmp_path / "missing.bin"))
    h.load_G(0, Gs[0], gobj[0])  # still usable
    h.set_tile_map([1] * 49)
    h.set_source_port(3, 3, 1, 2)
    h.prepare()
    assert np.isfinite(h.objective())
    h.close()
    assert os.path.exists(p)
