"""The device-resident DBS loop (pngf_dbs_set_device_loop) against the
reference's golden logs and the host driver.

The hat's draws (std::mt19937 and std::uniform_int_distribution restated in
pngf_gb300/csrc/hat_rng.h) and every decision without an accept run on the
GPU inside one CUDA graph with a WHILE node; accepts return to the host.
Bar: the host driver's -- identical flip sequence, accept decisions and final
design as the reference, logged objectives within 1e-10 relative -- and, on
the same inputs, a log, counters and design equal to the host driver's bit
for bit (both take the same kernels in the same order)."""
import numpy as np
import pytest

from conftest import case_G, golden_log
from test_gpu_parity import compare_log

pytestmark = pytest.mark.gpu


def run(c, Gs, gobj, device, batch=0, max_evals=None, precision=None, drift_every=0, drift_tol=0.0):
    from pngf_gb300 import lib
    prec = lib.PREC_FP64 if precision is None else precision
    h = lib.Handle(c["tiles"], c["tiles"], c["freqs"], precision=prec, max_flips=4 if c["mode"] == "sym" else 1)
    for f, G in enumerate(Gs):
        h.load_G(f, G, gobj[f])
    d = lib.Dbs(h, mode=lib.DBS_SYMMETRIC if c["mode"] == "sym" else lib.DBS_SINGLE,
                init=lib.INIT_RANDOM if c["init"] == "random" else lib.INIT_EMPTY, seed=c["seed"],
                max_evals=c["max_evals"] if max_evals is None else max_evals, batch=batch,
                drift_every=drift_every, drift_tol=drift_tol, device_loop=device)
    s = d.run()
    return h, d, s


def assert_same_run(a, b):
    (ha, da, sa), (hb, db, sb) = a, b
    la, lb = da.log(), db.log()
    for key in ("tile", "accept", "F", "F_best", "perf"):
        assert np.array_equal(la[key], lb[key], equal_nan=True), key
    for key in ("evals", "accepts", "launched", "converged", "F_best", "drift_checks", "refreshes"):
        assert getattr(sa, key) == getattr(sb, key), key
    assert list(ha.tile_map()) == list(hb.tile_map())


@pytest.mark.parametrize("name", ["sym_7x7_f1_seed1", "sym_7x7_f5_empty", "single_7x7_f2_seed1",
                                  "sym_9x9_f2_seed3", "single_11x11_f3_seed2"])
def test_device_loop_matches_reference(name, cases, built_lib):
    c = cases[name]
    Gs, gobj = case_G(c, built_lib)
    h, d, s = run(c, Gs, gobj, True)
    compare_log(d, h, golden_log(name), s)
    assert 0 < s.device_launches <= s.device_decisions


@pytest.mark.parametrize("batch", [1, 5, -2, -16, 0])
def test_device_loop_equals_host_driver(batch, cases, built_lib):
    """11x11 single-tile hat (121 entries): batches above and below the
    small-batch kernel form's limit, fixed, adaptive and whole-hat."""
    c = cases["single_11x11_f3_seed2"]
    Gs, gobj = case_G(c, built_lib)
    host = run(c, Gs, gobj, False, batch=batch)
    dev = run(c, Gs, gobj, True, batch=batch)
    assert_same_run(host, dev)
    s = dev[2]
    # decisions without an accept stayed on the device (with whole-hat batches
    # a decision without an accept happens only at convergence, which this
    # 300-evaluation run may not reach)
    assert s.device_decisions > s.accepts if batch != 0 else s.device_decisions >= s.accepts


@pytest.mark.parametrize("max_evals", [1, 37, 250])
def test_device_loop_evaluation_budget(max_evals, cases, built_lib):
    c = cases["sym_9x9_f2_seed3"]
    Gs, gobj = case_G(c, built_lib)
    host = run(c, Gs, gobj, False, batch=-4, max_evals=max_evals)
    dev = run(c, Gs, gobj, True, batch=-4, max_evals=max_evals)
    assert_same_run(host, dev)
    assert dev[2].evals == min(max_evals, host[2].evals)


def test_device_loop_complex64_with_refreshes(cases, built_lib):
    """Complex64 state with a drift check after every second accept and a
    tolerance that forces rebuilds: the host's new F_best reaches the device."""
    from pngf_gb300 import lib
    c = cases["single_11x11_f3_seed2"]
    Gs, gobj = case_G(c, built_lib)
    host = run(c, Gs, gobj, False, batch=-8, max_evals=400, precision=lib.PREC_C64, drift_every=2, drift_tol=1e-12)
    dev = run(c, Gs, gobj, True, batch=-8, max_evals=400, precision=lib.PREC_C64, drift_every=2, drift_tol=1e-12)
    assert host[2].refreshes > 0
    assert_same_run(host, dev)


def test_device_loop_api_rules(cases, built_lib):
    from pngf_gb300 import lib
    c = cases["single_7x7_f2_seed1"]
    Gs, gobj = case_G(c, built_lib)
    h = lib.Handle(7, 7, c["freqs"], max_flips=1)
    for f, G in enumerate(Gs):
        h.load_G(f, G, gobj[f])
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, seed=1, batch=-4)
    d.step()
    with pytest.raises(lib.PngfError) as e:
        d.set_device_loop(True)
    assert e.value.code == 6  # PNGF_ERR_STATE: chosen before the first step
    d.close()
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, seed=1, batch=-4, device_loop=True)
    prop = lib.Proposal(h, seed=1)
    with pytest.raises(lib.PngfError) as e:
        lib.dbs_set_proposal(d, prop, topk=0)
    assert e.value.code == 8  # PNGF_ERR_UNSUPPORTED
    # a group's members all run device-resident decisions or none does
    h2 = lib.Handle(7, 7, c["freqs"], max_flips=1)
    for f, G in enumerate(Gs):
        h2.load_G(f, G, gobj[f])
    d2 = lib.Dbs(h2, mode=lib.DBS_SINGLE, seed=2, batch=-4)
    with pytest.raises(lib.PngfError) as e:
        lib.Group([d, d2])
    assert e.value.code == 8


@pytest.mark.parametrize("device", [False, True])
def test_timed_out_update_is_reported(device, cases, built_lib):
    """An accept update whose bounded waits gave up (the error flag it leaves,
    set here from the host) stops both drivers with PNGF_ERR_TIMEOUT before
    they decide on the state it left; the handle stays usable."""
    from pngf_gb300 import lib
    c = cases["single_7x7_f2_seed1"]
    Gs, gobj = case_G(c, built_lib)
    h = lib.Handle(7, 7, c["freqs"], max_flips=1)
    for f, G in enumerate(Gs):
        h.load_G(f, G, gobj[f])
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, seed=1, batch=-4, device_loop=device)
    assert d.step()
    rows = len(d.log()["tile"])
    h.inject_update_timeout(21)
    with pytest.raises(lib.PngfError) as e:
        d.step()
    assert e.value.code == 7  # PNGF_ERR_TIMEOUT
    assert len(d.log()["tile"]) == rows
    d.close()
    h.prepare()
    eo, F = h.eval_candidates([[3], [10]])
    assert np.all(np.isfinite(F))
