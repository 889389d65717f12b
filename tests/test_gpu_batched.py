"""GPU tests of batched windows: every window of a wave gives exactly what
it gives when run alone (and what the oracle gives), with and without the
captured launch graph, in waves of any size, in every allocation mode, and
when one window of a wave outgrows its pool."""
import numpy as np
import pytest

from cases import random_case
from gls import synth
from gls.capi import ALLOC_BOUND, ALLOC_EXACT, ALLOC_LEARNED, MLP_PARAMS, Simulator
from gpu_util import assert_same
from oracle.runner import run_oracle

pytestmark = pytest.mark.gpu


def windows_of(cfg, nl, seeds, lengths):
    out = []
    for s, cyc in zip(seeds, lengths):
        c = synth.scaled(cfg, cycles=cyc)
        out.append((synth.make_stimulus(c, nl.ppi_nets, seed=s), c.t_end))
    return out


def run_all(nl, wins, batched=None, alloc=ALLOC_BOUND, model=None, pool_events=0):
    with Simulator(alloc_mode=alloc, pool_events=pool_events) as s:
        if model is not None:
            s.set_presize_model(model)
        s.load(nl)
        ids = [s.add_window(st, 0, t_end) for st, t_end in wins]
        if batched is None:
            s.run()
        else:
            s.run_batched(**batched)
        res = [(s.lengths(w), s.saif(w)) for w in ids]
        waves = None
        if batched is None or not batched.get("saif_only"):
            drv = nl.gate_output_nets()[:200]
            waves = [{int(n): s.waveform(int(n), w) for n in drv} for w in ids]
        return res, waves, s.stats()


@pytest.fixture(scope="module")
def design():
    cfg = synth.scaled(synth.CONFIGS["c2"], cells=6_000, cycles=300, depth=16, ppi=512)
    nl = synth.make_netlist(cfg, seed=21)
    wins = windows_of(cfg, nl, seeds=[31, 32, 33, 34, 35, 36, 37], lengths=[300, 40, 900, 120, 300, 10, 500])
    return nl, wins


@pytest.mark.parametrize("opts", [dict(max_wave=0, use_graph=True), dict(max_wave=0, use_graph=False),
                                  dict(max_wave=3, use_graph=True), dict(max_wave=1, use_graph=True),
                                  dict(max_wave=2, use_graph=True, saif_only=True)])
def test_batched_equals_sequential(design, opts, gpu):
    nl, wins = design
    ref, ref_waves, ref_stats = run_all(nl, wins)
    got, waves, stats = run_all(nl, wins, batched=opts)
    for k, ((la, sa), (lb, sb)) in enumerate(zip(ref, got)):
        assert np.array_equal(la, lb) and np.array_equal(sa, sb), f"window {k}"
    if waves is not None:
        for a, b in zip(ref_waves, waves):
            for n in a:
                assert np.array_equal(a[n][0], b[n][0]) and np.array_equal(a[n][1], b[n][1])
    assert stats["gate_events"] == ref_stats["gate_events"]
    assert stats["output_events"] == ref_stats["output_events"]


def test_batched_saif_only_drops_waveforms(design, gpu):
    nl, wins = design
    with Simulator() as s:
        s.load(nl)
        for st, t_end in wins[:3]:
            s.add_window(st, 0, t_end)
        s.run_batched(saif_only=True)
        assert s.lengths(1).max() > 0
        with pytest.raises(Exception, match="saif_only"):
            s.waveform(int(nl.gate_output_nets()[0]), 1)
        s.run()   # runs again from the kept stimulus, waveforms back
        assert s.waveform(int(nl.gate_output_nets()[0]), 1) is not None


@pytest.mark.parametrize("alloc", [ALLOC_EXACT, ALLOC_LEARNED])
def test_batched_allocation_modes(design, alloc, gpu):
    nl, wins = design
    model = None
    if alloc == ALLOC_LEARNED:
        model = np.zeros(MLP_PARAMS, np.float32)
        model[-1] = 3.0   # short for busy gates: some fall back to exact placement
    ref, _, _ = run_all(nl, wins)
    got, _, stats = run_all(nl, wins, batched=dict(max_wave=4, use_graph=True), alloc=alloc, model=model)
    for (la, sa), (lb, sb) in zip(ref, got):
        assert np.array_equal(la, lb) and np.array_equal(sa, sb)
    if alloc == ALLOC_LEARNED:
        assert stats["presize_overflows"] > 0


def test_batched_pool_regrowth_inside_a_wave(design, gpu):
    """A pool far too small: every window of the wave overflows and is rerun alone."""
    nl, wins = design
    ref, _, _ = run_all(nl, wins[:4])
    got, _, stats = run_all(nl, wins[:4], batched=dict(max_wave=4, use_graph=True), pool_events=50_000)
    for (la, sa), (lb, sb) in zip(ref, got):
        assert np.array_equal(la, lb) and np.array_equal(sa, sb)


def test_batched_random_cases_vs_oracle(gpu, oracle_bin):
    nl, st0 = random_case(801, max_gates=50, max_in=6, horizon=4000, max_events=300)
    stims = [st0] + [random_case(801 + k, max_gates=50, max_in=6, horizon=4000, max_events=300)[1] for k in (1, 2)]
    # the other seeds draw other netlists: keep only stimuli on this netlist's inputs
    stims = [st for st in stims if np.array_equal(np.sort(st.nets), np.sort(st0.nets))] or [st0]
    with Simulator() as s:
        s.load(nl)
        ids = [s.add_window(st, 0, 5000) for st in stims] + [s.add_window(st0, 100, 3000)]
        s.run_batched(use_graph=True)
        for w, (st, tb, te) in zip(ids, [(st, 0, 5000) for st in stims] + [(st0, 100, 3000)]):
            ow, osaif, _ = run_oracle(nl, st, tb, te)
            gw = {n: s.waveform(n, w) for n in ow}
            assert_same(gw, s.saif(w), ow, osaif, f"window {w}")


def test_autotune_keeps_results(design, gpu):
    nl, wins = design
    ref, _, _ = run_all(nl, wins)
    with Simulator() as s:
        s.load(nl)
        ids = [s.add_window(st, 0, t_end) for st, t_end in wins]
        t = s.autotune(max_wave=4)
        # 9 in the first stage, 4 flag sets on the best of them
        assert len(t["candidates"]) == 13 and t["windows"] == 4
        first = t["candidates"][:9]
        stage1 = min(first, key=lambda c: c["ms"])
        assert all(c["flags"] == 0 for c in first)
        assert [c["flags"] for c in t["candidates"][9:]] == [1, 2, 4, 6]
        assert all((c["seg_per_sm"], c["warp_mask"]) == (stage1["seg_per_sm"], stage1["warp_mask"])
                   for c in t["candidates"][9:])
        assert t["best"]["ms"] == min(c["ms"] for c in t["candidates"])
        s.run_batched(max_wave=4)
        for w, (la, sa) in zip(ids, ref):
            assert np.array_equal(s.lengths(w), la) and np.array_equal(s.saif(w), sa)
