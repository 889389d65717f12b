"""Event times past 2^30 - 2, up to 2^32 - 2 (the 32-bit times of the
reference GPU tool, src/simulate.cuh:36): such a window runs in 64-bit
event words.  Bit-exact against the oracle (64-bit times throughout) on
every waveform and SAIF count:

* a stimulus already past 2^30 - 2 is packed in 64-bit words when the
  window is added;
* a stimulus within 2^30 - 2 whose gate outputs pass it runs in 32-bit
  words first, then again in 64-bit words;
* times right below 2^32 - 2, and SAIF windows that reach past 2^32;
* wide windows inside a batched run (each runs alone, the others in waves);
* an output past 2^32 - 2 is GLS_ERANGE, and the context stays usable."""
import numpy as np
import pytest

from cases import random_case, stimulus
from gls.capi import GlsError, Simulator
from gls.levelize import assemble
from gls.netlist import Stimulus
from gpu_util import assert_same, gpu_run
from oracle.runner import run_oracle

pytestmark = pytest.mark.gpu

NARROW_MAX = (1 << 30) - 2
WIDE_MAX = (1 << 32) - 2
HORIZON = 600
SPAN = HORIZON + 16 * 80 + 8   # the stimulus horizon plus the longest path (16 gates, delays below 80)


def shifted(st: Stimulus, base: int) -> Stimulus:
    t = st.time.astype(np.uint64) + np.uint64(base)
    assert int(t.max(initial=0)) <= WIDE_MAX
    return Stimulus(st.nets.copy(), st.ev_start.copy(), t.astype(np.uint32), st.value.copy())


def base_for(where: str, st: Stimulus) -> int:
    if where == "stimulus":
        return 3_000_000_000
    if where == "outputs":   # the last stimulus event lands on 2^30 - 2 exactly
        return NARROW_MAX - int(st.time.max(initial=0))
    return WIDE_MAX - SPAN   # "top"


def crosses(ow) -> bool:
    return any(len(t) and int(np.max(t)) > NARROW_MAX for t, _ in ow.values())


@pytest.mark.parametrize("mask", [7, 0])
@pytest.mark.parametrize("where", ["stimulus", "outputs", "top"])
@pytest.mark.parametrize("seed", range(6))
def test_gpu_wide_times_vs_oracle(seed, where, mask, gpu, oracle_bin):
    nl, st0 = random_case(seed, max_gates=16, max_in=6, horizon=HORIZON, max_events=80)
    base = base_for(where, st0)
    st = shifted(st0, base)
    seg = (8, 13, 0)[seed % 3]
    for t_begin, t_end in ((base, base + SPAN + 50), (0, 1 << 33), (base + HORIZON // 2, (1 << 32) + 7)):
        ow, osaif, _ = run_oracle(nl, st, t_begin, t_end)
        gw, gs, _, stats = gpu_run(nl, st, t_begin, t_end, seg=seg, warp_mask=mask)
        assert_same(gw, gs, ow, osaif, f"{where} seed {seed} window [{t_begin}, {t_end})")
        # 64-bit words exactly when some time passes 2^30 - 2
        want = where != "outputs" or crosses(ow)
        assert stats["wide_windows"] == (1 if want else 0), (where, seed)


@pytest.mark.parametrize("alloc", [1, 0])
def test_gpu_wide_windows_in_a_batched_run(alloc, gpu, oracle_bin):
    """Windows of 32- and 64-bit words mixed in one batched run: each gives
    the oracle's result."""
    nl, st0 = random_case(7, max_gates=16, max_in=6, horizon=HORIZON, max_events=80)
    plan = [(0, (0, 700)), (3_000_000_000, None), (0, (100, 650)), (WIDE_MAX - SPAN, None),
            (NARROW_MAX - int(st0.time.max(initial=0)), None), (0, (0, 900))]
    cases = []
    for base, win in plan:
        st = shifted(st0, base)
        b, e = win if win else (base, base + SPAN)
        cases.append((st, b, e, run_oracle(nl, st, b, e)))
    with Simulator(alloc_mode=alloc) as s:
        s.load(nl)
        ids = [s.add_window(st, b, e) for st, b, e, _ in cases]
        s.run_batched(use_graph=True)
        stats = s.stats()
        for k, (wid, (_, b, e, (ow, osaif, _))) in enumerate(zip(ids, cases)):
            lens = s.lengths(wid)
            gw = {n: s.waveform(n, wid) for n in range(nl.n_nets) if lens[n] != 2**32 - 1}
            assert_same(gw, s.saif(wid), ow, osaif, f"batched window {k}")
    assert stats["wide_windows"] >= 2


def test_gpu_output_past_the_time_range(gpu, oracle_bin):
    """An inverter of delay 10 fed at 2^32 - 5: its output would land past
    2^32 - 2, which is GLS_ERANGE; a stimulus time of 2^32 - 1 is refused
    when the window is added.  The context stays usable after both."""
    nl = assemble([("GEN_INV_D1", [0], [1], [(2, "i", "zn", 10, 10)])])
    with Simulator() as s:
        s.load(nl)
        bad = stimulus({0: [(0, 0), (5, 3)]})
        bad.time[1] = (1 << 32) - 1
        with pytest.raises(GlsError, match="largest event time"):
            s.add_window(bad, 0, 10)
        late = stimulus({0: [(0, 0), (5, 3)]})
        late.time[1] = (1 << 32) - 5
        s.add_window(late, 0, 1 << 32)
        with pytest.raises(GlsError) as e:
            s.run()
        assert e.value.code == 5 and "largest event time" in str(e.value)   # GLS_ERANGE
        s.clear_windows()
        ok = stimulus({0: [(0, 0), (5, 3)]})
        ok.time[1] = WIDE_MAX - 10   # the output lands on 2^32 - 2 exactly
        w = s.add_window(ok, 0, 1 << 32)
        s.run()
        ow, osaif, _ = run_oracle(nl, ok, 0, 1 << 32)
        gw = {n: s.waveform(n, w) for n in range(nl.n_nets)}
        assert_same(gw, s.saif(w), ow, osaif, "output at 2^32 - 2")
        assert int(gw[1][0][-1]) == WIDE_MAX
