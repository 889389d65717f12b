"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference's golden vectors, bit-exact on every waveform and SAIF count."""
import json
from pathlib import Path

import numpy as np
import pytest

from cases import random_case, stimulus
from gls import synth
from gls.capi import CALC_FIXED, CALC_LITERAL, GlsError, Simulator
from gls.levelize import assemble
from gpu_util import assert_same, gpu_run, waveform_properties
from oracle.runner import run_oracle

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def golden_cases():
    return json.loads((GOLD / "cases.json").read_text())


@pytest.mark.parametrize("seg", [8, 0])
@pytest.mark.parametrize("idx", range(len(golden_cases())))
def test_gpu_matches_golden(idx, seg, gpu):
    r = golden_cases()[idx]
    insts = [(c, ins, outs, [tuple(a) for a in arcs]) for c, ins, outs, arcs in r["instances"]]
    nl = assemble(insts, n_nets=r["n_nets"])
    st = stimulus({int(k): [tuple(e) for e in v] for k, v in r["stimulus"].items()})
    calc = CALC_LITERAL if r["calc"] == "literal" else CALC_FIXED
    gw, gs, _, _ = gpu_run(nl, st, *r["window"], calc=calc, seg=seg)
    for net, ev in r["waves"].items():
        exp = np.array(ev, np.int64).reshape(-1, 2)
        t, v = gw[int(net)]
        assert np.array_equal(t.astype(np.int64), exp[:, 0]) and np.array_equal(v.astype(np.int64), exp[:, 1]), \
            f"{r['label']}: net {net}"
    for net, rec in r["saif"].items():
        assert gs[int(net)].tolist() == rec, f"{r['label']}: SAIF net {net}"


@pytest.mark.parametrize("mask", [7, 0])
@pytest.mark.parametrize("seg", [8, 13, 256])
@pytest.mark.parametrize("seed", range(16))
def test_gpu_random_vs_oracle(seed, seg, mask, gpu, oracle_bin):
    """Random small designs; mask 7 runs the 1-3 input gates warp-per-segment,
    mask 0 thread-per-segment."""
    nl, st = random_case(seed, max_gates=16, max_in=6, horizon=600, max_events=80,
                         zero_delay=(seed % 5 == 0))
    calc = "literal" if seed % 4 == 3 else "fixed"
    try:
        ow, osaif, _ = run_oracle(nl, st, 0, 700, calc=calc)
    except Exception:
        pytest.skip("oracle rejects this case (zero delay at time 0)")
    gw, gs, _, _ = gpu_run(nl, st, 0, 700, calc=CALC_LITERAL if calc == "literal" else CALC_FIXED, seg=seg,
                           warp_mask=mask)
    assert_same(gw, gs, ow, osaif, f"seed {seed} seg {seg} mask {mask}")


@pytest.mark.parametrize("seed", range(4))
def test_gpu_dense_random_vs_oracle(seed, gpu, oracle_bin):
    """Many gates and long lists: every level has several segments per gate."""
    nl, st = random_case(900 + seed, max_gates=120, max_in=8, horizon=20000, max_events=2000, xz=seed % 2 == 0)
    ow, osaif, _ = run_oracle(nl, st, 100, 15000, threads=4)
    for seg, mask in ((16, 7), (512, 7), (200, 0), (0, 7), (0, 0)):
        gw, gs, _, _ = gpu_run(nl, st, 100, 15000, seg=seg, warp_mask=mask)
        assert_same(gw, gs, ow, osaif, f"dense seed {seed} seg {seg} mask {mask}")


def test_gpu_pool_offsets_past_2_34_events(gpu, oracle_bin):
    """Gate outputs placed past 2^34 events (64 GiB) into the pool: list
    offsets and 16-byte chunk indexes need 64 bits there (the full large
    configuration's pool reaches 4.2e10 events)."""
    nl, st = random_case(950, max_gates=120, max_in=8, horizon=20000, max_events=2000)
    ow, osaif, _ = run_oracle(nl, st, 100, 15000, threads=4)
    gap = {"GLS_POOL_GAP_EVENTS": str((1 << 34) + 4)}
    for seg, mask in ((16, 0), (0, 0), (0, 7)):
        gw, gs, _, stats = gpu_run(nl, st, 100, 15000, seg=seg, warp_mask=mask, env=gap)
        assert stats["pool_events"] > 1 << 34
        assert_same(gw, gs, ow, osaif, f"gap seg {seg} mask {mask}")


@pytest.mark.parametrize("knobs", [{"GLS_SIM_CONCURRENT": "0"}, {"GLS_SIM_PIPELINE": "0"}, {"GLS_PLAN_OVERLAP": "0"},
                                   {"GLS_COPY_LANES": "4"}, {"GLS_COPY_LANES": "16"}, {"GLS_COPY_LANES": "32"},
                                   {"profile": True}, {"schedule": (512, 7, 0)}, {"schedule": (8192, 1, 1)},
                                   {"schedule": (2048, 0, 1)}, {"schedule": (2048, 0, 2)}, {"schedule": (1024, 0, 4)},
                                   {"schedule": (4096, 1, 6)}, {"schedule": (256, 0, 7)}])
def test_gpu_schedules_and_streams_agree(knobs, gpu, oracle_bin):
    """Results never depend on how a level is scheduled: fan-in classes in
    turn or concurrently, link and copy per class or per level, the next
    level's plan beside the copies or after them, lanes per copied segment,
    profiled runs, segments per SM, warp-per-segment classes, the gate
    kernel's block size (flag 2) and load width (flag 4)."""
    nl, st = random_case(960, max_gates=120, max_in=8, horizon=20000, max_events=2000)
    ow, osaif, _ = run_oracle(nl, st, 100, 15000, threads=4)
    env = {k: v for k, v in knobs.items() if k.startswith("GLS_")}
    from gpu_util import simulator
    with simulator(None, env, profile=bool(knobs.get("profile"))) as s:
        if "schedule" in knobs:
            s.set_schedule(*knobs["schedule"])
        s.load(nl)
        w = s.add_window(st, 100, 15000)
        s.run()
        gw = {n: s.waveform(n, w) for n in ow}
        assert_same(gw, s.saif(w), ow, osaif, str(knobs))


def test_gpu_c1_full_config(gpu, oracle_bin):
    """The small benchmark configuration end to end: 2,000 cells, depth 20,
    192 pseudo-primary inputs, 1,000 cycles, window 0..1,000,000 ps."""
    cfg = synth.CONFIGS["c1"]
    nl = synth.make_netlist(cfg, seed=1)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=2)
    ow, osaif, _ = run_oracle(nl, st, 0, cfg.t_end, threads=8)
    gw, gs, _, stats = gpu_run(nl, st, 0, cfg.t_end)
    assert_same(gw, gs, ow, osaif, "c1")
    assert stats["gate_events"] > 0 and stats["output_events"] > 0


def test_gpu_c2_shape_scaled(gpu, oracle_bin):
    """The medium configuration's generator at 20,000 cells and 1,500 cycles."""
    cfg = synth.scaled(synth.CONFIGS["c2"], cells=20_000, cycles=1_500)
    nl = synth.make_netlist(cfg, seed=3)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=4)
    ow, osaif, _ = run_oracle(nl, st, 0, cfg.t_end, threads=16)
    gw, gs, _, _ = gpu_run(nl, st, 0, cfg.t_end)
    assert_same(gw, gs, ow, osaif, "c2-scaled")


def test_gpu_segment_size_invariance_and_properties(gpu):
    cfg = synth.scaled(synth.CONFIGS["c3"], cells=30_000, cycles=3_000, depth=40, ppi=2048)
    nl = synth.make_netlist(cfg, seed=5)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=6)
    driven = set(nl.gate_output_nets().tolist())
    a = gpu_run(nl, st, 0, cfg.t_end, seg=32)
    b = gpu_run(nl, st, 0, cfg.t_end, seg=4096)
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[1], b[1])
    for n in a[0]:
        assert np.array_equal(a[0][n][0], b[0][n][0]) and np.array_equal(a[0][n][1], b[0][n][1])
    waveform_properties(a[0], a[1], 0, cfg.t_end, driven)


def test_gpu_window_inside_activity(gpu, oracle_bin):
    nl, st = random_case(31, max_gates=30, max_in=5, horizon=5000, max_events=300)
    for tb, te in [(1000, 1001), (1234, 4321), (0, 1), (4999, 9000)]:
        ow, osaif, _ = run_oracle(nl, st, tb, te)
        gw, gs, _, _ = gpu_run(nl, st, tb, te)
        assert_same(gw, gs, ow, osaif, f"window {tb}..{te}")


def test_gpu_empty_and_constant_inputs(gpu, oracle_bin):
    # net 0 has no events at all (reads X), net 1 is a constant, net 2 toggles
    nl = assemble([("GEN_AND2_D1", [0, 2], [3], [(2, "a1", "z", 5, 7), (2, "a2", "z", 9, 11)]),
                   ("GEN_OR2_D1", [1, 2], [4], [(2, "a1", "z", 5, 7), (2, "a2", "z", 9, 11)]),
                   ("GEN_MUX2_D1", [3, 4, 1], [5], [(2, "i0", "z", 3, 4), (2, "i1", "z", 5, 6),
                                                   (0, "s", "z", 7, 8), (1, "s", "z", 9, 10)])])
    st = stimulus({0: [], 1: [(0, 3)], 2: [(0, 0), (100, 3), (105, 0), (300, 3)]})
    ow, osaif, _ = run_oracle(nl, st, 0, 1000)
    gw, gs, _, _ = gpu_run(nl, st, 0, 1000)
    assert_same(gw, gs, ow, osaif, "empty/constant")


def test_gpu_rejects_bad_input(gpu):
    nl = assemble([("GEN_INV_D1", [0], [1], [(2, "i", "zn", 5, 5)])])
    with Simulator() as s:
        s.load(nl)
        with pytest.raises(GlsError):          # read net 0 has no stimulus
            s.add_window(stimulus({}), 0, 10)
        with pytest.raises(GlsError):          # times must strictly increase
            s.add_window(stimulus({0: [(0, 0), (5, 3), (5, 0)]}), 0, 10)
        with pytest.raises(GlsError):          # the stimulus cannot drive a gate output
            s.add_window(stimulus({0: [(0, 0)], 1: [(0, 0)]}), 0, 10)
        with pytest.raises(GlsError):          # empty window
            s.add_window(stimulus({0: [(0, 0)]}), 10, 10)
        with pytest.raises(GlsError):          # not simulated yet
            s.saif(0)


def test_gpu_saif_table_matches_counts(gpu, oracle_bin):
    """The interleaved SAIF table and the three-array call read the same counts."""
    nl, st = random_case(7, max_gates=24, max_in=4, horizon=900, max_events=120)
    ow, osaif, _ = run_oracle(nl, st, 0, 1000)
    with Simulator() as s:
        s.load(nl)
        w = s.add_window(st, 0, 1000)
        s.run()
        t3 = s.saif(w)
        t0, t1, tx = s.saif_counts(w)
    assert t3.shape == (nl.n_nets, 3)
    assert np.array_equal(t3, np.stack([t0, t1, tx], axis=1))
    done = t3[:, 0] != np.iinfo(np.uint64).max
    assert np.array_equal(t3[done], osaif[done])


def test_gpu_rejects_bad_stimulus_values(gpu):
    """A value above 3 or a time of 2^32-1 is refused when the window is added."""
    nl = assemble([("GEN_INV_D1", [0], [1], [(2, "i", "zn", 5, 5)])])
    with Simulator() as s:
        s.load(nl)
        bad_v = stimulus({0: [(0, 0), (5, 3)]})
        bad_v.value[1] = 7
        with pytest.raises(GlsError, match="value above 3"):
            s.add_window(bad_v, 0, 10)
        bad_t = stimulus({0: [(0, 0), (5, 3)]})
        bad_t.time[1] = (1 << 32) - 1
        with pytest.raises(GlsError, match="largest event time"):
            s.add_window(bad_t, 0, 10)
        s.add_window(stimulus({0: [(0, 0), (5, 3)]}), 0, 10)   # the context stays usable


def test_gpu_pool_regrowth(gpu, oracle_bin):
    """A deliberately tiny initial event pool must grow and give the same result."""
    nl, st = random_case(44, max_gates=40, max_in=4, horizon=4000, max_events=400)
    ow, osaif, _ = run_oracle(nl, st, 0, 4000)
    gw, gs, _, stats = gpu_run(nl, st, 0, 4000, pool_events=64)
    assert stats["overflow_retries"] >= 1
    assert_same(gw, gs, ow, osaif, "regrowth")


@pytest.mark.parametrize("seg", [0, 8, 13])
@pytest.mark.parametrize("calc", [CALC_FIXED, CALC_LITERAL])
def test_gpu_controlled_inputs(seg, calc, gpu, oracle_bin):
    """Gates whose output a slow input controls (NAND/NOR/AND/OR at their
    controlling value, AOI/OAI, a mux select) fed a fast input whose events
    the kernels read past while the output cannot change: long runs, events
    at the very time the slow input changes, X and Z on both, segments that
    cut through the runs."""
    cells = [("GEN_NAND2_D1", 2), ("GEN_NOR3_D1", 3), ("GEN_AND2_D1", 2), ("GEN_OR2_D1", 2), ("GEN_AOI21_D1", 3),
             ("GEN_OAI21_D1", 3), ("GEN_MUX2_D1", 3), ("GEN_XOR2_D1", 2)]
    from gls.cells import LIBRARY
    insts = []
    n_in = 3
    for k, (name, n) in enumerate(cells):
        c = LIBRARY[name]
        ins = [0, 1, 2][:n] if k % 2 == 0 else [1, 0, 2][:n]
        arcs = [(e, i, o, float(5 + 3 * k), float(7 + 2 * k)) for e, i, o in c.arcs]
        insts.append((name, ins, [n_in + k], arcs))
    nl = assemble(insts, n_nets=n_in + len(cells))
    rng = np.random.default_rng(11)
    slow = [(t, int(v)) for t, v in zip(range(0, 20000, 1000), rng.choice([0, 3, 0, 3, 1], 20))]
    fast_t = sorted(set(rng.integers(0, 20000, 1500).tolist()) | {1000, 3000, 7000, 12000})
    fast = [(t, int(v)) for t, v in zip(fast_t, rng.choice([0, 3, 0, 3, 1, 2], len(fast_t)))]
    mid_t = sorted(set(rng.integers(0, 20000, 300).tolist()) | {3000, 12000})
    mid = [(t, int(v)) for t, v in zip(mid_t, rng.choice([0, 3, 2], len(mid_t)))]
    st = stimulus({0: slow, 1: fast, 2: mid})
    cn = "literal" if calc == CALC_LITERAL else "fixed"
    ow, osaif, _ = run_oracle(nl, st, 0, 21000, calc=cn)
    gw, gs, _, _ = gpu_run(nl, st, 0, 21000, calc=calc, seg=seg, warp_mask=0)
    assert_same(gw, gs, ow, osaif, f"controlled inputs seg {seg} calc {cn}")
