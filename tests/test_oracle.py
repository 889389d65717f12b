"""CPU tests: the oracle against the reference's golden vectors, the cell
truth tables of libgls against the reference's calc, and (where the
reference sources are present) the oracle against the reference core on
fresh random cases."""
import json
from pathlib import Path

import numpy as np
import pytest

from cases import random_case, stimulus
from gls.capi import CALC_FIXED, CALC_LITERAL, cell_lut
from gls.cells import LIBRARY, SYNTH_CELLS
from gls.levelize import assemble
from oracle.runner import run_oracle, run_reference

GOLD = Path(__file__).resolve().parent / "golden"
U64 = 2**64 - 1


def golden_cases():
    return json.loads((GOLD / "cases.json").read_text())


def case_from_record(r):
    insts = [(c, ins, outs, [tuple(a) for a in arcs]) for c, ins, outs, arcs in r["instances"]]
    nl = assemble(insts, n_nets=r["n_nets"])
    st = stimulus({int(k): [tuple(e) for e in v] for k, v in r["stimulus"].items()})
    return nl, st


def compare(waves, saif, r, what):
    for net, ev in r["waves"].items():
        net = int(net)
        assert net in waves, f"{what}: net {net} missing"
        t, v = waves[net]
        exp = np.array(ev, np.int64).reshape(-1, 2)
        assert np.array_equal(np.asarray(t, np.int64), exp[:, 0]) and np.array_equal(np.asarray(v, np.int64), exp[:, 1]), \
            f"{what}: net {net} waveform differs"
    for net, rec in r["saif"].items():
        assert [int(x) for x in saif[int(net)]] == rec, f"{what}: SAIF of net {net} differs"


@pytest.mark.parametrize("idx", range(len(golden_cases())))
def test_oracle_matches_golden(idx, oracle_bin):
    r = golden_cases()[idx]
    nl, st = case_from_record(r)
    waves, saif, _ = run_oracle(nl, st, *r["window"], calc=r["calc"])
    compare(waves, saif, r, r["label"])


def test_cell_tables_match_reference_calc(libgls):
    tabs = json.loads((GOLD / "cell_tables.json").read_text())
    assert set(tabs) == set(SYNTH_CELLS)
    for name in SYNTH_CELLS:
        c = LIBRARY[name]
        cells, prims = assemble([(name, list(range(c.n_in)), [c.n_in], [])]).cell_arrays()
        for mode, key in ((CALC_FIXED, "fixed"), (CALC_LITERAL, "literal")):
            lut = cell_lut(cells[0], prims, 0, mode)
            assert lut.tolist() == tabs[name][key], f"{name} {key}"


def test_literal_calc_differs_where_reference_is_wrong():
    tabs = json.loads((GOLD / "cell_tables.json").read_text())
    # 1^x inversion under the 0/X=1/Z=2/1=3 encoding: NAND2(0,0) reads X
    assert tabs["GEN_NAND2_D1"]["literal"][0] == 1 and tabs["GEN_NAND2_D1"]["fixed"][0] == 3
    # AND2 / OR2 / XOR2 / BUF / MUX2 agree between the modes on inputs without Z
    for name in ("GEN_AND2_D1", "GEN_OR2_D1", "GEN_XOR2_D1", "GEN_BUF_D1", "GEN_MUX2_D1"):
        n_in = LIBRARY[name].n_in
        for idx, (a, b) in enumerate(zip(tabs[name]["literal"], tabs[name]["fixed"])):
            if all(((idx >> (2 * p)) & 3) != 2 for p in range(n_in)):
                assert a == b, (name, idx)


@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_reference_core(seed, oracle_bin, ref_bin):
    nl, st = random_case(5000 + seed, max_gates=10, max_events=40)
    calc = "literal" if seed % 2 else "fixed"
    w1, s1, _ = run_oracle(nl, st, 0, 450, calc=calc)
    w2, s2, _ = run_reference(nl, st, 0, 450, calc=calc)
    assert set(w1) == set(w2)
    for n in w1:
        assert np.array_equal(w1[n][0], w2[n][0]) and np.array_equal(w1[n][1], w2[n][1]), f"net {n}"
    assert np.array_equal(s1, s2)


def test_oracle_threads_agree(oracle_bin):
    nl, st = random_case(77, max_gates=40, max_in=6, horizon=3000, max_events=150)
    w1, s1, _ = run_oracle(nl, st, 0, 3000, threads=1)
    w4, s4, _ = run_oracle(nl, st, 0, 3000, threads=4)
    assert np.array_equal(s1, s4)
    for n in w1:
        assert np.array_equal(w1[n][0], w4[n][0])


def test_oracle_delay_factor(oracle_bin):
    # delays are scaled then truncated: 35 * 0.1 -> 3
    nl = assemble([("GEN_BUF_D1", [0], [1], [(2, "i", "z", 35.0, 47.0)])])
    st = stimulus({0: [(0, 0), (100, 3), (200, 0)]})
    w, _, _ = run_oracle(nl, st, 0, 300, factor=0.1)
    assert list(zip(w[1][0].tolist(), w[1][1].tolist())) == [(0, 1), (4, 0), (103, 3), (204, 0)]


@pytest.mark.parametrize("seed", range(8))
def test_oracle_cursor_values_equal_get_value_at(seed, oracle_bin):
    """The oracle takes each step's current and previous input values from
    its merge cursors; --verify-lookup also runs the binary search of
    GetValueAt (src/simulate.cpp:1459-1506) at every step and stops on any
    difference.  Random cases with X/Z, duplicate nets and repeated times
    across nets."""
    nl, st = random_case(6100 + seed, max_gates=30, max_in=6, horizon=2000, max_events=120, xz=True)
    w1, s1, _ = run_oracle(nl, st, 0, 2100, verify_lookup=True)
    assert w1


def test_oracle_keep_mode_matches_full_run(oracle_bin):
    """--keep drops every list after the last level that reads it: the kept
    nets' waveforms and every net's SAIF counts equal a full run's."""
    from gls import synth
    cfg = synth.scaled(synth.CONFIGS["c2"], cells=3_000, cycles=300, depth=12)
    nl = synth.make_netlist(cfg, seed=8)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=9)
    full_w, full_s, _ = run_oracle(nl, st, 0, cfg.t_end, threads=4)
    keep = np.arange(0, nl.n_nets, 97)
    lean_w, lean_s, _ = run_oracle(nl, st, 0, cfg.t_end, threads=4, keep=keep)
    assert set(lean_w) == {int(n) for n in keep if int(n) in full_w}
    for n in lean_w:
        assert np.array_equal(lean_w[n][0], full_w[n][0]) and np.array_equal(lean_w[n][1], full_w[n][1])
    assert np.array_equal(lean_s, full_s)
