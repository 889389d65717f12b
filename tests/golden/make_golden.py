"""Generate the golden vectors in this directory from the reference's own
serial simulator core (oracle/_ref/ref_sim, built from the reference sources
by oracle/build.py).  Run from the repository root:

    python tests/golden/make_golden.py

Writes:
  cell_tables.json   output of every synthetic cell for every 4-state input
                     combination, in both calc modes (via RunFunction + calc)
  cases.json         small netlists with stimulus, window, and the
                     reference's output waveforms and SAIF records
"""
from __future__ import annotations

import itertools
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path[:0] = [str(REPO), str(REPO / "gate-level-simulator_gb300"), str(REPO / "tests")]

import numpy as np  # noqa: E402

from cases import random_case, stimulus  # noqa: E402
from gls.cells import LIBRARY, SYNTH_CELLS  # noqa: E402
from gls.levelize import assemble, default_arcs  # noqa: E402
from oracle.runner import run_reference  # noqa: E402

STEP = 1000


def table_stimulus(n_in: int):
    """Pin waveforms walking through all 4^n_in input combinations, one per
    STEP, recording only changes."""
    combos = list(itertools.product(range(4), repeat=n_in))
    d = {p: [] for p in range(n_in)}
    for i, combo in enumerate(combos):
        for p, v in enumerate(combo):
            if not d[p] or d[p][-1][1] != v:
                d[p].append((i * STEP, v))
    return combos, d


def value_at(wave, t):
    ts, vs = wave
    k = np.searchsorted(ts, t, side="right") - 1
    return int(vs[k]) if k >= 0 else 1


def cell_tables():
    out = {}
    for name in SYNTH_CELLS:
        c = LIBRARY[name]
        combos, d = table_stimulus(c.n_in)
        nl = assemble([(name, list(range(c.n_in)), [c.n_in], default_arcs(c, 1.0, 1.0))], n_nets=c.n_in + 1)
        st = stimulus(d)
        entry = {}
        for calc in ("fixed", "literal"):
            waves, _, _ = run_reference(nl, st, 0, len(combos) * STEP, calc=calc)
            tab = [0] * (4 ** c.n_in)
            for i, combo in enumerate(combos):
                idx = sum(v << (2 * p) for p, v in enumerate(combo))
                tab[idx] = value_at(waves[c.n_in], i * STEP + STEP // 2)
            entry[calc] = tab
        out[name] = entry
    return out


def case_record(nl, st, t_begin, t_end, calc, label):
    waves, saif, _ = run_reference(nl, st, t_begin, t_end, calc=calc)
    insts = []
    for i in range(nl.n_inst):
        c = nl.cells[int(nl.inst_cell[i])]
        arcs = [[int(a["edge"]), int(a["in_pin"]), int(a["out_pin"]), float(a["rise"]), float(a["fall"])]
                for a in nl.arcs[int(nl.arc_start[i]): int(nl.arc_start[i + 1])]]
        insts.append([c.name, nl.inputs_of(i).tolist(), nl.outputs_of(i).tolist(), arcs])
    stim = {int(st.nets[k]): [[int(t), int(v)] for t, v in zip(*st.events_of(k))] for k in range(len(st.nets))}
    return {
        "label": label, "calc": calc, "n_nets": int(nl.n_nets), "instances": insts, "stimulus": stim,
        "window": [int(t_begin), int(t_end)],
        "waves": {int(n): [[int(t), int(v)] for t, v in zip(*w)] for n, w in waves.items()},
        "saif": {int(n): [int(x) for x in saif[n]] for n in range(nl.n_nets) if saif[n][0] != 2**64 - 1},
    }


def cases():
    recs = []
    # the AND2 / XOR2 / NAND2 pulse cases: a 10 ps low pulse on a2 is swallowed
    pulse = {0: [(0, 0), (1000, 3), (3000, 0)], 1: [(0, 3), (2000, 0), (2010, 3)]}
    for cell, arcs in [("GEN_AND2_D1", [(2, "a1", "z", 30, 40), (2, "a2", "z", 50, 60)]),
                       ("GEN_XOR2_D1", [(0, "a1", "z", 30, 40), (1, "a1", "z", 35, 45),
                                        (0, "a2", "z", 50, 60), (1, "a2", "z", 55, 65)]),
                       ("GEN_NAND2_D1", [(2, "a1", "zn", 30, 40), (2, "a2", "zn", 50, 60)])]:
        nl = assemble([(cell, [0, 1], [2], arcs)])
        for calc in ("fixed", "literal"):
            recs.append(case_record(nl, stimulus(pulse), 0, 5000, calc, f"pulse-{cell}"))
    # a 200 ps pulse passes, a 10 ps pulse does not
    nl = assemble([("GEN_AND2_D1", [0, 1], [2], [(2, "a1", "z", 30, 40), (2, "a2", "z", 50, 60)])])
    st = stimulus({0: [(0, 3)], 1: [(0, 3), (2000, 0), (2010, 3), (2200, 0), (2400, 3)]})
    recs.append(case_record(nl, st, 0, 5000, "fixed", "pulse-widths"))
    # random netlists, windows inside and around the activity
    for seed in range(24):
        nl, st = random_case(1000 + seed)
        tb, te = [(0, 500), (50, 300), (120, 121), (0, 2000)][seed % 4]
        recs.append(case_record(nl, st, tb, te, "fixed" if seed % 3 else "literal", f"random-{seed}"))
    for seed in range(6):
        nl, st = random_case(2000 + seed, max_gates=30, max_in=6, horizon=3000, max_events=200, xz=False)
        recs.append(case_record(nl, st, 0, 3000, "fixed", f"random-large-{seed}"))
    return recs


if __name__ == "__main__":
    (HERE / "cell_tables.json").write_text(json.dumps(cell_tables()))
    (HERE / "cases.json").write_text(json.dumps(cases()))
    print("wrote", HERE / "cell_tables.json", HERE / "cases.json")
