"""Shared test workloads: small hand-made and random netlists + stimuli."""
from __future__ import annotations

import numpy as np

from gls.cells import LIBRARY, SYNTH_CELLS
from gls.levelize import assemble
from gls.netlist import Stimulus


def stimulus(d: dict[int, list[tuple[int, int]]]) -> Stimulus:
    nets = sorted(d)
    ev, T, V = [0], [], []
    for n in nets:
        for t, v in d[n]:
            T.append(t)
            V.append(v)
        ev.append(len(T))
    return Stimulus(np.array(nets, np.uint32), np.array(ev, np.uint64), np.array(T, np.uint32),
                    np.array(V, np.uint8))


def random_case(seed: int, max_gates: int = 12, max_in: int = 4, horizon: int = 400, max_events: int = 60,
                zero_delay: bool = False, xz: bool = True, dmax_choices=(3, 20, 80), cells=None):
    """Random small netlist (duplicate fan-in nets allowed, some arcs missing)
    with a dense random stimulus that includes X, Z and repeated values."""
    rng = np.random.default_rng(seed)
    names = cells or SYNTH_CELLS
    n_in_nets = int(rng.integers(1, max_in + 1))
    n_g = int(rng.integers(1, max_gates + 1))
    insts, nn = [], n_in_nets
    for _ in range(n_g):
        c = LIBRARY[names[int(rng.integers(len(names)))]]
        ins = [int(rng.integers(0, nn)) for _ in range(c.n_in)]
        dmax = int(rng.choice(dmax_choices))
        lo = 0 if zero_delay else 1
        arcs = [(e, i, o, float(rng.integers(lo, dmax)), float(rng.integers(lo, dmax))) for e, i, o in c.arcs]
        if rng.random() < 0.2 and arcs:
            arcs = arcs[:-1]
        insts.append((c.name, ins, [nn], arcs))
        nn += 1
    nl = assemble(insts, n_nets=nn)
    probs = [0.4, 0.1, 0.05, 0.45] if xz else [0.5, 0.0, 0.0, 0.5]
    d = {}
    for net in nl.ppi_nets:
        k = int(rng.integers(0, max_events))
        ts = np.unique(rng.integers(0, horizon, size=k))
        if rng.random() < 0.6:
            ts = np.unique(np.concatenate([[0], ts]))
        vs = rng.choice([0, 1, 2, 3], size=len(ts), p=probs)
        d[int(net)] = list(zip(ts.tolist(), vs.tolist()))
    return nl, stimulus(d)
