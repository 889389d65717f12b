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


def standard_vcd(seed: int, n_scalar: int = 12, n_bus: int = 5, n_times: int = 1500) -> str:
    """A VCD as simulators write it, in the subset the reference's reader
    (src/VCDParser.cpp) handles: distinct identifier codes, every change on
    its own line, full-width bus values, one change per signal and time,
    one value per signal at time 0 (in $dumpvars), and enough timestamps
    (> 2 x cores squared) for the reader's chunking of the body by "\\n#"."""
    rng = np.random.default_rng(seed)
    code = lambda k: "".join(chr(33 + d) for d in ([k % 94] if k < 94 else [k // 94 - 1, k % 94]))   # noqa: E731
    head = ["$date today $end", "$timescale 1ps $end", "$scope module top $end"]
    sigs = []
    for k in range(n_scalar):
        head.append(f"$var wire 1 {code(k)} s{k} $end")
        sigs.append((code(k), 0))
    for b in range(n_bus):
        w = int(rng.integers(2, 9))
        c = code(n_scalar + b)
        if b % 2:
            head.append(f"$var wire {w} {c} v{b} [0:{w - 1}] $end")
        else:
            head.append(f"$var wire {w} {c} v{b} [{w - 1}:0] $end")
        sigs.append((c, w))
    head += ["$upscope $end", "$enddefinitions $end"]
    body = ["#0", "$dumpvars"]
    alpha = "01xz"

    def val(w):
        return alpha[int(rng.choice(4, p=[0.45, 0.45, 0.06, 0.04]))] if w == 0 else \
            "".join(alpha[int(x)] for x in rng.choice(4, size=w, p=[0.45, 0.45, 0.06, 0.04]))

    for c, w in sigs:
        body.append(val(w) + c if w == 0 else f"b{val(w)} {c}")
    body.append("$end")
    t = 0
    for _ in range(n_times):
        t += int(rng.integers(1, 40))
        body.append(f"#{t}")
        for j in rng.permutation(len(sigs))[: int(rng.integers(1, len(sigs) + 1))]:
            c, w = sigs[int(j)]
            body.append(val(w) + c if w == 0 else f"b{val(w)} {c}")
    return "\n".join(head + body) + "\n"
