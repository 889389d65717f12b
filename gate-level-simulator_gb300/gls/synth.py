"""Seeded synthetic netlists and stimuli of the benchmark shapes.

The reference's example design is not distributed, so workloads are
generated: a levelized combinational netlist of GEN_*_D1 cells with exact
logic depth (every gate of level L reads at least one output of level L-1,
so Kahn levelization, src/process.cpp:128-176, gives back the same levels),
SDF IOPATH delays drawn per arc, and a clocked stimulus on the pseudo-primary
inputs (primary inputs plus register Q pins, which `process` leaves undriven
because it skips the sequential cells, src/PreProcess.cpp:632-636).

Fan-out: every net gets an exponential attractiveness and pins pick their
source in proportion to it inside their eligible window, which makes the
fan-out of a net a mixed Poisson with exponential mean, i.e. geometric; a
hard cap is then enforced by re-drawing the excess pins.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .cells import LIBRARY, SYNTH_CELLS, SYNTH_WEIGHTS
from .netlist import ARC_DTYPE, Netlist, Stimulus, V0, V1, VX


@dataclass
class SynthConfig:
    name: str
    n_cells: int
    depth: int
    n_pi: int
    n_reg: int
    fanout_max: int
    cycles: int
    toggle: tuple          # ("const", p) | ("beta", a, b) | ("loguniform", lo, hi)
    period: int = 1000
    x_init: float = 0.01
    delay_lo: int = 5
    delay_hi: int = 80

    @property
    def n_ppi(self) -> int:
        return self.n_pi + self.n_reg

    @property
    def t_end(self) -> int:
        return self.cycles * self.period


CONFIGS = {
    # 2,000 cells, depth 20, 64 PIs + 128 register Q pins, 1,000 cycles, p = 0.2
    "c1": SynthConfig("c1", 2_000, 20, 64, 128, 32, 1_000, ("const", 0.2)),
    # 200,000 cells, depth 60, 4,096 pseudo-primary inputs, 10,000 cycles, p ~ Beta(2, 8)
    "c2": SynthConfig("c2", 200_000, 60, 1_024, 3_072, 256, 10_000, ("beta", 2.0, 8.0)),
    # 2,000,000 cells, depth 120, 65,536 pseudo-primary inputs, 20,000 cycles, p log-uniform
    "c3": SynthConfig("c3", 2_000_000, 120, 16_384, 49_152, 256, 20_000, ("loguniform", 0.01, 0.5)),
}


def scaled(cfg: SynthConfig, cells: int | None = None, cycles: int | None = None,
           depth: int | None = None, ppi: int | None = None) -> SynthConfig:
    """A smaller instance of a configuration (for tests that must finish fast)."""
    d = dict(cfg.__dict__)
    if cells is not None:
        d["n_cells"] = cells
    if cycles is not None:
        d["cycles"] = cycles
    if depth is not None:
        d["depth"] = depth
    if ppi is not None:
        d["n_pi"] = max(1, ppi // 3)
        d["n_reg"] = ppi - d["n_pi"]
    d["name"] = cfg.name + "-scaled"
    return SynthConfig(**d)


def make_netlist(cfg: SynthConfig, seed: int) -> Netlist:
    rng = np.random.default_rng(seed)
    cells = [LIBRARY[n] for n in SYNTH_CELLS]
    w = np.array(SYNTH_WEIGHTS, np.float64)
    n, P, D = cfg.n_cells, cfg.n_ppi, cfg.depth
    ctype = rng.choice(len(cells), size=n, p=w / w.sum()).astype(np.uint32)
    n_in = np.array([c.n_in for c in cells], np.int64)[ctype]
    n_out = np.array([c.n_out for c in cells], np.int64)[ctype]
    # level sizes: as even as possible
    lv_sizes = np.full(D, n // D, np.int64)
    lv_sizes[: n % D] += 1
    level_start = np.zeros(D + 1, np.int64)
    np.cumsum(lv_sizes, out=level_start[1:])
    # nets: PPIs first, then gate outputs in level order (single-output cells)
    assert (n_out == 1).all()
    n_nets = P + n
    attract = rng.exponential(1.0, size=n_nets)
    cum = np.concatenate([[0.0], np.cumsum(attract)])
    pin_start = np.zeros(n + 1, np.int64)
    np.cumsum(n_in + n_out, out=pin_start[1:])
    pin_net = np.zeros(int(pin_start[-1]), np.int64)

    def pick(lo, hi, k):
        """k nets from [lo, hi) in proportion to their attractiveness."""
        u = rng.random(k) * (cum[hi] - cum[lo]) + cum[lo]
        return np.clip(np.searchsorted(cum, u, side="right") - 1, lo, hi - 1)

    for L in range(D):
        g0, g1 = int(level_start[L]), int(level_start[L + 1])
        if g1 == g0:
            continue
        prev_lo = P + int(level_start[L - 1]) if L > 0 else 0
        prev_hi = P + g0 if L > 0 else P
        near_lo = P + int(level_start[max(0, L - 4)]) if L >= 4 else 0
        gates = np.arange(g0, g1)
        ni = n_in[gates]
        base = pin_start[gates]
        # first input from the previous level keeps the depth exact
        pin_net[base] = pick(prev_lo, prev_hi, len(gates))
        for k in range(1, 3):
            sel = gates[ni > k]
            if not len(sel):
                continue
            near = rng.random(len(sel)) < 0.7
            src = np.where(near, pick(near_lo, P + g0, len(sel)), pick(0, P + g0, len(sel)))
            pin_net[pin_start[sel] + k] = src
        # distinct nets per gate: re-draw duplicates a few times
        for _ in range(4):
            dup = np.zeros(len(gates), bool)
            for k in range(1, 3):
                m = ni > k
                for j in range(k):
                    dup[m] |= pin_net[base[m] + k] == pin_net[base[m] + j]
            if not dup.any():
                break
            sel = gates[dup]
            for k in range(1, 3):
                s2 = sel[n_in[sel] > k]
                pin_net[pin_start[s2] + k] = pick(0, P + g0, len(s2))
        pin_net[base + ni] = P + gates
    # enforce the fan-out cap
    inp_mask = np.ones(len(pin_net), bool)
    inp_mask[pin_start[1:] - 1] = False   # output pin of each single-output cell
    for _ in range(20):
        fo = np.bincount(pin_net[inp_mask], minlength=n_nets)
        over = np.nonzero(fo > cfg.fanout_max)[0]
        if not len(over):
            break
        pins = np.nonzero(inp_mask)[0]
        for net in over:
            users = pins[pin_net[pins] == net]
            excess = users[rng.permutation(len(users))[: len(users) - cfg.fanout_max]]
            gate_of = np.searchsorted(pin_start, excess, side="right") - 1
            lv = np.searchsorted(level_start, gate_of, side="right") - 1
            first = excess == pin_start[gate_of]
            for p, g, L, f in zip(excess, gate_of, lv, first):
                if f and L > 0:
                    pin_net[p] = pick(P + int(level_start[L - 1]), P + int(level_start[L]), 1)[0]
                elif f:
                    pin_net[p] = pick(0, P, 1)[0]
                else:
                    pin_net[p] = pick(0, P + int(level_start[L]), 1)[0]
    # arcs with integer delays
    arc_counts = np.array([len(c.arcs) for c in cells], np.int64)[ctype]
    arc_start = np.zeros(n + 1, np.int64)
    np.cumsum(arc_counts, out=arc_start[1:])
    arcs = np.zeros(int(arc_start[-1]), ARC_DTYPE)
    for t, c in enumerate(cells):
        sel = np.nonzero(ctype == t)[0]
        for a, (edge, ip, op) in enumerate(c.arcs):
            idx = arc_start[sel] + a
            arcs["edge"][idx] = edge
            arcs["in_pin"][idx] = c.inputs.index(ip)
            arcs["out_pin"][idx] = c.outputs.index(op)
    arcs["rise"] = rng.integers(cfg.delay_lo, cfg.delay_hi + 1, size=len(arcs)).astype(np.float64)
    arcs["fall"] = rng.integers(cfg.delay_lo, cfg.delay_hi + 1, size=len(arcs)).astype(np.float64)
    return Netlist(
        n_nets=n_nets, cells=cells, inst_cell=ctype,
        level_start=level_start.astype(np.uint32), pin_start=pin_start.astype(np.uint32),
        pin_net=pin_net.astype(np.uint32), arc_start=arc_start.astype(np.uint32), arcs=arcs,
        ppi_nets=np.arange(P, dtype=np.uint32),
        extra={"config": cfg.name, "seed": seed, "n_pi": cfg.n_pi, "n_reg": cfg.n_reg},
    )


def toggle_rates(cfg: SynthConfig, k: int, rng) -> np.ndarray:
    kind = cfg.toggle[0]
    if kind == "const":
        return np.full(k, float(cfg.toggle[1]))
    if kind == "beta":
        return rng.beta(cfg.toggle[1], cfg.toggle[2], size=k)
    if kind == "loguniform":
        lo, hi = np.log(cfg.toggle[1]), np.log(cfg.toggle[2])
        return np.exp(rng.uniform(lo, hi, size=k))
    raise ValueError(kind)


def make_stimulus(cfg: SynthConfig, nets: np.ndarray, seed: int, cycles: int | None = None) -> Stimulus:
    """Clocked stimulus: each net toggles at a clock edge with its own rate;
    the initial value is 0 or 1 with probability (1 - x_init) / 2 each, else X."""
    rng = np.random.default_rng(seed)
    C = cfg.cycles if cycles is None else cycles
    k = len(nets)
    p = np.clip(toggle_rates(cfg, k, rng), 1e-6, 1.0)
    init = np.where(rng.random(k) < cfg.x_init, VX, np.where(rng.random(k) < 0.5, V0, V1)).astype(np.uint8)
    times, values, starts = [], [], [0]
    for i in range(k):
        expect = p[i] * (C - 1)
        m = int(expect + 6.0 * np.sqrt(expect + 1.0) + 16)
        while True:
            edges = np.cumsum(rng.geometric(p[i], size=m))
            if edges[-1] >= C or m > 4 * C:
                break
            m *= 2
        edges = edges[edges < C]
        t = np.empty(len(edges) + 1, np.uint32)
        t[0] = 0
        t[1:] = edges * cfg.period
        v = np.empty(len(edges) + 1, np.uint8)
        v[0] = init[i]
        if len(edges):
            first = init[i] if init[i] != VX else (V0 if rng.random() < 0.5 else V1)
            # after the first toggle the value alternates
            alt = np.arange(len(edges)) % 2 == 0
            if init[i] == VX:
                v[1:] = np.where(alt, first, V0 + V1 - first)
            else:
                v[1:] = np.where(alt, V0 + V1 - first, first)
        times.append(t)
        values.append(v)
        starts.append(starts[-1] + len(t))
    return Stimulus(nets=np.asarray(nets, np.uint32), ev_start=np.array(starts, np.uint64),
                    time=np.concatenate(times) if times else np.zeros(0, np.uint32),
                    value=np.concatenate(values) if values else np.zeros(0, np.uint8))
