"""TEST INFRASTRUCTURE ONLY: a fixed-seed sample of a design's gates run
through the reference's own serial core, one gate at a time.

Every sampled gate becomes an independent single gate whose input nets are
stimulus nets carrying the waveforms the caller supplies (the GPU's own, for
an inductive check of those gates, or the C oracle's exact ones).  The
reference core (oracle/_ref/ref_sim: src/simulate.cpp:872-1506 with the level
loop of :1569-1668) then computes their outputs, which are compared with the
design run's outputs bit for bit, and timed for the CPU baseline.  Only tests/
and bench.py's reference legs use this module.
"""
from __future__ import annotations

import numpy as np

SAMPLE_SEED, SAMPLE_MAX = 7, 4000


def sample_order(nl, seed: int = SAMPLE_SEED, k_max: int = SAMPLE_MAX) -> np.ndarray:
    """A fixed-seed permutation of the gates cut to k_max; a sample of k gates
    is its first k, so every smaller sample is part of a larger one."""
    rng = np.random.default_rng(seed)
    return rng.permutation(nl.n_inst)[: min(k_max, nl.n_inst)]


def sample_input_nets(nl, gates) -> np.ndarray:
    """The input nets of the given gates (the lists a sample needs)."""
    if not len(gates):
        return np.zeros(0, np.uint32)
    return np.unique(np.concatenate([nl.inputs_of(int(i)) for i in gates]))


def sample_case(nl, waves_of, gates):
    """The gates rewired as independent single gates fed by stimulus nets with
    the waveforms waves_of(net) -> (times, values).
    -> (netlist, stimulus, gate_events, [(gate, sample output net, design output net)])."""
    from gls.levelize import assemble
    from gls.netlist import Stimulus
    insts, stim, nxt, gev = [], {}, 0, 0
    for i in gates:
        c = nl.cells[int(nl.inst_cell[i])]
        local = {}
        ins = []
        for n in nl.inputs_of(int(i)).tolist():
            if n not in local:
                local[n] = nxt
                stim[nxt] = waves_of(n)
                nxt += 1
            ins.append(local[n])
            gev += len(stim[local[n]][0])
        arcs = [(int(a["edge"]), int(a["in_pin"]), int(a["out_pin"]), float(a["rise"]), float(a["fall"]))
                for a in nl.arcs[int(nl.arc_start[i]): int(nl.arc_start[i + 1])]]
        insts.append([c.name, ins, [-1] * c.n_out, arcs, int(i)])
    outs = []
    for inst in insts:
        design_outs = nl.outputs_of(inst[4]).tolist()
        inst[2][:] = list(range(nxt, nxt + len(inst[2])))
        outs += [(inst[4], nxt + k, int(design_outs[k])) for k in range(len(inst[2]))]
        nxt += len(inst[2])
    sn = sorted(stim)
    ev = np.zeros(len(sn) + 1, np.uint64)
    ev[1:] = np.cumsum([len(stim[n][0]) for n in sn])
    T = np.concatenate([np.asarray(stim[n][0], np.uint32) for n in sn]) if sn else np.zeros(0, np.uint32)
    V = np.concatenate([np.asarray(stim[n][1], np.uint8) for n in sn]) if sn else np.zeros(0, np.uint8)
    snl = assemble([tuple(x[:4]) for x in insts], n_nets=nxt)
    return snl, Stimulus(np.array(sn, np.uint32), ev, T, V), gev, outs


def run_sample(nl, waves_of, gates, t_begin, t_end, threads):
    """The reference core (the C oracle where the reference sources are
    absent) on the given gates.  -> dict(rate, sec, gates, gev, kind, snl,
    sst, outs, waves, saif, run)."""
    from . import build
    from .runner import run_oracle, run_reference
    have_ref = build.build_reference() is not None
    run = run_reference if have_ref else run_oracle
    # the heaviest gates first (fan-in events of their distinct input nets):
    # the threads take gates in this order, so the last ones to start are
    # short and the threads finish together
    gates = np.sort(np.asarray(gates))
    work = np.array([sum(len(waves_of(int(n))[0]) for n in np.unique(nl.inputs_of(int(i)))) for i in gates],
                    np.int64)
    gates = gates[np.argsort(-work, kind="stable")]
    snl, sst, gev, outs = sample_case(nl, waves_of, gates)
    waves, saif, sec = run(snl, sst, t_begin, t_end, threads=threads)
    return dict(rate=gev / sec, sec=sec, gates=len(gates), gev=gev, kind="reference" if have_ref else "port",
                snl=snl, sst=sst, outs=outs, waves=waves, saif=saif, run=run)


def sized_sample(nl, waves_of, t_end, threads, order, budget_s):
    """run_sample on the first k gates of `order`, k grown until one run takes
    about budget_s / 3 or more (or the order is used up)."""
    k = min(24, len(order))
    while True:
        r = run_sample(nl, waves_of, order[:k], 0, t_end, threads)
        if r["sec"] >= budget_s / 3 or k >= len(order):
            return r
        k = min(len(order), int(k * max(2.0, budget_s / max(r["sec"], 1e-3) * 0.8)))


def compare_outputs(waveform_of, saif_table, r) -> dict:
    """The design run's outputs of the sampled gates (waveform_of(net) ->
    (times, values); saif_table (n_nets, 3)) against the sample's, bit for bit."""
    bad = []
    for gate, local, net in r["outs"]:
        gt, gv = waveform_of(net)
        rt, rv = r["waves"].get(local, (None, None))
        same = (rt is not None and np.array_equal(np.asarray(gt, np.int64), np.asarray(rt, np.int64))
                and np.array_equal(np.asarray(gv, np.int64), np.asarray(rv, np.int64))
                and np.array_equal(np.asarray(saif_table[net], np.uint64), np.asarray(r["saif"][local], np.uint64)))
        if not same:
            bad.append(int(gate))
    return {"gates_checked": r["gates"], "outputs_checked": len(r["outs"]), "mismatches": len(bad),
            "mismatched_gates": bad[:16], "checker": r["kind"]}
