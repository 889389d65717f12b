"""Levelization and netlist assembly from an instance list.

`levelize` restates the reference's Kahn levelization (GenerateAdjacencyList,
SetInDegrees, TopologyOrder; src/process.cpp:90-176): an edge runs from
instance i to every instance that reads one of i's output nets, level 0 is
every instance with no such predecessor, and each later level takes, in
instance order, the instances whose predecessors are all placed.  A netlist
with a combinational loop is rejected (the reference degrades it to one
instance per level, src/process.cpp:143-155).
"""
from __future__ import annotations

import numpy as np

from .cells import CellDef, LIBRARY
from .netlist import ARC_DTYPE, Netlist


def levelize(in_nets: list[list[int]], out_nets: list[list[int]]) -> list[list[int]]:
    n = len(in_nets)
    readers: dict[int, list[int]] = {}
    for i, ins in enumerate(in_nets):
        for net in ins:
            readers.setdefault(net, []).append(i)
    succ = []
    for i in range(n):
        s = set()
        for net in out_nets[i]:
            s.update(readers.get(net, ()))
        succ.append(sorted(s))
    indeg = np.zeros(n, np.int64)
    for s in succ:
        for j in s:
            indeg[j] += 1
    levels, placed = [], 0
    while placed < n:
        q = [i for i in range(n) if indeg[i] == 0]
        if not q:
            raise ValueError("combinational loop: netlist cannot be levelized")
        for i in q:
            indeg[i] = -1
        for i in q:
            for j in succ[i]:
                indeg[j] -= 1
        levels.append(q)
        placed += len(q)
    return levels


def assemble(instances, n_nets: int | None = None, cells: dict[str, CellDef] | None = None,
             net_names: list[str] | None = None, inst_names: list[str] | None = None) -> Netlist:
    """Build a levelized Netlist.

    instances: list of (cell name, [input nets], [output nets],
               [(edge, in_port, out_port, rise, fall), ...]) with ports given
               by name or by index.
    Nets that no instance drives are the stimulus nets (`ppi_nets`).
    """
    lib = cells or LIBRARY
    names = sorted({inst[0] for inst in instances})
    cdefs = [lib[nm] for nm in names]
    cidx = {nm: k for k, nm in enumerate(names)}
    ins = [list(map(int, x[1])) for x in instances]
    outs = [list(map(int, x[2])) for x in instances]
    for k, x in enumerate(instances):
        c = lib[x[0]]
        if len(ins[k]) != c.n_in or len(outs[k]) != c.n_out:
            raise ValueError(f"instance {k}: {x[0]} needs {c.n_in} inputs / {c.n_out} outputs")
    levels = levelize(ins, outs)
    order = [i for lv in levels for i in lv]
    level_start = np.zeros(len(levels) + 1, np.uint32)
    np.cumsum([len(lv) for lv in levels], out=level_start[1:])
    all_nets = [v for a in ins + outs for v in a]
    nn = n_nets if n_nets is not None else (max(all_nets) + 1 if all_nets else 0)
    pin_start, pin_net, arc_start, arcs = [0], [], [0], []
    for i in order:
        c = lib[instances[i][0]]
        pin_net += ins[i] + outs[i]
        pin_start.append(len(pin_net))
        for edge, ip, op, rise, fall in instances[i][3]:
            ipi = c.inputs.index(ip) if isinstance(ip, str) else int(ip)
            opi = c.outputs.index(op) if isinstance(op, str) else int(op)
            arcs.append((edge, ipi, opi, (0,) * 5, float(rise), float(fall)))
        arc_start.append(len(arcs))
    driven = {v for o in outs for v in o}
    read = {v for a in ins for v in a}
    ppi = sorted(read - driven)
    return Netlist(
        n_nets=nn, cells=cdefs,
        inst_cell=np.array([cidx[instances[i][0]] for i in order], np.uint32),
        level_start=level_start, pin_start=np.array(pin_start, np.uint32),
        pin_net=np.array(pin_net, np.uint32), arc_start=np.array(arc_start, np.uint32),
        arcs=np.array(arcs, ARC_DTYPE) if arcs else np.zeros(0, ARC_DTYPE),
        ppi_nets=np.array(ppi, np.uint32), net_names=net_names,
        inst_names=[inst_names[i] for i in order] if inst_names else None,
        extra={"order": order},
    )


def default_arcs(cell: CellDef, rise: float, fall: float):
    """The cell's specify arcs, all with the same rise / fall delay."""
    return [(e, i, o, rise, fall) for e, i, o in cell.arcs]
