"""Structure-of-arrays netlist and stimulus containers.

`Netlist` carries what `process` packs into inter.dat for the simulate stage
(src/process.cpp:58-79): the cells' function programs, the instances in
level order with their input and output nets, the SDF IOPATH arcs of every
instance, and the level boundaries.  `Stimulus` carries the change lists of
the nets the VCD drives (src/VCDParser.h:46-57).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .cells import CellDef

ARC_DTYPE = np.dtype([("edge", "u1"), ("in_pin", "u1"), ("out_pin", "u1"), ("reserved", "u1", (5,)),
                      ("rise", "<f8"), ("fall", "<f8")])
CELL_DTYPE = np.dtype([("n_in", "u1"), ("n_out", "u1"), ("n_prim", "u1"), ("reserved", "u1"),
                       ("prim_start", "<u4")])
PRIM_DTYPE = np.dtype([("func", "u1"), ("n_pins", "u1"), ("pins", "u1", (14,))])

V0, VX, VZ, V1 = 0, 1, 2, 3


@dataclass
class Netlist:
    n_nets: int
    cells: list[CellDef]
    inst_cell: np.ndarray          # uint32 [n_inst], level order
    level_start: np.ndarray        # uint32 [n_levels + 1]
    pin_start: np.ndarray          # uint32 [n_inst + 1]
    pin_net: np.ndarray            # uint32: per instance n_in inputs then n_out outputs
    arc_start: np.ndarray          # uint32 [n_inst + 1]
    arcs: np.ndarray               # ARC_DTYPE
    ppi_nets: np.ndarray           # uint32: nets the stimulus must drive
    net_names: list[str] | None = None
    inst_names: list[str] | None = None
    extra: dict = field(default_factory=dict)

    @property
    def n_inst(self) -> int:
        return int(self.inst_cell.shape[0])

    @property
    def n_levels(self) -> int:
        return int(self.level_start.shape[0] - 1)

    def net_name(self, n: int) -> str:
        return self.net_names[n] if self.net_names is not None else f"n{n}"

    def inst_name(self, i: int) -> str:
        return self.inst_names[i] if self.inst_names is not None else f"U{i}"

    def cell_arrays(self):
        """(cells, prims) packed as CELL_DTYPE / PRIM_DTYPE arrays."""
        cells = np.zeros(len(self.cells), CELL_DTYPE)
        plist = []
        for k, c in enumerate(self.cells):
            prog = c.program()
            cells[k] = (c.n_in, c.n_out, len(prog), 0, len(plist))
            for fn, pins in prog:
                if len(pins) > 14:
                    raise ValueError(f"{c.name}: primitive with {len(pins)} pins")
                row = np.zeros((), PRIM_DTYPE)
                row["func"] = fn
                row["n_pins"] = len(pins)
                row["pins"][: len(pins)] = pins
                plist.append(row)
        prims = np.array(plist, PRIM_DTYPE) if plist else np.zeros(1, PRIM_DTYPE)
        return cells, prims

    def inputs_of(self, i: int) -> np.ndarray:
        c = self.cells[int(self.inst_cell[i])]
        p = int(self.pin_start[i])
        return self.pin_net[p: p + c.n_in]

    def outputs_of(self, i: int) -> np.ndarray:
        c = self.cells[int(self.inst_cell[i])]
        p = int(self.pin_start[i]) + c.n_in
        return self.pin_net[p: p + c.n_out]

    def gate_output_nets(self) -> np.ndarray:
        """Output nets of every instance, in instance order."""
        n_in = np.array([c.n_in for c in self.cells], np.int64)[self.inst_cell]
        n_out = np.array([c.n_out for c in self.cells], np.int64)[self.inst_cell]
        idx = np.concatenate([np.arange(s + a, s + a + b) for s, a, b in
                              zip(self.pin_start[:-1].astype(np.int64), n_in, n_out)]) if self.n_inst else np.zeros(0, np.int64)
        return self.pin_net[idx]


@dataclass
class Stimulus:
    nets: np.ndarray        # uint32 [k]
    ev_start: np.ndarray    # uint64 [k + 1]
    time: np.ndarray        # uint32
    value: np.ndarray       # uint8, 0 / 1=X / 2=Z / 3

    @property
    def n_events(self) -> int:
        return int(self.ev_start[-1])

    def events_of(self, k: int):
        a, b = int(self.ev_start[k]), int(self.ev_start[k + 1])
        return self.time[a:b], self.value[a:b]
