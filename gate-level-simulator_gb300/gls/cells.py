"""Cell library used by the synthetic netlists.

The cells are the GEN_*_D1 modules of the reference's generic standard-cell
library (examples/GENERIC_STD_CELL.vlib), restated here as primitive programs
in the reference's function-program encoding (Instance::function_id_vec,
src/PreProcess.cpp:1194-1263): the primitive ids of that file (and 0 ...
udp_mux2 9), supply0 = pin 16, supply1 = pin 17, cell input k is pin k,
cell output k is pin n_in + k, internal wires follow.  Port names and declaration order match the
library so that netlists written by `gls.files` read back through the
reference's `process` front end.

Each cell also lists its `specify` arcs (edge, input port, output port) with
edge 0 = posedge, 1 = negedge, 2 = both (Delay::edge, src/VCDTypes.h:166-186).
"""
from __future__ import annotations

from dataclasses import dataclass, field

F_AND, F_OR, F_XOR, F_XNOR, F_NOR, F_NAND, F_BUF, F_NOT, F_UDP_XBUF, F_UDP_MUX2 = range(10)
FUNC_NAMES = ["and", "or", "xor", "xnor", "nor", "nand", "buf", "not", "udp_xbuf", "udp_mux2"]
PIN_SUPPLY0 = 16
PIN_SUPPLY1 = 17


@dataclass
class CellDef:
    name: str
    inputs: list[str]
    outputs: list[str]
    # primitives in source order: (function name, output port/wire, [input ports/wires])
    prims: list[tuple[str, str, list[str]]]
    arcs: list[tuple[int, str, str]] = field(default_factory=list)
    wires: list[str] = field(default_factory=list)
    ignored: bool = False   # sequential cells the `process` front end skips

    @property
    def n_in(self) -> int:
        return len(self.inputs)

    @property
    def n_out(self) -> int:
        return len(self.outputs)

    def pin_code(self, name: str) -> int:
        if name in self.inputs:
            return self.inputs.index(name)
        if name in self.outputs:
            return self.n_in + self.outputs.index(name)
        if name in self.wires:
            return self.n_in + self.n_out + self.wires.index(name)
        raise KeyError(name)

    def program(self) -> list[tuple[int, list[int]]]:
        """[(func id, [input pin codes..., driven pin code])] in source order."""
        out = []
        for fn, o, ins in self.prims:
            out.append((FUNC_NAMES.index(fn), [self.pin_code(x) for x in ins] + [self.pin_code(o)]))
        return out


def _both(cell_inputs, out):
    return [(2, i, out) for i in cell_inputs]


def _edges(cell_inputs, out):
    arcs = []
    for i in cell_inputs:
        arcs += [(0, i, out), (1, i, out)]
    return arcs


def _gate(name, fn, ins, out, edge_arcs=False):
    return CellDef(name, list(ins), [out], [(fn, out, list(ins))],
                   _edges(ins, out) if edge_arcs else _both(ins, out))


LIBRARY: dict[str, CellDef] = {}


def _add(c: CellDef):
    LIBRARY[c.name] = c


_add(_gate("GEN_INV_D1", "not", ["i"], "zn"))
_add(_gate("GEN_BUF_D1", "buf", ["i"], "z"))
_add(_gate("GEN_NAND2_D1", "nand", ["a1", "a2"], "zn"))
_add(_gate("GEN_NAND3_D1", "nand", ["a1", "a2", "a3"], "zn"))
_add(_gate("GEN_NOR2_D1", "nor", ["a1", "a2"], "zn"))
_add(_gate("GEN_NOR3_D1", "nor", ["a1", "a2", "a3"], "zn"))
_add(_gate("GEN_AND2_D1", "and", ["a1", "a2"], "z"))
_add(_gate("GEN_OR2_D1", "or", ["a1", "a2"], "z"))
_add(_gate("GEN_XOR2_D1", "xor", ["a1", "a2"], "z", edge_arcs=True))
_add(_gate("GEN_XNOR2_D1", "xnor", ["a1", "a2"], "zn", edge_arcs=True))
_add(CellDef("GEN_MUX2_D1", ["i0", "i1", "s"], ["z"], [("udp_mux2", "z", ["i0", "i1", "s"])],
             [(2, "i0", "z"), (2, "i1", "z"), (0, "s", "z"), (1, "s", "z")]))
_add(CellDef("GEN_AOI21_D1", ["a1", "a2", "b"], ["zn"],
             [("and", "net0", ["a1", "a2"]), ("or", "net1", ["net0", "b"]), ("not", "zn", ["net1"])],
             _both(["a1", "a2", "b"], "zn"), wires=["net0", "net1"]))
_add(CellDef("GEN_OAI21_D1", ["a1", "a2", "b"], ["zn"],
             [("or", "net0", ["a1", "a2"]), ("and", "net1", ["net0", "b"]), ("not", "zn", ["net1"])],
             _both(["a1", "a2", "b"], "zn"), wires=["net0", "net1"]))
# register: an ignored module, its Q net becomes a pseudo-primary input
_add(CellDef("GEN_DF_D1", ["d", "cp"], ["q"], [], [], ignored=True))

# The 13 combinational cells of the synthetic configurations and their draw
# weights.  The configuration text lists 12 weights for 13 cells; they are
# given in order to the first 12 and OAI21 gets 6.
SYNTH_CELLS = ["GEN_INV_D1", "GEN_BUF_D1", "GEN_NAND2_D1", "GEN_NAND3_D1", "GEN_NOR2_D1",
               "GEN_NOR3_D1", "GEN_AND2_D1", "GEN_OR2_D1", "GEN_XOR2_D1", "GEN_XNOR2_D1",
               "GEN_MUX2_D1", "GEN_AOI21_D1", "GEN_OAI21_D1"]
SYNTH_WEIGHTS = [15, 5, 15, 10, 10, 10, 8, 3, 3, 8, 7, 6, 6]
