"""File forms of a workload: Verilog cell library, gate-level netlist, SDF,
VCD, and the native inter.dat written by gls_process.

The netlist is written the way the reference's front end reads it
(src/PreProcess.cpp:650-1274): a flat top module with named port
connections; register Q pins come from GEN_DF_D1 instances, which the front
end skips, so their nets are driven by the VCD.  The SDF carries IOPATH
delays (the only delays the reference reads, src/PreProcess.cpp:1276-1464)
and, to show they are ignored, INTERCONNECT entries.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

from .cells import FUNC_NAMES, LIBRARY, CellDef
from .netlist import ARC_DTYPE, Netlist, Stimulus


def _verilog_cell(c: CellDef) -> str:
    ports = c.inputs + c.outputs
    lines = [f"module {c.name} ({','.join(ports)});"]
    lines += [f"  input {p};" for p in c.inputs]
    lines += [f"  output {p};" for p in c.outputs]
    if c.wires:
        lines.append(f"  wire {', '.join(c.wires)};")
    if c.ignored:
        lines += ["  reg notifier;", "  supply1 cdn;", "  supply1 sdn;",
                  f"  udp_dff udpi0 ({c.outputs[0]}, {', '.join(c.inputs)}, cdn, sdn, notifier);"]
    for k, (fn, out, ins) in enumerate(c.prims):
        inst = f" udpi{k}" if fn.startswith("udp_") else ""
        lines.append(f"  {fn}{inst} ({out}, {', '.join(ins)});")
    lines.append("  specify")
    for edge, i, o in c.arcs:
        src = i if edge == 2 else f"{'posedge' if edge == 0 else 'negedge'} {i}"
        lines.append(f"    ({src} => {o}) = (1, 1);")
    lines += ["  endspecify", "endmodule"]
    return "\n".join(lines)


def write_vlib(path, cells=None) -> None:
    """The cells as a Verilog library module file (our restatement of the
    GEN_*_D1 modules) with the two UDPs they use."""
    cells = cells or list(LIBRARY.values())
    udps = """primitive udp_xbuf (o, i, check_signal);
  output o;
  input i, check_signal;
  table
    0 1 : 0;
    1 1 : 1;
    x 1 : 1;
  endtable
endprimitive
primitive udp_mux2 (z, i0, i1, s);
  output z;
  input i0, i1, s;
  table
    1 ? 0 : 1;
    0 ? 0 : 0;
    ? 1 1 : 1;
    ? 0 1 : 0;
    0 0 x : 0;
    1 1 x : 1;
  endtable
endprimitive
"""
    Path(path).write_text("`timescale 1ps/1ps\n" + udps + "\n".join(_verilog_cell(c) for c in cells) + "\n")


def write_gv(path, nl: Netlist, top: str = "top", order=None) -> None:
    """The netlist as a flat gate-level Verilog file; `order` lists the
    instances in the order to write them (default: instance order)."""
    n_reg = int(nl.extra.get("n_reg", 0))
    ppi = [int(x) for x in nl.ppi_nets]
    regs = ppi[len(ppi) - n_reg:] if n_reg else []
    pis = ppi[: len(ppi) - n_reg] if n_reg else ppi
    out = [f"module {top} (clk, {', '.join(nl.net_name(n) for n in pis)});",
           "input clk;"]
    out += [f"input {nl.net_name(n)};" for n in pis]
    driven = set(int(x) for x in nl.gate_output_nets())
    wires = [n for n in range(nl.n_nets) if n not in set(pis)]
    for k in range(0, len(wires), 16):
        out.append("wire " + ", ".join(nl.net_name(n) for n in wires[k: k + 16]) + ";")
    gate_outs = sorted(driven)
    for k, q in enumerate(regs):
        d = nl.net_name(gate_outs[k % len(gate_outs)]) if gate_outs else "clk"
        out.append(f"GEN_DF_D1 R{k} ( .d({d}), .cp(clk), .q({nl.net_name(q)}) );")
    for i in (range(nl.n_inst) if order is None else (int(x) for x in order)):
        c = nl.cells[int(nl.inst_cell[i])]
        ins, outs = nl.inputs_of(i), nl.outputs_of(i)
        conns = [f".{p}({nl.net_name(int(n))})" for p, n in zip(c.inputs, ins)]
        conns += [f".{p}({nl.net_name(int(n))})" for p, n in zip(c.outputs, outs)]
        out.append(f"{c.name} {nl.inst_name(i)} ( {', '.join(conns)} );")
    out.append("endmodule")
    Path(path).write_text("\n".join(out) + "\n")


def write_sdf(path, nl: Netlist, top: str = "top", interconnect: bool = True) -> None:
    out = ['(DELAYFILE', '  (SDFVERSION "3.0")', f'  (DESIGN "{top}")', "  (TIMESCALE 1ps)"]
    rng = np.random.default_rng(0)
    if interconnect:
        out += ['  (CELL (CELLTYPE "top") (INSTANCE)', "    (DELAY (ABSOLUTE"]
        for i in range(min(nl.n_inst, 50)):
            c = nl.cells[int(nl.inst_cell[i])]
            d = int(rng.integers(0, 11))
            out.append(f"      (INTERCONNECT {nl.net_name(int(nl.inputs_of(i)[0]))} {nl.inst_name(i)}/{c.inputs[0]} "
                       f"({d}:{d}:{d}))")
        out += ["    ))", "  )"]
    for i in range(nl.n_inst):
        c = nl.cells[int(nl.inst_cell[i])]
        out.append(f'  (CELL (CELLTYPE "{c.name}") (INSTANCE {nl.inst_name(i)})')
        out.append("    (DELAY (ABSOLUTE")
        for a in nl.arcs[int(nl.arc_start[i]): int(nl.arc_start[i + 1])]:
            ip, op = c.inputs[int(a["in_pin"])], c.outputs[int(a["out_pin"])]
            src = ip if int(a["edge"]) == 2 else f"({'posedge' if int(a['edge']) == 0 else 'negedge'} {ip})"
            r, f = a["rise"], a["fall"]
            out.append(f"      (IOPATH {src} {op} ({r:g}:{r:g}:{r:g}) ({f:g}:{f:g}:{f:g}))")
        out.append("    ))")
        out.append("  )")
    out.append(")")
    Path(path).write_text("\n".join(out) + "\n")


def _vcd_id(k: int) -> str:
    s = ""
    k += 1
    while k:
        k, r = divmod(k - 1, 94)
        s = chr(33 + r) + s
    return s


def write_vcd(path, nl: Netlist, st: Stimulus, top: str = "top") -> None:
    names = [nl.net_name(int(n)) for n in st.nets]
    ids = [_vcd_id(k) for k in range(len(names))]
    head = ["$timescale 1ps $end", f"$scope module {top} $end"]
    head += [f"$var wire 1 {i} {n} $end" for i, n in zip(ids, names)]
    head += ["$upscope $end", "$enddefinitions $end"]
    lens = np.diff(st.ev_start.astype(np.int64))
    who = np.repeat(np.arange(len(names)), lens)
    order = np.lexsort((who, st.time))
    t_sorted, w_sorted, v_sorted = st.time[order], who[order], st.value[order]
    ch = "0xz1"
    body = []
    cur = None
    for t, w, v in zip(t_sorted.tolist(), w_sorted.tolist(), v_sorted.tolist()):
        if t != cur:
            body.append(f"#{t}")
            if cur is None:
                body.append("$dumpvars")
            cur = t
        body.append(f"{ch[v]}{ids[w]}")
    Path(path).write_text("\n".join(head + body) + "\n")


def write_stim_bin(path, nl: Netlist, st: Stimulus, time_res: int = 1, time_unit: str = "ps") -> None:
    """The stimulus as the tools' binary stimulus file (layout in
    host/vcd.h), the same bytes gls_vcd2stim writes for write_vcd's file:
    one scalar signal per stimulus net, named as the netlist names it."""
    names = [nl.net_name(int(n)) for n in st.nets]
    out = bytearray(b"GLSSTIM1")
    out += struct.pack("<III", time_res, len(names), len(names))
    u = time_unit.encode()
    out += struct.pack("<I", len(u)) + u
    for nm in names:
        b = nm.encode()
        out += struct.pack("<I", len(b)) + b
    for nm in names:
        b = nm.encode()
        out += struct.pack("<I", len(b)) + b + b"\x00"
    out += np.asarray(st.ev_start, "<u8").tobytes()
    out += np.asarray(st.time, "<u8").tobytes()
    out += np.asarray(st.value, "u1").tobytes()
    Path(path).write_bytes(bytes(out))


def read_stim_bin(path):
    """A binary stimulus file as (time_res, time_unit, names, decl_bits,
    start, time, value); decl_bits is a list of (name, bus)."""
    b = Path(path).read_bytes()
    if b[:8] != b"GLSSTIM1":
        raise ValueError("not a GLSSTIM1 file")
    res, ns, nd = struct.unpack_from("<III", b, 8)
    off = 20

    def s():
        nonlocal off
        (k,) = struct.unpack_from("<I", b, off)
        off += 4 + k
        return b[off - k: off].decode()

    unit = s()
    names = [s() for _ in range(ns)]
    decls = []
    for _ in range(nd):
        nm = s()
        decls.append((nm, b[off] != 0))
        off += 1
    start = np.frombuffer(b, "<u8", ns + 1, off)
    off += 8 * (ns + 1)
    total = int(start[-1])
    time = np.frombuffer(b, "<u8", total, off)
    value = np.frombuffer(b, "u1", total, off + 8 * total)
    return res, unit, names, decls, start, time, value


def read_inter(path):
    """The native inter.dat of gls_process as a dict of plain arrays."""
    b = Path(path).read_bytes()
    if b[:8] != b"GLSINTR1":
        raise ValueError("not a gls inter.dat")
    off = 8

    def u8():
        nonlocal off
        off += 1
        return b[off - 1]

    def u32():
        nonlocal off
        off += 4
        return struct.unpack_from("<I", b, off - 4)[0]

    def f64():
        nonlocal off
        off += 8
        return struct.unpack_from("<d", b, off - 8)[0]

    def s():
        n = u32()
        nonlocal off
        off += n
        return b[off - n: off].decode()

    top = s()
    nets = [s() for _ in range(u32())]
    cells = []
    for _ in range(u32()):
        name = s()
        ins = [s() for _ in range(u32())]
        outs = [s() for _ in range(u32())]
        prims = []
        for _ in range(u32()):
            f = u8()
            k = u8()
            prims.append((f, [u8() for _ in range(k)]))
        cells.append((name, ins, outs, prims))
    insts = []
    for _ in range(u32()):
        name = s()
        cell = u32()
        pins = [u32() for _ in range(u32())]
        arcs = [(u8(), u8(), u8(), f64(), f64()) for _ in range(u32())]
        insts.append((name, cell, pins, arcs))
    level_start = [u32() for _ in range(u32())]
    constants = [(u32(), u8()) for _ in range(u32())]
    aliases = [(u32(), u32()) for _ in range(u32())]
    bus_bits = [u32() for _ in range(u32())]
    return dict(top=top, nets=nets, cells=cells, insts=insts, level_start=level_start, constants=constants,
                aliases=aliases, bus_bits=bus_bits)


def parse_saif(text: str) -> dict[str, tuple[int, int, int]]:
    """net -> (T0, T1, TX) of every NET record of a SAIF file, with nested
    instance records named inst[net]."""
    import re

    out = {}
    inst_stack = []
    lines = text.splitlines()
    for k, line in enumerate(lines):
        s = line.strip()
        m = re.match(r"\(INSTANCE (\S+)", s)
        if m:
            inst_stack.append(m.group(1))
            continue
        m = re.match(r"\(T0 (\d+)\) \(T1 (\d+)\) \(TX (\d+)\)", s)
        if m:
            name = lines[k - 1].strip()[1:]
            if len(inst_stack) > 1:
                name = f"{inst_stack[-1]}[{name}]"
            out[name] = (int(m.group(1)), int(m.group(2)), int(m.group(3)))
    return out


def netlist_from_inter(d: dict):
    """A Netlist equal to what gls_simulate hands to libgls for an inter.dat
    (reads through assign aliases resolved), plus the constant nets."""
    from .cells import CellDef
    from .netlist import ARC_DTYPE, Netlist

    alias = dict(d["aliases"])

    def resolve(n):
        for _ in range(64):
            if n not in alias:
                break
            n = alias[n]
        return n

    cells = []
    for name, ins, outs, prims in d["cells"]:
        c = CellDef(name, list(ins), list(outs), [])
        c._program = [(f, list(p)) for f, p in prims]
        c.program = (lambda prog: (lambda: prog))(c._program)
        cells.append(c)
    inst_cell, pin_start, pin_net, arc_start, arcs = [], [0], [], [0], []
    for name, cell, pins, arcl in d["insts"]:
        n_in = len(d["cells"][cell][1])
        inst_cell.append(cell)
        pin_net += [resolve(p) if k < n_in else p for k, p in enumerate(pins)]
        pin_start.append(len(pin_net))
        arcs += [(e, i, o, (0,) * 5, r, f) for e, i, o, r, f in arcl]
        arc_start.append(len(arcs))
    n_in_of = [len(d["cells"][c][1]) for c in inst_cell]
    read = {pin_net[pin_start[i] + k] for i in range(len(inst_cell)) for k in range(n_in_of[i])}
    driven = {pin_net[pin_start[i] + k] for i in range(len(inst_cell))
              for k in range(n_in_of[i], pin_start[i + 1] - pin_start[i])}
    return Netlist(
        n_nets=len(d["nets"]), cells=cells, inst_cell=np.array(inst_cell, np.uint32),
        level_start=np.array(d["level_start"], np.uint32), pin_start=np.array(pin_start, np.uint32),
        pin_net=np.array(pin_net, np.uint32), arc_start=np.array(arc_start, np.uint32),
        arcs=np.array(arcs, ARC_DTYPE) if arcs else np.zeros(0, ARC_DTYPE),
        ppi_nets=np.array(sorted(read - driven), np.uint32), net_names=list(d["nets"]),
        inst_names=[x[0] for x in d["insts"]], extra={"constants": dict(d["constants"]), "aliases": alias})
