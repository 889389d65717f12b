"""TEST INFRASTRUCTURE ONLY: the case / result files the CPU oracles read.

Case file (little endian):
    "GLSCASE1"
    u32 n_nets
    u32 n_cells; per cell: u8 n_in, u8 n_out, u8 n_prim,
                  per primitive: u8 func, u8 n_pins, u8 pins[n_pins] (driven pin last)
    u32 n_inst;  per instance (level order): u32 cell, u32 level,
                  u32 in_net[n_in], u32 out_net[n_out],
                  u16 n_arcs, per arc: u8 edge, u8 in_pin, u8 out_pin, u8 0, f64 rise, f64 fall
    u32 n_stim;  per stimulus net: u32 net, u32 n, u64 time[n], u8 value[n]
    u64 t_begin, u64 t_end
Result file:
    "GLSRES01", u32 n_nets,
    per net: u64 n (UINT64_MAX = not produced), u64 time[n], u8 value[n]
    per net: u64 T0, T1, TX
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np


def write_case(path, nl, st, t_begin: int, t_end: int, inst_range: tuple[int, int] | None = None,
               stim_override=None) -> None:
    """Write netlist + stimulus.  `inst_range` restricts the instances written;
    `stim_override` replaces the stimulus (dict net -> (times, values))."""
    out = bytearray()
    out += b"GLSCASE1"
    out += struct.pack("<I", nl.n_nets)
    out += struct.pack("<I", len(nl.cells))
    for c in nl.cells:
        prog = c.program()
        out += struct.pack("<BBB", c.n_in, c.n_out, len(prog))
        for fn, pins in prog:
            out += struct.pack("<BB", fn, len(pins)) + bytes(pins)
    lo, hi = inst_range if inst_range else (0, nl.n_inst)
    lv_of = np.searchsorted(nl.level_start, np.arange(nl.n_inst), side="right") - 1
    out += struct.pack("<I", hi - lo)
    for i in range(lo, hi):
        c = nl.cells[int(nl.inst_cell[i])]
        p = int(nl.pin_start[i])
        out += struct.pack("<II", int(nl.inst_cell[i]), int(lv_of[i]))
        out += np.asarray(nl.pin_net[p: p + c.n_in + c.n_out], "<u4").tobytes()
        a0, a1 = int(nl.arc_start[i]), int(nl.arc_start[i + 1])
        out += struct.pack("<H", a1 - a0)
        for a in nl.arcs[a0:a1]:
            out += struct.pack("<BBBBdd", int(a["edge"]), int(a["in_pin"]), int(a["out_pin"]), 0,
                               float(a["rise"]), float(a["fall"]))
    if stim_override is not None:
        items = list(stim_override.items())
    else:
        items = [(int(st.nets[k]), st.events_of(k)) for k in range(len(st.nets))]
    out += struct.pack("<I", len(items))
    for net, (t, v) in items:
        out += struct.pack("<II", int(net), len(t))
        out += np.asarray(t, "<u8").tobytes()
        out += np.asarray(v, "u1").tobytes()
    out += struct.pack("<QQ", t_begin, t_end)
    Path(path).write_bytes(bytes(out))


def read_result(path):
    """-> (waves: dict net -> (times u64, values u8), saif: (n_nets, 3) uint64)."""
    b = Path(path).read_bytes()
    assert b[:8] == b"GLSRES01", "bad result magic"
    (n,) = struct.unpack_from("<I", b, 8)
    off = 12
    waves = {}
    for net in range(n):
        (cnt,) = struct.unpack_from("<Q", b, off)
        off += 8
        if cnt == 2**64 - 1:
            continue
        t = np.frombuffer(b, "<u8", cnt, off)
        off += 8 * cnt
        v = np.frombuffer(b, "u1", cnt, off)
        off += cnt
        waves[net] = (t.copy(), v.copy())
    saif = np.frombuffer(b, "<u8", 3 * n, off).reshape(n, 3).copy()
    return waves, saif
