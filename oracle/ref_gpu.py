"""TEST INFRASTRUCTURE ONLY: the reference's own GPU `simulate` tool timed on
this GPU beside gls_simulate, on the same files.

oracle/_ref/ref_gpu_sim is src/simulate.cu of the reference (with its VCD
and PreProcess sources) built for sm_103a by oracle/build.py, reading its
inter.dat through the text-archive reader of oracle/boost_archive.  It is
a timing reference, not a parity oracle: the reference GPU tool deviates
from the serial core (32-bit times, t = 0 rows not evaluated, chunk seams,
and more), so its SAIF counts are compared only to report how many records
differ.

A workload is written as the reference's inputs: the cell library, the
netlist and SDF (gls.files), inter.dat by gls_process (the reference's Boost
text archive) and the stimulus VCD.  Both tools then run on those files:
the reference prints its own phase times ("total time of simulating",
"total time(all)"), gls_simulate its phase times and kernel time.

Command line (one GPU):
    python -m oracle.ref_gpu --config c1 [--cells N --depth D --cycles C] [--timeout S] [--gls-only]
"""
from __future__ import annotations

import argparse
import json
import re
import subprocess
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "gate-level-simulator_gb300"))


def write_inputs(d: Path, nl, st, tools) -> None:
    from gls import files
    files.write_vlib(d / "lib.vlib")
    files.write_gv(d / "d.gv", nl)
    files.write_sdf(d / "d.sdf", nl)
    files.write_vcd(d / "d.vcd", nl, st)
    r = subprocess.run([str(tools["gls_process"]), str(d / "lib.vlib"), str(d / "d.gv"), str(d / "d.sdf"),
                        str(d / "inter.dat")], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"gls_process failed:\n{r.stdout}")


# A small design that exercises what the generator's netlists do not: bus
# ports, assign aliases and constants, pins tied off, an output left open,
# a declared output bit nothing drives, input bits nothing reads, and VCD
# signals the design does not have.  The reference GPU tool made an illegal
# memory access on it (its RemoveInvalidStatesGPU kernel, at the second
# level; the GPU logged Xid 31), so this harness runs only gls_simulate on
# it.
BUS_GV = """module t (a, b, sel, d, o);
input [7:0] a;
input b, sel;
input [3:0] d;
wire [1:0] w;
wire x, y, z, k0, k1;
output [3:0] o;
assign k0 = 1'b1;
assign k1 = 1'b0;
assign y = x;
GEN_AND2_D1 U0 ( .a1(a[0]), .a2(a[1]), .z(x) );
GEN_NOR2_D1 U1 ( .a1(y), .a2(b), .zn(w[0]) );
GEN_MUX2_D1 U2 ( .i0(w[0]), .i1(a[3]), .s(sel), .z(w[1]) );
GEN_NAND2_D1 U3 ( .a1(k0), .a2(w[1]), .zn(o[0]) );
GEN_XOR2_D1 U4 ( .a1(1'b0), .a2(a[2]), .z(z) );
GEN_INV_D1 U5 ( .i(z) );
GEN_OR2_D1 U6 ( .a1(d[1]), .a2(a[5]), .z(o[2]) );
GEN_NAND3_D1 U7 ( .a1(a[6]), .a2(a[7]), .a3(k1), .zn(o[3]) );
endmodule
"""
BUS_SDF = """(DELAYFILE (TIMESCALE 1ps)
 (CELL (CELLTYPE "GEN_AND2_D1") (INSTANCE U0) (DELAY (ABSOLUTE (IOPATH a1 z (11:11:11) (13:13:13)) (IOPATH a2 z (17:17:17) (19:19:19)))))
 (CELL (CELLTYPE "GEN_NOR2_D1") (INSTANCE U1) (DELAY (ABSOLUTE (IOPATH a1 zn (5:5:5) (7:7:7)) (IOPATH a2 zn (9:9:9) (12:12:12)))))
 (CELL (CELLTYPE "GEN_MUX2_D1") (INSTANCE U2) (DELAY (ABSOLUTE (IOPATH i0 z (20:20:20) (21:21:21)) (IOPATH i1 z (22:22:22) (23:23:23))
    (IOPATH (posedge s) z (30:30:30) (31:31:31)) (IOPATH (negedge s) z (32:32:32) (33:33:33)))))
 (CELL (CELLTYPE "GEN_NAND2_D1") (INSTANCE U3) (DELAY (ABSOLUTE (IOPATH a1 zn (8:8:8) (9:9:9)) (IOPATH a2 zn (10:10:10) (14:14:14)))))
 (CELL (CELLTYPE "GEN_XOR2_D1") (INSTANCE U4) (DELAY (ABSOLUTE (IOPATH (posedge a1) z (4:4:4) (5:5:5)) (IOPATH (negedge a1) z (6:6:6) (7:7:7))
    (IOPATH (posedge a2) z (8:8:8) (9:9:9)) (IOPATH (negedge a2) z (10:10:10) (11:11:11)))))
 (CELL (CELLTYPE "GEN_INV_D1") (INSTANCE U5) (DELAY (ABSOLUTE (IOPATH i zn (3:3:3) (4:4:4)))))
 (CELL (CELLTYPE "GEN_OR2_D1") (INSTANCE U6) (DELAY (ABSOLUTE (IOPATH a1 z (6:6:6) (8:8:8)) (IOPATH a2 z (7:7:7) (9:9:9)))))
 (CELL (CELLTYPE "GEN_NAND3_D1") (INSTANCE U7) (DELAY (ABSOLUTE (IOPATH a1 zn (6:6:6) (7:7:7)) (IOPATH a2 zn (8:8:8) (9:9:9))
    (IOPATH a3 zn (10:10:10) (11:11:11)))))
)
"""


def bus_vcd(seed: int, n_times: int = 1500) -> str:
    """A VCD for BUS_GV in the subset the reference's reader handles (every
    change on its own line, full-width bus values, more than (2 x cores)^2
    timestamps), with two signals the design does not have."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sigs = [("!", "a", 8), ('"', "b", 0), ("#", "sel", 0), ("$", "d", 4), ("%", "e", 0), ("&", "f", 2)]
    head = ["$timescale 1ps $end", "$scope module t $end"]
    head += [f"$var wire {max(w, 1)} {c} {n}{f' [{w - 1}:0]' if w else ''} $end" for c, n, w in sigs]
    head += ["$upscope $end", "$enddefinitions $end"]
    alpha = "01xz"

    def val(w):
        pick = lambda: alpha[int(rng.choice(4, p=[0.46, 0.46, 0.05, 0.03]))]   # noqa: E731
        return pick() if w == 0 else "".join(pick() for _ in range(w))

    body = ["#0", "$dumpvars"] + [val(w) + c if w == 0 else f"b{val(w)} {c}" for c, _, w in sigs] + ["$end"]
    t = 0
    for _ in range(n_times):
        t += int(rng.integers(5, 60))
        body.append(f"#{t}")
        for j in rng.permutation(len(sigs))[: int(rng.integers(1, len(sigs) + 1))]:
            c, _, w = sigs[int(j)]
            body.append(val(w) + c if w == 0 else f"b{val(w)} {c}")
    return "\n".join(head + body) + "\n", t


def parse_ref_times(text: str) -> dict:
    """The phase times the reference GPU tool prints (milliseconds)."""
    keys = {"simulating": r"total time of simulating: (\d+)ms", "gpu": r"total time of gpu: (\d+)ms",
            "vcd_parse": r"total time of vcd parse: (\d+)ms", "all": r"total time\(all\): (\d+)ms",
            "without_vcd": r"total time\(not including read-vcd\): (\d+)ms"}
    out = {}
    for k, pat in keys.items():
        m = re.search(pat, text)
        if m:
            out[k] = int(m.group(1))
    return out


def parse_gls_times(text: str) -> dict:
    m = re.search(r"timing \(ms\): design ([\d.]+), stimulus ([\d.]+), simulate ([\d.]+) \(GPU kernels ([\d.]+)\), "
                  r"SAIF ([\d.]+), total ([\d.]+)", text)
    if not m:
        return {}
    return dict(zip(("design", "stimulus", "simulate", "gpu_kernels", "saif", "total"), map(float, m.groups())))


def record_names(text: str) -> list:
    """NET record names of a SAIF file, in file order."""
    lines = text.splitlines()
    return [lines[k - 1].strip()[1:] for k, x in enumerate(lines) if re.match(r"\s*\(T0 \d+\)", x)]


def compare_order(ref_text: str, gls_text: str) -> dict:
    """The reference GPU tool's SAIF file against gls_simulate's
    --saif-order=ref file: the record names in sequence, and the whole text
    with the counts blanked (their values differ where the reference GPU
    tool deviates from the serial core)."""
    a, b = record_names(ref_text), record_names(gls_text)
    k = 0
    while k < min(len(a), len(b)) and a[k] == b[k]:
        k += 1
    blank = lambda t: re.sub(r"\((T0|T1|TX) \d+\)", r"(\1 _)", t)
    return {"records_ref": len(a), "records_gls": len(b), "same_sequence": a == b,
            "first_difference": None if a == b else k, "same_text_without_counts": blank(ref_text) == blank(gls_text)}


def compare_saif(a: str, b: str) -> dict:
    from gls.files import parse_saif
    ra, rb = parse_saif(a), parse_saif(b)
    common = set(ra) & set(rb)
    return {"records_ref": len(ra), "records_gls": len(rb), "common": len(common),
            "differing": sum(ra[k] != rb[k] for k in common)}


def run(d: Path, t_begin: int, t_end: int, timeout: float, reference: bool = True) -> dict:
    from gls import hostbuild
    from oracle import build
    tools = hostbuild.build()
    res = {}
    r = None
    if reference:
        exe = build.build_reference_gpu()
        if exe is None:
            return {"unavailable": "the reference sources were not extracted (oracle/_ref/src)"}
        t0 = time.perf_counter()
        r = subprocess.run([str(exe), str(d / "inter.dat"), str(d / "d.vcd"), str(t_begin), str(t_end),
                            str(d / "ref.saif")], capture_output=True, text=True, timeout=timeout, cwd=d)
        res["ref_wall_s"] = time.perf_counter() - t0
        res["ref_rc"] = r.returncode
        res["ref_ms"] = parse_ref_times(r.stdout)
        (d / "ref.log").write_text(r.stdout + r.stderr)
    t0 = time.perf_counter()
    g = subprocess.run([str(tools["gls_simulate"]), str(d / "inter.dat"), str(d / "d.vcd"), str(t_begin), str(t_end),
                        str(d / "gls.saif")], capture_output=True, text=True, timeout=timeout)
    res["gls_wall_s"] = time.perf_counter() - t0
    res["gls_rc"] = g.returncode
    res["gls_ms"] = parse_gls_times(g.stdout)
    m = re.search(r"(\d+) gate-events", g.stdout)
    res["gate_events"] = int(m.group(1)) if m else None
    if r is not None and r.returncode == 0 and g.returncode == 0:
        res["saif"] = compare_saif((d / "ref.saif").read_text(), (d / "gls.saif").read_text())
        # the same files in the reference GPU tool's record order
        o = subprocess.run([str(tools["gls_simulate"]), str(d / "inter.dat"), str(d / "d.vcd"), str(t_begin),
                            str(t_end), str(d / "gls_ref_order.saif"), "--saif-order=ref"], capture_output=True,
                           text=True, timeout=timeout)
        if o.returncode == 0:
            res["saif_order"] = compare_order((d / "ref.saif").read_text(), (d / "gls_ref_order.saif").read_text())
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c1")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cells", type=int)
    ap.add_argument("--depth", type=int)
    ap.add_argument("--cycles", type=int)
    ap.add_argument("--timeout", type=float, default=900)
    ap.add_argument("--dir", default="/tmp/gls_ref_gpu")
    ap.add_argument("--gls-only", action="store_true", help="time gls_simulate alone (the reference tool is not run)")
    ap.add_argument("--design", default="generated", choices=["generated", "buses"],
                    help="buses: the small bus / alias / constant design of this file instead of the generator's "
                         "(gls_simulate only: the reference GPU tool faults on it)")
    args = ap.parse_args()
    from gls import files, hostbuild, synth
    if args.design == "buses":
        d = Path(args.dir)
        d.mkdir(parents=True, exist_ok=True)
        files.write_vlib(d / "lib.vlib")
        (d / "d.gv").write_text(BUS_GV)
        (d / "d.sdf").write_text(BUS_SDF)
        text, t_last = bus_vcd(args.seed)
        (d / "d.vcd").write_text(text)
        tools = hostbuild.build()
        r = subprocess.run([str(tools["gls_process"]), str(d / "lib.vlib"), str(d / "d.gv"), str(d / "d.sdf"),
                            str(d / "inter.dat")], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"gls_process failed:\n{r.stdout}")
        res = run(d, 50, t_last + 100, args.timeout, reference=False)
        res["workload"] = "buses"
        print(json.dumps(res))
        return
    cfg = synth.CONFIGS[args.config]
    if args.cells or args.depth or args.cycles:
        cfg = synth.scaled(cfg, cells=args.cells, depth=args.depth, cycles=args.cycles)
    d = Path(args.dir)
    d.mkdir(parents=True, exist_ok=True)
    t0 = time.time()
    nl = synth.make_netlist(cfg, seed=args.seed)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=args.seed)
    write_inputs(d, nl, st, hostbuild.build())
    prep = time.time() - t0
    res = run(d, 0, cfg.t_end, args.timeout, reference=not args.gls_only)
    res.update({"workload": args.config, "cells": int(nl.n_inst), "levels": int(nl.n_levels),
                "stimulus_events": int(st.n_events), "t_end": int(cfg.t_end), "inputs_written_s": prep})
    if res.get("gate_events") and res.get("ref_ms", {}).get("simulating"):
        res["ref_gate_events_per_s"] = res["gate_events"] / (res["ref_ms"]["simulating"] / 1000.0)
    if res.get("gate_events") and res.get("gls_ms", {}).get("simulate"):
        res["gls_gate_events_per_s"] = res["gate_events"] / (res["gls_ms"]["simulate"] / 1000.0)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
