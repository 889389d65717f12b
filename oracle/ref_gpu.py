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
    args = ap.parse_args()
    from gls import hostbuild, synth
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
