"""TEST INFRASTRUCTURE ONLY: run the CPU oracles on a netlist + stimulus.

`run_oracle` runs the C restatement (oracle/gls_oracle.c); `run_reference`
runs the reference's own serial simulator core (oracle/_ref/ref_sim) and
parses the SAIF file the reference's DumpSaif writes.
"""
from __future__ import annotations

import re
import subprocess
import tempfile
import time
from pathlib import Path

import numpy as np

from . import build
from .casefile import read_result, write_case

SAIF_NET = re.compile(r"^\s*\((\S+)\s*\n\s*\(T0 (\d+)\) \(T1 (\d+)\) \(TX (\d+)\)", re.M)


def parse_saif_records(text: str) -> dict[str, tuple[int, int, int]]:
    """net name -> (T0, T1, TX) of every NET record of a SAIF file."""
    return {m.group(1): (int(m.group(2)), int(m.group(3)), int(m.group(4))) for m in SAIF_NET.finditer(text)}


def run_oracle(nl, st, t_begin, t_end, calc="fixed", threads=1, factor=1.0, workdir=None, keep=None,
               verify_lookup=False, **case_kw):
    """keep: only these nets' waveforms come back (every list is dropped
    after the last level that reads it, so a large design fits in host
    memory); SAIF counts come back for every net either way."""
    exe = build.build_oracle()
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        case, res = Path(d) / "c.bin", Path(d) / "r.bin"
        write_case(case, nl, st, t_begin, t_end, **case_kw)
        cmd = [str(exe), str(case), str(res), "--calc", calc, "--threads", str(threads), "--factor", repr(factor)]
        if keep is not None:
            k = np.unique(np.asarray(keep, np.uint32))
            (Path(d) / "keep.bin").write_bytes(np.uint32(len(k)).tobytes() + k.astype("<u4").tobytes())
            cmd += ["--keep", str(Path(d) / "keep.bin")]
        if verify_lookup:
            cmd += ["--verify-lookup"]
        t0 = time.perf_counter()
        subprocess.run(cmd, check=True)
        el = time.perf_counter() - t0
        waves, saif = read_result(res)
    return waves, saif, el


def run_reference(nl, st, t_begin, t_end, calc="fixed", threads=1, repeat=1, workdir=None, **case_kw):
    exe = build.build_reference()
    if exe is None:
        raise RuntimeError("reference sources not available (oracle/_ref/src missing)")
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        case, res, saif_path = Path(d) / "c.bin", Path(d) / "r.bin", Path(d) / "out.saif"
        write_case(case, nl, st, t_begin, t_end, **case_kw)
        r = subprocess.run([str(exe), str(case), str(res), str(saif_path), "--calc", calc,
                            "--threads", str(threads), "--repeat", str(repeat)],
                           check=True, capture_output=True, text=True)
        m = re.search(r"simulate ([0-9.eE+-]+) s", r.stderr)
        sim_s = float(m.group(1)) if m else float("nan")
        waves, saif = read_result(res)
        recs = parse_saif_records(saif_path.read_text())
    n = saif.shape[0]
    for name, v in recs.items():
        if name.startswith("n") and name[1:].isdigit() and int(name[1:]) < n:
            saif[int(name[1:])] = v
    return waves, saif, sim_s
