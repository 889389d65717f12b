"""Build of the command-line tools gls_process, gls_simulate and
gls_vcd2stim (C++, host only) into gate-level-simulator_gb300/bin, linked
against libgls."""
from __future__ import annotations

import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

from .build import BIN_DIR, LIB, LIB_DIR, PKG, REPO

HOST = PKG / "host"
TOOLS = {
    "gls_process": ["design.cpp", "boost_inter.cpp", "pack_gpu.cpp", "gls_process.cpp"],
    "gls_simulate": ["design.cpp", "boost_inter.cpp", "vcd.cpp", "stim_bin.cpp", "gls_simulate.cpp"],
    "gls_vcd2stim": ["design.cpp", "boost_inter.cpp", "vcd.cpp", "stim_bin.cpp", "gls_vcd2stim.cpp"],
}


def _build_tool(name: str, srcs: list[str], force: bool) -> Path:
    out = BIN_DIR / name
    deps = [HOST / s for s in srcs] + list(HOST.glob("*.h")) + [REPO / "include" / "gls.h"]
    if not force and out.exists() and all(d.stat().st_mtime <= out.stat().st_mtime for d in deps):
        return out
    cmd = ["g++", "-std=c++17", "-O2", f"-I{REPO / 'include'}", f"-I{HOST}", *map(str, (HOST / s for s in srcs)),
           "-o", str(out), "-pthread"]
    cmd += [f"-L{LIB_DIR}", "-lgls", "-Wl,-rpath,$ORIGIN/../lib"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"building {name} failed:\n{r.stdout}\n{r.stderr}")
    return out


def build(force: bool = False) -> dict[str, Path]:
    BIN_DIR.mkdir(exist_ok=True)
    if not LIB.exists():
        raise RuntimeError("libgls.so must be built first")
    with ThreadPoolExecutor(max_workers=len(TOOLS)) as ex:
        futs = {n: ex.submit(_build_tool, n, s, force) for n, s in TOOLS.items()}
        return {n: f.result() for n, f in futs.items()}
