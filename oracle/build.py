"""TEST INFRASTRUCTURE ONLY: build the CPU oracles.

1. oracle/_build/gls_oracle -- the C restatement (oracle/gls_oracle.c).
2. oracle/_ref/ref_sim      -- the reference's own serial simulator core.
3. oracle/_ref/ref_levels   -- the reference's levelization (GenerateAdjacencyList,
   SetInDegrees, TopologyOrder: src/process.cpp, from the second declaration
   of GenerateAdjacencyList, its definition, up to `main`) with
   oracle/ref_levels_driver.cpp.
4. oracle/_ref/ref_vcd      -- the reference's VCD reader (src/VCDParser.cpp and
   src/VCDValue.cpp as they are) with oracle/ref_vcd_driver.cpp.
5. oracle/_ref/ref_gpu_sim  -- the reference's GPU `simulate` tool (src/simulate.cu
   with its reader sources, as they are) for sm_103a, with the text-archive
   reader of oracle/boost_archive standing in for Boost: the reference GPU
   tool timed on the same GPU (it is not a parity oracle: it deviates from
   the serial core).
   Recipe: take src/simulate.cpp of the reference up to its `main` (which
   does not compile against the shipped VCDParser), rename its `calc` so
   oracle/ref_driver.cpp can choose the calc mode, and compile it with the
   reference headers, empty Boost stubs (oracle/boost_stub) and the shim
   header oracle/ref_shim/simulate.h.  The extracted sources are written to
   oracle/_ref/src (git-ignored, never committed) so that a machine without
   the reference checkout can rebuild the same binary.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
BUILD = ORACLE / "_build"
REF = ORACLE / "_ref"
REF_SRC = REF / "src"
REFERENCE = Path(os.environ.get("GLS_REFERENCE", "/root/reference"))
REF_HEADERS = ["VCDTypes.h", "Function.h", "Instance.h", "PreProcess.h", "VCDValue.h", "VCDParser.h", "simulate.cuh"]
REF_SOURCES = ["VCDParser.cpp", "VCDValue.cpp", "simulate.cu", "PreProcess.cpp"]

ORACLE_BIN = BUILD / "gls_oracle"
REF_BIN = REF / "ref_sim"
REF_LEVELS_BIN = REF / "ref_levels"
REF_VCD_BIN = REF / "ref_vcd"
REF_GPU_BIN = REF / "ref_gpu_sim"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"{' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    src = ORACLE / "gls_oracle.c"
    if force or not ORACLE_BIN.exists() or ORACLE_BIN.stat().st_mtime < src.stat().st_mtime:
        _run(["gcc", "-O2", "-std=c11", "-pthread", "-o", str(ORACLE_BIN), str(src)])
    return ORACLE_BIN


def extract_reference() -> bool:
    """Write oracle/_ref/src from the reference checkout; False if absent."""
    sim = REFERENCE / "src" / "simulate.cpp"
    if not sim.exists():
        return False
    REF_SRC.mkdir(parents=True, exist_ok=True)
    text = sim.read_text()
    cut = text.index("\nint main(")
    core = text[:cut]
    core, n = re.subn(r"\bvoid calc\(std::string name", "void gls_ref_calc_literal(std::string name", core)
    if n != 1:
        raise RuntimeError("reference calc definition not found")
    (REF_SRC / "ref_core.cpp").write_text(core)
    proc = (REFERENCE / "src" / "process.cpp").read_text()
    decl = "void GenerateAdjacencyList("
    first = proc.index(decl)
    body = proc.index(decl, first + len(decl))   # the definition follows the declarations
    levels = proc[body: proc.index("\nint main(")]
    (REF_SRC / "ref_levels_core.cpp").write_text(
        "#include <algorithm>\n#include <map>\n#include <string>\n#include <vector>\n#include \"Instance.h\"\n"
        "using namespace std;\n" + levels)
    for h in REF_HEADERS + REF_SOURCES:
        shutil.copyfile(REFERENCE / "src" / h, REF_SRC / h)
    return True


def build_reference(force: bool = False) -> Path | None:
    """Build oracle/_ref/ref_sim; None when no reference sources are present."""
    have = extract_reference() or (REF_SRC / "ref_core.cpp").exists()
    if not have:
        return None
    deps = [REF_SRC / "ref_core.cpp", ORACLE / "ref_driver.cpp", ORACLE / "ref_shim" / "simulate.h"]
    if force or not REF_BIN.exists() or any(REF_BIN.stat().st_mtime < d.stat().st_mtime for d in deps):
        # -DNDEBUG: the reference's asserts would abort on inputs its release
        # behaviour handles (an X input edge is taken as posedge).
        _run(["g++", "-O2", "-std=c++17", "-DNDEBUG", "-pthread", "-w",
              f"-I{ORACLE / 'ref_shim'}", f"-I{ORACLE / 'boost_stub'}", f"-I{REF_SRC}",
              "-o", str(REF_BIN), str(REF_SRC / "ref_core.cpp"), str(ORACLE / "ref_driver.cpp")])
    _build_ref_tool(REF_LEVELS_BIN, [REF_SRC / "ref_levels_core.cpp", ORACLE / "ref_levels_driver.cpp"], force)
    _build_ref_tool(REF_VCD_BIN, [REF_SRC / "VCDParser.cpp", REF_SRC / "VCDValue.cpp", ORACLE / "ref_vcd_driver.cpp"],
                    force)
    return REF_BIN


def _build_ref_tool(exe: Path, srcs: list[Path], force: bool):
    if not all(p.exists() for p in srcs):
        return
    if force or not exe.exists() or any(exe.stat().st_mtime < p.stat().st_mtime for p in srcs):
        _run(["g++", "-O2", "-std=c++17", "-DNDEBUG", "-pthread", "-w", f"-I{ORACLE / 'boost_stub'}", f"-I{REF_SRC}",
              "-o", str(exe), *map(str, srcs)])


def build_reference_gpu(force: bool = False) -> Path | None:
    """Build oracle/_ref/ref_gpu_sim (nvcc, sm_103a); None without the sources."""
    if not (REF_SRC / "simulate.cu").exists() and not extract_reference():
        return None
    srcs = [REF_SRC / "simulate.cu", REF_SRC / "VCDParser.cpp", REF_SRC / "VCDValue.cpp", REF_SRC / "PreProcess.cpp"]
    stub = ORACLE / "boost_archive"
    deps = srcs + list((stub / "boost" / "archive").glob("*.hpp"))
    if force or not REF_GPU_BIN.exists() or any(REF_GPU_BIN.stat().st_mtime < d.stat().st_mtime for d in deps):
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        _run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w", "-DNDEBUG",
              f"-I{stub}", f"-I{REF_SRC}", "-o", str(REF_GPU_BIN), *map(str, srcs)])
    return REF_GPU_BIN


def build_all(force: bool = False):
    return build_oracle(force), build_reference(force)


if __name__ == "__main__":
    print(build_all(force=True))
