"""In-tree build of libgls.so (CUDA for sm_103a) and the host tools.

nvcc compiles every translation unit in parallel with one -gencode for
sm_103a; outputs go to gate-level-simulator_gb300/lib and .../bin.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent          # gate-level-simulator_gb300/
REPO = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
BIN_DIR = PKG / "bin"
OBJ_DIR = PKG / "_build"
LIB = LIB_DIR / "libgls.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", f"-I{REPO / 'include'}", f"-I{CSRC}"]

LIB_SOURCES = ["gls_kernels.cu", "gls_capi.cpp", "gls_cells.cpp", "gls_static.cu", "gls_presize.cu",
               "gls_levelize.cu", "gls_vcd.cu", "gls_pack.cu"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libgls")
    return exe


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, obj: Path):
    extra = os.environ.get("GLS_NVCC_FLAGS", "").split()   # tuning builds, e.g. -DGLS_SIM3_BLOCKS=7
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")


def build_lib(force: bool = False) -> Path:
    LIB_DIR.mkdir(exist_ok=True)
    OBJ_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [REPO / "include" / "gls.h"]
    srcs = [CSRC / s for s in LIB_SOURCES]
    objs = [OBJ_DIR / (s.name + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, [s, *headers])]
    with ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 1))) as ex:
        list(ex.map(lambda so: _compile(*so), todo))
    if force or todo or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"link of libgls.so failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def build_all(force: bool = False) -> None:
    build_lib(force)
    from . import hostbuild   # the command-line tools

    hostbuild.build(force)


if __name__ == "__main__":
    build_all(force=True)
    print(LIB)
