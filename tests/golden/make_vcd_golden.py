"""Golden output of the reference's own VCD reader (src/VCDParser.cpp,
compiled from the reference sources by oracle/build.py as oracle/_ref/ref_vcd)
on VCDs as simulators write them (tests/cases.py: standard_vcd, fixed seeds).
For every declared bit the file keeps the SHA-256 prefix of its change list
("name t:v t:v ...", as ref_vcd prints it) and the list's length, so that
machines without the reference sources (the GPU tests) can check a reader
against it.  Run: python tests/golden/make_vcd_golden.py"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
CASES = [{"seed": 50, "n_scalar": 12, "n_bus": 5, "n_times": 1500},
         {"seed": 51, "n_scalar": 16, "n_bus": 6, "n_times": 1800}]


def digest(line: str) -> str:
    return hashlib.sha256(line.encode()).hexdigest()[:20]


def main():
    sys.path[:0] = [str(REPO), str(REPO / "gate-level-simulator_gb300"), str(REPO / "tests")]
    from cases import standard_vcd
    from oracle import build
    if build.build_reference() is None:
        raise SystemExit("the reference sources are needed")
    out = []
    with tempfile.TemporaryDirectory() as d:
        for c in CASES:
            p = Path(d) / "s.vcd"
            p.write_text(standard_vcd(c["seed"], n_scalar=c["n_scalar"], n_bus=c["n_bus"], n_times=c["n_times"]))
            r = subprocess.run([str(build.REF_VCD_BIN), str(p), "0", str(10**9)], capture_output=True, text=True,
                               check=True)
            lists = {}
            for line in r.stdout.splitlines():
                if line.startswith("@ "):
                    body = line[2:]
                    lists[body.split()[0]] = {"sha": digest(body), "n": len(body.split()) - 1}
            out.append(dict(c, lists=lists))
    (HERE / "vcd_reference.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
