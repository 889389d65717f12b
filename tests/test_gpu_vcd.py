"""GPU scan of VCD bodies (gls_vcd_scan) against the token-by-token reading
of the reference's VCDParser (src/VCDParser.cpp:508-717; restated below
as `ref_changes`, the same reading as host/vcd.cpp), and gls_simulate with
the GPU scan against gls_simulate --host-vcd."""
import subprocess

import numpy as np
import pytest

from gls import files, synth
from gls.capi import vcd_scan

pytestmark = pytest.mark.gpu
CODE = {ord("0"): 0, ord("1"): 3, ord("x"): 1, ord("X"): 1, ord("z"): 2, ord("Z"): 2}


def ref_changes(body: bytes, codes):
    """Every bit change in file order as (signal, time, value, bus); value 255
    for a character that is no value."""
    toks = body.split()
    out, now, i = [], 0, 0
    while i < len(toks):
        t = toks[i]
        i += 1
        c = t[0]
        if c == ord("#"):
            digits = b""
            for ch in t[1:]:
                if not 48 <= ch <= 57:
                    break
                digits += bytes([ch])
            now = int(digits) if digits else 0
            continue
        if c == ord("$"):
            if t == b"$comment":
                while i < len(toks) and toks[i] != b"$end":
                    i += 1
                i += 1
            continue
        if c in (ord("b"), ord("B")):
            if i >= len(toks):
                break
            code = toks[i].decode()
            i += 1
            bits = t[1:]
            for sig, bus in codes.get(code, []):
                w = len(sig)
                full = bits
                if len(full) < w:
                    f = full[:1]
                    pad = b"x" if f in (b"x", b"X") else (b"z" if f in (b"z", b"Z") else b"0")
                    full = pad * (w - len(full)) + full
                off = len(full) - w
                for b in range(w):
                    out.append((sig[b], now, CODE.get(full[off + b], 255), int(bus)))
            continue
        if c in (ord("r"), ord("R")):
            i += 1
            continue
        v = CODE.get(c)
        if v is None:
            continue
        for sig, bus in codes.get(t[1:].decode(), []):
            for k in sig:
                out.append((k, now, v, int(bus)))
    return out


def random_vcd(seed):
    rng = np.random.default_rng(seed)
    pool = [chr(c) for c in range(33, 127)]
    codes, n_sig = {}, 0
    names = ["#", "b", "0", "r", "1x", "!", "$a"]      # codes that look like other tokens
    while len(names) < 40:
        names.append("".join(rng.choice(pool, int(rng.integers(1, 5)))))
    for name in dict.fromkeys(names):
        decls = []
        for _ in range(int(rng.integers(1, 3))):       # some codes are declared twice
            w = int(rng.choice([1, 1, 1, 2, 4, 8]))
            decls.append((list(range(n_sig, n_sig + w)), w > 1 or bool(rng.integers(0, 2))))
            n_sig += w
        codes[name] = decls
    known = list(codes)
    parts, now = ["$dumpvars"], 0
    for _ in range(3000):
        r = rng.random()
        code = known[int(rng.integers(0, len(known)))] if rng.random() < 0.9 else "zz9unknown"
        if r < 0.08:
            now += int(rng.integers(0, 50))
            parts.append(f"#{now}")
        elif r < 0.55:
            parts.append(str(rng.choice(list("01xzXZq"))) + code)
        elif r < 0.85:
            bits = "".join(rng.choice(list("01xzXZ01"), int(rng.integers(0, 11))))
            parts.append(f"b{bits} {code}")
        elif r < 0.9:
            parts.append(f"r1.25 {code}")
        elif r < 0.93:
            parts.append("$comment b1 # 0! #99 $dumpvars $end")
        elif r < 0.96:
            parts.append(str(rng.choice(["$end", "$dumpall", "junk", "?x"])))
        else:
            parts.append(f"B{''.join(rng.choice(list('01'), 3))} {code}")
    seps = [" ", "\n", "\t", "  \n", "\r\n"]
    body = ""
    for p in parts:
        body += p + str(rng.choice(seps))
    return body.encode(), codes


@pytest.mark.parametrize("seed", range(8))
def test_gpu_vcd_scan_matches_token_reading(seed, gpu):
    body, codes = random_vcd(seed)
    sig, tim, val, bus, fallback = vcd_scan(body, codes)
    assert not fallback
    ref = ref_changes(body, codes)
    got = list(zip(sig.tolist(), tim.tolist(), val.tolist(), bus.tolist()))
    assert got == ref


def test_gpu_vcd_scan_edges(gpu):
    codes = {"!": [([0], False)], "#": [([1, 2, 3], True)]}
    assert vcd_scan(b"", codes)[0].size == 0
    assert vcd_scan(b"   \n\t ", codes)[0].size == 0
    body = b"#5 1! b1 # b10 #\n#7 b"            # the code '#' is no time; a trailing b has no code
    sig, tim, val, bus, fb = vcd_scan(body, codes)
    assert (sig.tolist(), tim.tolist(), val.tolist()) == ([0, 1, 2, 3, 1, 2, 3], [5] * 7, [3, 0, 0, 3, 0, 3, 0])
    # a code read where a keyword stands: the host reads that body
    assert vcd_scan(b"b1 $comment 1! $end", codes)[4]


def test_gls_simulate_gpu_vcd_same_saif(libgls, tmp_path):
    from gls import hostbuild
    tools = hostbuild.build()
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=900, cycles=300, depth=12)
    nl = synth.make_netlist(cfg, 3)
    st = synth.make_stimulus(cfg, nl.ppi_nets, 4)
    files.write_vlib(tmp_path / "lib.vlib")
    files.write_gv(tmp_path / "d.gv", nl)
    files.write_sdf(tmp_path / "d.sdf", nl)
    files.write_vcd(tmp_path / "d.vcd", nl, st)
    r = subprocess.run([str(tools["gls_process"]), str(tmp_path / "lib.vlib"), str(tmp_path / "d.gv"),
                        str(tmp_path / "d.sdf"), str(tmp_path / "inter.dat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    saifs = []
    for extra in ([], ["--host-vcd"]):
        out = tmp_path / f"out{len(extra)}.saif"
        r = subprocess.run([str(tools["gls_simulate"]), str(tmp_path / "inter.dat"), str(tmp_path / "d.vcd"), "0",
                            str(cfg.t_end), str(out), *extra], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        saifs.append(out.read_text())
    assert saifs[0] == saifs[1]


GPU_READER = r"""
#include <cstdio>
#include <fstream>
#include <sstream>
#include "vcd.h"
int main(int argc, char **argv)
{
    std::ifstream f(argv[1], std::ios::binary);
    std::stringstream ss;
    ss << f.rdbuf();
    glsh::VcdData v;
    std::string err;
    const int rc = glsh::parse_vcd_gpu(ss.str(), v, &err, 0);
    if (rc < 0) { printf("ERR %s\n", err.c_str()); return 1; }
    if (rc == 0) { printf("ERR the host read the body\n"); return 1; }
    for (size_t k = 0; k < v.names.size(); ++k) {
        printf("%s", v.names[k].c_str());
        for (size_t j = 0; j < v.times[k].size(); ++j)
            printf(" %llu:%u", (unsigned long long)v.times[k][j], (unsigned)v.values[k][j]);
        printf("\n");
    }
    return 0;
}
"""


def golden_vcd_cases():
    import json
    from pathlib import Path
    return json.loads((Path(__file__).resolve().parent / "golden" / "vcd_reference.json").read_text())


def list_digests(text):
    """SHA-256 prefix and length of every "name t:v ..." line (the golden's form)."""
    import hashlib
    out = {}
    for line in text.splitlines():
        parts = line.split()
        if parts:
            out[parts[0]] = {"sha": hashlib.sha256(line.encode()).hexdigest()[:20], "n": len(parts) - 1}
    return out


@pytest.mark.parametrize("case", range(2))
def test_gpu_vcd_reading_matches_reference_reader(case, gpu, tmp_path):
    """The GPU body scan (gls_vcd_scan through the host's parse_vcd_gpu)
    against the reference's own VCDParser (src/VCDParser.cpp): the golden
    digests of its change lists (tests/golden/make_vcd_golden.py) on VCDs as
    simulators write them."""
    from cases import standard_vcd
    from gls.build import LIB_DIR, PKG, REPO
    c = golden_vcd_cases()[case]
    (tmp_path / "drv.cpp").write_text(GPU_READER)
    exe = tmp_path / "drv"
    r = subprocess.run(["g++", "-O1", "-std=c++17", f"-I{REPO / 'include'}", f"-I{PKG / 'host'}", str(tmp_path / "drv.cpp"),
                        str(PKG / "host" / "vcd.cpp"), f"-L{LIB_DIR}", "-lgls", f"-Wl,-rpath,{LIB_DIR}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    (tmp_path / "s.vcd").write_text(standard_vcd(c["seed"], n_scalar=c["n_scalar"], n_bus=c["n_bus"],
                                                 n_times=c["n_times"]))
    r = subprocess.run([str(exe), str(tmp_path / "s.vcd")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert list_digests(r.stdout) == c["lists"]
