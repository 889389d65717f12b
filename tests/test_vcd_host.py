"""The command-line tools' host VCD reader (host/vcd.cpp, parse_vcd) against
a restatement of the reference's reading (src/VCDParser.cpp:283-717): the
body's token-by-token changes (`ref_changes` of test_gpu_vcd) appended per
signal with the same-time replacement and the bus-bit filtering.  No GPU."""
import subprocess

import pytest

from test_gpu_vcd import random_vcd, ref_changes

DRIVER = r"""
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
    if (!glsh::parse_vcd(ss.str(), v, &err)) { printf("ERR %s\n", err.c_str()); return 1; }
    for (size_t k = 0; k < v.names.size(); ++k) {
        printf("%s", v.names[k].c_str());
        for (size_t j = 0; j < v.times[k].size(); ++j)
            printf(" %llu:%u", (unsigned long long)v.times[k][j], (unsigned)v.values[k][j]);
        printf("\n");
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def reader(libgls, tmp_path_factory):
    from gls.build import LIB_DIR, PKG, REPO
    d = tmp_path_factory.mktemp("vcdrd")
    (d / "drv.cpp").write_text(DRIVER)
    exe = d / "drv"
    r = subprocess.run(["g++", "-O1", "-std=c++17", f"-I{REPO / 'include'}", f"-I{PKG / 'host'}", str(d / "drv.cpp"),
                        str(PKG / "host" / "vcd.cpp"), f"-L{LIB_DIR}", "-lgls", f"-Wl,-rpath,{LIB_DIR}", "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def expected_lists(body, codes, n_sig):
    """Per signal (time, value) lists: bus bits keep only real changes,
    starting from Z; a later change at the same time replaces an earlier."""
    lists = [[] for _ in range(n_sig)]
    last = [2] * n_sig
    for k, t, v, bus in ref_changes(body, codes):
        if v == 255:
            continue
        if bus:
            if v == last[k]:
                continue
            last[k] = v
        if lists[k] and lists[k][-1][0] == t:
            lists[k][-1] = (t, v)
        else:
            lists[k].append((t, v))
    return lists


@pytest.mark.parametrize("seed", range(4))
def test_host_vcd_reader_matches_restatement(seed, reader, tmp_path):
    body, codes = random_vcd(seed)
    # a one-bit declaration is a scalar in a header (no range makes it a bus)
    codes = {c: [(bits, len(bits) > 1) for bits, _ in decls] for c, decls in codes.items()}
    # a header declaring every code's bits as scalars or buses of fresh names
    head = ["$timescale 1ps $end", "$scope module top $end"]
    names = {}
    sig = 0
    for code, decls in codes.items():
        for bits, bus in decls:
            if bus:
                base = f"v{sig}"
                head.append(f"$var wire {len(bits)} {code} {base} [{len(bits) - 1}:0] $end")
                for i, b in enumerate(bits):
                    names[b] = f"{base}[{len(bits) - 1 - i}]"
            else:
                # a scalar declared on its own: one bit, no filtering
                assert len(bits) == 1
                head.append(f"$var wire 1 {code} s{sig} $end")
                names[bits[0]] = f"s{sig}"
            sig += len(bits)
    head += ["$upscope $end", "$enddefinitions $end"]
    text = ("\n".join(head) + "\n").encode() + body
    (tmp_path / "t.vcd").write_bytes(text)
    r = subprocess.run([str(reader), str(tmp_path / "t.vcd")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    got = {}
    for line in r.stdout.splitlines():
        parts = line.split()
        got[parts[0]] = [tuple(int(x) for x in p.split(":")) for p in parts[1:]]
    exp = expected_lists(body, codes, sig)
    for k in range(sig):
        assert got.get(names[k], []) == exp[k], names[k]


@pytest.fixture(scope="module")
def ref_vcd():
    from oracle import build
    if build.build_reference() is None or not build.REF_VCD_BIN.exists():
        pytest.skip("reference sources not available on this machine")
    return build.REF_VCD_BIN


def reference_lists(exe, path, t_end):
    """Every declared bit's change list as the reference's own reader gives it."""
    r = subprocess.run([str(exe), str(path), "0", str(t_end)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = {}
    for line in r.stdout.splitlines():
        if line.startswith("@ "):
            parts = line[2:].split()
            out[parts[0]] = [tuple(int(x) for x in p.split(":")) for p in parts[1:]]
    return out


@pytest.mark.parametrize("seed", range(4))
def test_host_vcd_reader_matches_reference_reader(seed, reader, ref_vcd, tmp_path):
    """The host reader against the reference's VCDParser (src/VCDParser.cpp,
    compiled from the reference sources) on VCDs as simulators write them."""
    from cases import standard_vcd
    (tmp_path / "s.vcd").write_text(standard_vcd(seed, n_scalar=10 + seed, n_bus=3 + seed))
    exp = reference_lists(ref_vcd, tmp_path / "s.vcd", 10**9)
    r = subprocess.run([str(reader), str(tmp_path / "s.vcd")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    got = {}
    for line in r.stdout.splitlines():
        parts = line.split()
        got[parts[0]] = [tuple(int(x) for x in p.split(":")) for p in parts[1:]]
    assert set(got) == set(exp)
    for name in exp:
        assert got[name] == exp[name], name


@pytest.mark.parametrize("case", range(2))
def test_host_vcd_reader_matches_reference_golden(case, reader, tmp_path):
    """The host reader against the golden digests of the reference reader's
    change lists (tests/golden/vcd_reference.json)."""
    from cases import standard_vcd
    from test_gpu_vcd import golden_vcd_cases, list_digests
    c = golden_vcd_cases()[case]
    (tmp_path / "s.vcd").write_text(standard_vcd(c["seed"], n_scalar=c["n_scalar"], n_bus=c["n_bus"],
                                                 n_times=c["n_times"]))
    r = subprocess.run([str(reader), str(tmp_path / "s.vcd")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert list_digests(r.stdout) == c["lists"]
