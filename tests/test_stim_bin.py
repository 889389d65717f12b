"""The binary stimulus file (host/stim_bin.cpp, layout in host/vcd.h), on
the CPU:

* gls_vcd2stim writes exactly the change lists, timescale and declarations
  that the tools' VCD reader gives for the same VCD, and gls_simulate's
  loader reads them back unchanged;
* on the golden VCDs the loaded lists match the digests of the reference
  reader's lists (tests/golden/vcd_reference.json);
* the Python writer (gls.files.write_stim_bin) gives the converter's bytes
  for the VCD that gls.files.write_vcd writes of the same stimulus;
* damaged files are rejected with a message."""
import subprocess

import numpy as np
import pytest

from gls import files, synth

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
    const std::string b = ss.str();
    glsh::VcdData v;
    std::string err;
    const bool ok = glsh::is_stim_bin(b) ? glsh::load_stim_bin(b, v, &err) : glsh::parse_vcd(b, v, &err);
    if (!ok) { printf("ERR %s\n", err.c_str()); return 1; }
    printf("timescale %u %s\n", v.time_res, v.time_unit.c_str());
    for (auto &d : v.decl_bits) printf("decl %s %d\n", d.first.c_str(), d.second ? 1 : 0);
    for (size_t k = 0; k < v.names.size(); ++k) {
        if (v.index.at(v.names[k]) != k) { printf("ERR index\n"); return 1; }
        printf("%s", v.names[k].c_str());
        for (size_t j = 0; j < v.times[k].size(); ++j)
            printf(" %llu:%u", (unsigned long long)v.times[k][j], (unsigned)v.values[k][j]);
        printf("\n");
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def tools(libgls):
    from gls import hostbuild
    return hostbuild.build()


@pytest.fixture(scope="module")
def reader(libgls, tmp_path_factory):
    from gls.build import LIB_DIR, PKG, REPO
    d = tmp_path_factory.mktemp("stimrd")
    (d / "drv.cpp").write_text(DRIVER)
    exe = d / "drv"
    host = PKG / "host"
    r = subprocess.run(["g++", "-O1", "-std=c++17", f"-I{REPO / 'include'}", f"-I{host}", str(d / "drv.cpp"),
                        str(host / "vcd.cpp"), str(host / "stim_bin.cpp"), f"-L{LIB_DIR}", "-lgls",
                        f"-Wl,-rpath,{LIB_DIR}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def dump(reader, path):
    r = subprocess.run([str(reader), str(path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    return r.stdout


def convert(tools, vcd, out):
    r = subprocess.run([str(tools["gls_vcd2stim"]), str(vcd), str(out), "--host-vcd"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    return out.read_bytes()


@pytest.mark.parametrize("seed", range(4))
def test_converter_keeps_what_the_vcd_reader_reads(seed, tools, reader, tmp_path):
    from cases import standard_vcd
    (tmp_path / "s.vcd").write_text(standard_vcd(seed, n_scalar=10 + seed, n_bus=3 + seed))
    convert(tools, tmp_path / "s.vcd", tmp_path / "s.stim")
    a = dump(reader, tmp_path / "s.vcd")
    b = dump(reader, tmp_path / "s.stim")
    assert a == b
    assert any(line.startswith("decl ") and line.endswith(" 1") for line in b.splitlines()), "no bus bits"


@pytest.mark.parametrize("case", range(2))
def test_loaded_lists_match_reference_golden(case, tools, reader, tmp_path):
    from cases import standard_vcd
    from test_gpu_vcd import golden_vcd_cases, list_digests
    c = golden_vcd_cases()[case]
    (tmp_path / "s.vcd").write_text(standard_vcd(c["seed"], n_scalar=c["n_scalar"], n_bus=c["n_bus"],
                                                 n_times=c["n_times"]))
    convert(tools, tmp_path / "s.vcd", tmp_path / "s.stim")
    body = [line for line in dump(reader, tmp_path / "s.stim").splitlines()
            if not line.startswith(("timescale ", "decl "))]
    assert list_digests("\n".join(body) + "\n") == c["lists"]


def test_python_writer_matches_converter(tools, tmp_path):
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=400, cycles=50, depth=6)
    nl = synth.make_netlist(cfg, 5)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=6)
    files.write_vcd(tmp_path / "s.vcd", nl, st)
    files.write_stim_bin(tmp_path / "p.stim", nl, st)
    assert convert(tools, tmp_path / "s.vcd", tmp_path / "c.stim") == (tmp_path / "p.stim").read_bytes()
    res, unit, names, decls, start, t, v = files.read_stim_bin(tmp_path / "p.stim")
    assert (res, unit) == (1, "ps") and names == [nl.net_name(int(n)) for n in st.nets]
    assert decls == [(n, False) for n in names]
    assert np.array_equal(start, st.ev_start) and np.array_equal(t, st.time) and np.array_equal(v, st.value)


@pytest.mark.parametrize("damage", ["cut_header", "cut_index", "cut_values", "extra", "value", "order", "magic"])
def test_damaged_files_are_rejected(damage, tools, reader, tmp_path):
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=200, cycles=20, depth=4)
    nl = synth.make_netlist(cfg, 3)
    st = synth.make_stimulus(cfg, nl.ppi_nets, seed=4)
    files.write_stim_bin(tmp_path / "ok.stim", nl, st)
    b = bytearray((tmp_path / "ok.stim").read_bytes())
    total = int(st.ev_start[-1])
    first_two = int(np.argmax(np.diff(st.ev_start.astype(np.int64)) >= 2))   # a net with two changes or more
    t0 = len(b) - 9 * total   # the time array
    if damage == "cut_header":
        b = b[:30]
    elif damage == "cut_index":
        b = b[:t0 - 12]
    elif damage == "cut_values":
        b = b[:-5]
    elif damage == "extra":
        b += b"\0"
    elif damage == "value":
        b[-1] = 7
    elif damage == "order":
        a = int(st.ev_start[first_two])
        b[t0 + 8 * (a + 1): t0 + 8 * (a + 2)] = b[t0 + 8 * a: t0 + 8 * (a + 1)]
    else:
        b[7:8] = b"2"
    (tmp_path / "bad.stim").write_bytes(bytes(b))
    r = subprocess.run([str(reader), str(tmp_path / "bad.stim")], capture_output=True, text=True)
    if damage == "magic":   # no longer a binary file: read as a VCD, which it is not either
        assert r.returncode == 1
    else:
        assert r.returncode == 1 and r.stdout.startswith("ERR binary stimulus"), r.stdout
