"""The reference's inter.dat format (a Boost text archive of class `inter`,
src/process.cpp:23-81) in the command-line tools, on the CPU:

* gls_process writes it by default; reading it back gives the same
  simulation model as the tools' native format;
* loading an archive and saving it again reproduces it byte for byte;
* the hand-written archive in tests/golden (made token by token by
  tests/golden/make_boost_inter.py, independently of the C++ writer) reads
  into the expected design, and the C++ writer, given that design, writes
  exactly those bytes;
* damaged archives are rejected with a message.

Agreement with archives written by a real Boost build is not checked here:
Boost is not installed."""
import subprocess
from pathlib import Path

import pytest

from gls import files, synth

GOLD = Path(__file__).resolve().parent / "golden"

DRIVER = r"""
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include "boost_inter.h"
#include "design.h"
using namespace glsh;
static std::string slurp(const char *p)
{
    std::ifstream f(p, std::ios::binary);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}
int main(int argc, char **argv)
{
    std::string err;
    if (!strcmp(argv[1], "resave")) {   // archive -> ref::Inter -> archive
        ref::Inter in;
        if (!load_boost_inter(slurp(argv[2]), in, &err)) { printf("ERR %s\n", err.c_str()); return 1; }
        const std::string t = save_boost_inter(in);
        fwrite(t.data(), 1, t.size(), stdout);
        return 0;
    }
    if (!strcmp(argv[1], "design")) {   // either format -> the simulation model, as text
        Design d;
        if (!read_inter(argv[2], d, &err)) { printf("ERR %s\n", err.c_str()); return 1; }
        printf("top %s\n", d.top.c_str());
        for (size_t L = 0; L + 1 < d.level_start.size(); ++L) {
            printf("level %zu\n", L);
            for (uint32_t k = d.level_start[L]; k < d.level_start[L + 1]; ++k) {
                const Instance &in = d.insts[k];
                const Cell &c = d.cells[in.cell];
                printf("inst %s in", in.name.c_str());
                for (size_t p = 0; p < c.inputs.size(); ++p) printf(" %s", d.net_names[in.pins[p]].c_str());
                printf(" out");
                for (size_t p = c.inputs.size(); p < in.pins.size(); ++p) printf(" %s", d.net_names[in.pins[p]].c_str());
                printf(" prog");
                for (auto &pr : c.prims) {
                    printf(" %u:", pr.func);
                    for (auto q : pr.pins) printf("%u,", q);
                }
                for (auto &a : in.arcs)
                    printf(" arc %u %s %s %.6g %.6g", a.edge, d.net_names[in.pins[a.in_pin]].c_str(),
                           d.net_names[in.pins[c.inputs.size() + a.out_pin]].c_str(), a.rise, a.fall);
                printf("\n");
            }
        }
        for (auto &c : d.constants) printf("const %s %u\n", d.net_names[c.first].c_str(), c.second);
        for (auto &a : d.aliases) printf("alias %s %s\n", d.net_names[a.first].c_str(), d.net_names[a.second].c_str());
        for (auto b : d.bus_bits) printf("busbit %s\n", d.net_names[b].c_str());
        return 0;
    }
    return 2;
}
"""


@pytest.fixture(scope="module")
def tools(libgls):
    from gls import hostbuild
    return hostbuild.build()


@pytest.fixture(scope="module")
def driver(tools, tmp_path_factory):
    from gls.build import PKG, REPO
    d = tmp_path_factory.mktemp("boostdrv")
    (d / "drv.cpp").write_text(DRIVER)
    exe = d / "drv"
    host = PKG / "host"
    r = subprocess.run(["g++", "-std=c++17", "-O1", f"-I{REPO / 'include'}", f"-I{host}", str(d / "drv.cpp"),
                        str(host / "boost_inter.cpp"), str(host / "design.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run(exe, *args):
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True)
    assert r.returncode == 0, r.stdout.decode(errors="replace")
    return r.stdout


@pytest.fixture(scope="module")
def design(tmp_path_factory, tools):
    d = tmp_path_factory.mktemp("boost")
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=300, cycles=20, depth=8)
    nl = synth.make_netlist(cfg, 17)
    files.write_vlib(d / "lib.vlib")
    files.write_gv(d / "d.gv", nl)
    files.write_sdf(d / "d.sdf", nl)
    for extra, out in (([], "boost.dat"), (["--native"], "native.dat")):
        r = subprocess.run([str(tools["gls_process"]), *extra, str(d / "lib.vlib"), str(d / "d.gv"),
                            str(d / "d.sdf"), str(d / out)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
    return d


def test_process_writes_the_reference_archive_by_default(design):
    text = (design / "boost.dat").read_bytes()
    assert text.startswith(b"22 serialization::archive 17 0 0 0 0 0 0 ")
    assert (design / "native.dat").read_bytes().startswith(b"GLSINTR1")


def test_archive_and_native_give_the_same_model(design, driver):
    """The same instances, programs, arcs, aliases and bus bits; the native
    file also lists the two tie-off constants whether or not a pin uses them
    (the archive keeps only the used ones, as the reference does)."""
    a = run(driver, "design", design / "boost.dat").decode().splitlines()
    b = run(driver, "design", design / "native.dat").decode().splitlines()
    unused = [x for x in ("const 1'b0 0", "const 1'b1 3") if not any(f" {x.split()[1]} " in f" {y} " for y in a
                                                                      if y.startswith("inst "))]
    assert a == [x for x in b if x not in unused]


def test_archive_resaves_byte_for_byte(design, driver):
    a = (design / "boost.dat").read_bytes()
    assert run(driver, "resave", design / "boost.dat") == a


def test_hand_written_archive(driver, tmp_path):
    """The hand-written archive reads into the design it spells out, and the
    C++ writer (gls_process on the same library, netlist and SDF) writes
    the same bytes."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_boost_inter", GOLD / "make_boost_inter.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    arch = GOLD / "inter_small.dat"
    assert arch.read_text() == mk.archive(), "tests/golden/inter_small.dat is stale: rerun make_boost_inter.py"
    model = run(driver, "design", arch).decode()
    assert model == mk.EXPECTED_MODEL
    for name, text in mk.SOURCES.items():
        (tmp_path / name).write_text(text)
    from gls import hostbuild
    exe = hostbuild.build()["gls_process"]
    r = subprocess.run([str(exe), str(tmp_path / "small.vlib"), str(tmp_path / "small.gv"),
                        str(tmp_path / "small.sdf"), str(tmp_path / "w.dat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert (tmp_path / "w.dat").read_text() == arch.read_text()


@pytest.mark.parametrize("cut", [10, 200, -40, -3])
def test_damaged_archives_are_rejected(design, driver, tmp_path, cut):
    a = (design / "boost.dat").read_bytes()
    (tmp_path / "bad.dat").write_bytes(a[:cut])
    r = subprocess.run([str(driver), "design", str(tmp_path / "bad.dat")], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.startswith("ERR ")


def test_wrong_signature_is_rejected(driver, tmp_path):
    (tmp_path / "x.dat").write_text("22 serialization::archivX 17 0 0\n")
    r = subprocess.run([str(driver), "design", str(tmp_path / "x.dat")], capture_output=True, text=True)
    assert r.returncode == 1 and "ERR" in r.stdout


def test_archive_keeps_buses_aliases_constants_and_open_outputs(driver, tools, tmp_path):
    """A netlist with bus ports, assign aliases, tie-offs and an output left
    open (its SDF arc names the port, as the reference records it): the
    archive and the native file give the same model."""
    from test_gpu_cli import GV, SDF
    files.write_vlib(tmp_path / "lib.vlib")
    (tmp_path / "d.gv").write_text(GV)
    (tmp_path / "d.sdf").write_text(SDF)
    for extra, out in (([], "a.dat"), (["--native"], "n.dat")):
        r = subprocess.run([str(tools["gls_process"]), *extra, str(tmp_path / "lib.vlib"), str(tmp_path / "d.gv"),
                            str(tmp_path / "d.sdf"), str(tmp_path / out)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
    a = run(driver, "design", tmp_path / "a.dat").decode().splitlines()
    b = run(driver, "design", tmp_path / "n.dat").decode().splitlines()
    assert any(x.startswith("inst U5 ") and " arc " in x for x in a), "the open output's arc was lost"
    unused = [x for x in ("const 1'b0 0", "const 1'b1 3") if not any(f" {x.split()[1]} " in f" {y} " for y in a
                                                                      if y.startswith("inst "))]
    assert a == [x for x in b if x not in unused]
