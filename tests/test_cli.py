"""CPU tests of the command-line front end (gls_process): Verilog library,
netlist and SDF parsing, levelization, and the inter.dat file."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from gls import files, synth
from gls.build import BIN_DIR
from gls.cells import LIBRARY
from oracle.build import REFERENCE

# the reference checkout's cell library (GLS_REFERENCE names the checkout)
REF_VLIB = REFERENCE / "examples" / "GENERIC_STD_CELL.vlib"


@pytest.fixture(scope="module")
def tools(libgls):
    from gls import hostbuild
    return hostbuild.build()


@pytest.fixture(scope="module")
def design(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=400, cycles=40, depth=8)
    nl = synth.make_netlist(cfg, 5)
    files.write_vlib(d / "lib.vlib")
    files.write_gv(d / "d.gv", nl)
    files.write_sdf(d / "d.sdf", nl)
    return d, nl


def process(tools, d, vlib, out="inter.dat"):
    """gls_process writing the native inter.dat, which these tests read in Python."""
    r = subprocess.run([str(tools["gls_process"]), "--native", str(vlib), str(d / "d.gv"), str(d / "d.sdf"),
                        str(d / out)], capture_output=True, text=True)
    return r


def test_process_rebuilds_the_levelized_netlist(tools, design):
    d, nl = design
    r = process(tools, d, d / "lib.vlib")
    assert r.returncode == 0, r.stdout
    it = files.read_inter(d / "inter.dat")
    assert it["level_start"] == [int(x) for x in nl.level_start]
    by_name = {x[0]: x for x in it["insts"]}
    for i in range(nl.n_inst):
        name, cell, pins, arcs = by_name[nl.inst_name(i)]
        c = nl.cells[int(nl.inst_cell[i])]
        assert it["cells"][cell][0] == c.name
        assert [it["nets"][p] for p in pins] == [nl.net_name(int(n)) for n in
                                                 list(nl.inputs_of(i)) + list(nl.outputs_of(i))]
        exp = [(int(a["edge"]), int(a["in_pin"]), int(a["out_pin"]), float(a["rise"]), float(a["fall"]))
               for a in nl.arcs[int(nl.arc_start[i]): int(nl.arc_start[i + 1])]]
        assert arcs == exp, name
    # the instances of each level are the netlist's, in the same order
    names = [x[0] for x in it["insts"]]
    assert names == [nl.inst_name(i) for i in range(nl.n_inst)]
    for name, ins, outs, prims in it["cells"]:
        c = LIBRARY[name]
        assert ins == c.inputs and outs == c.outputs
        assert [(f, list(p)) for f, p in prims] == c.program()


@pytest.mark.skipif(not REF_VLIB.exists(), reason="reference library not on this machine")
def test_reference_cell_library_gives_the_same_inter_dat(tools, design):
    d, _ = design
    assert process(tools, d, d / "lib.vlib", "a.dat").returncode == 0
    r = process(tools, d, REF_VLIB, "b.dat")
    assert r.returncode == 0 and "200 modules, 72 skipped" in r.stdout
    assert (d / "a.dat").read_bytes() == (d / "b.dat").read_bytes()


def test_process_rejects_a_combinational_loop(tools, tmp_path):
    files.write_vlib(tmp_path / "lib.vlib")
    (tmp_path / "d.gv").write_text("module t (a);\ninput a;\nwire x, y;\n"
                                   "GEN_AND2_D1 U0 ( .a1(a), .a2(y), .z(x) );\n"
                                   "GEN_INV_D1 U1 ( .i(x), .zn(y) );\nendmodule\n")
    (tmp_path / "d.sdf").write_text("(DELAYFILE (TIMESCALE 1ps))\n")
    r = subprocess.run([str(tools["gls_process"]), str(tmp_path / "lib.vlib"), str(tmp_path / "d.gv"),
                        str(tmp_path / "d.sdf"), str(tmp_path / "x.dat")], capture_output=True, text=True)
    assert r.returncode == 255 and "loop" in r.stdout


def test_process_usage_and_missing_files(tools, tmp_path):
    r = subprocess.run([str(tools["gls_process"])], capture_output=True, text=True)
    assert r.returncode == 255 and "USAGE" in r.stdout
    r = subprocess.run([str(tools["gls_process"]), "/nonexistent.vlib", "a", "b", str(tmp_path / "x")],
                       capture_output=True, text=True)
    assert r.returncode == 255


def test_sdf_timescale_and_edges(tools, tmp_path):
    files.write_vlib(tmp_path / "lib.vlib")
    (tmp_path / "d.gv").write_text("module t (a, b);\ninput a, b;\nwire z;\n"
                                   "GEN_XOR2_D1 U0 ( .a1(a), .a2(b), .z(z) );\nendmodule\n")
    (tmp_path / "d.sdf").write_text(
        '(DELAYFILE (TIMESCALE 1ns)\n (CELL (CELLTYPE "GEN_XOR2_D1") (INSTANCE U0)\n'
        '  (DELAY (ABSOLUTE (IOPATH (posedge a1) z (0.01:0.02:0.03) (0.04:0.05:0.06))\n'
        '   (IOPATH (negedge a1) z (0.007::0.009) (0.008))\n   (IOPATH a2 z (0.1:0.1:0.1))))))\n')
    r = subprocess.run([str(tools["gls_process"]), "--native", str(tmp_path / "lib.vlib"), str(tmp_path / "d.gv"),
                        str(tmp_path / "d.sdf"), str(tmp_path / "x.dat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    arcs = files.read_inter(tmp_path / "x.dat")["insts"][0][3]
    assert [a[:3] for a in arcs] == [(0, 0, 0), (1, 0, 0), (2, 1, 0)]
    # the second non-empty field (typ; max when typ is empty), ns -> ps; one value: fall = rise
    assert np.allclose([a[3:] for a in arcs], [(20, 50), (9, 8), (100, 100)])
