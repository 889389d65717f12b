"""GPU tests of the command-line drop-in: gls_process + gls_simulate over
files, SAIF records compared with the oracle run on the same design."""
import subprocess

import numpy as np
import pytest

from cases import stimulus
from gls import files, synth
from oracle.runner import run_oracle

pytestmark = pytest.mark.gpu
U64 = 2**64 - 1


@pytest.fixture(scope="module")
def tools(libgls):
    from gls import hostbuild
    return hostbuild.build()


def run_cli(tools, d, t_begin, t_end, extra=()):
    """gls_process (native inter.dat, which oracle_records reads in Python),
    then gls_simulate."""
    r = subprocess.run([str(tools["gls_process"]), "--native", str(d / "lib.vlib"), str(d / "d.gv"),
                        str(d / "d.sdf"), str(d / "inter.dat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    r = subprocess.run([str(tools["gls_simulate"]), str(d / "inter.dat"), str(d / "d.vcd"), str(t_begin),
                        str(t_end), str(d / "out.saif"), *extra], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return (d / "out.saif").read_text()


def oracle_records(d, stim_of, t_begin, t_end):
    """SAIF records the reference semantics give, by net name."""
    it = files.read_inter(d / "inter.dat")
    nl = files.netlist_from_inter(it)
    consts = nl.extra["constants"]
    st = {}
    for n in nl.ppi_nets.tolist():
        name = it["nets"][n]
        if name in stim_of:
            st[n] = stim_of[name]
        elif n in consts:
            st[n] = [(0, consts[n])]
        else:
            raise AssertionError(f"no waveform for {name}")
    for name, ev in stim_of.items():   # VCD nets no gate reads are reported too
        n = it["nets"].index(name) if name in it["nets"] else None
        if n is not None and n not in st:
            st[n] = ev
    _, saif, _ = run_oracle(nl, stimulus(st), t_begin, t_end)
    return it, nl, saif


def test_cli_end_to_end_matches_oracle(tools, tmp_path):
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=800, cycles=200, depth=10)
    nl0 = synth.make_netlist(cfg, 9)
    st0 = synth.make_stimulus(cfg, nl0.ppi_nets, 10)
    files.write_vlib(tmp_path / "lib.vlib")
    files.write_gv(tmp_path / "d.gv", nl0)
    files.write_sdf(tmp_path / "d.sdf", nl0)
    files.write_vcd(tmp_path / "d.vcd", nl0, st0)
    t_begin, t_end = 5_000, cfg.t_end - 3_000
    recs = files.parse_saif(run_cli(tools, tmp_path, t_begin, t_end))
    stim_of = {nl0.net_name(int(n)): list(zip(*[x.tolist() for x in st0.events_of(k)]))
               for k, n in enumerate(st0.nets)}
    it, nl, saif = oracle_records(tmp_path, stim_of, t_begin, t_end)
    checked = 0
    for n, name in enumerate(it["nets"]):
        if saif[n][0] == U64 or name.startswith("1'b"):
            continue
        assert recs[name] == tuple(int(x) for x in saif[n]), name
        checked += 1
    assert checked == nl.n_inst + len(st0.nets)
    text = (tmp_path / "out.saif").read_text()
    assert text.startswith(f"(TIMESCALE 1 ps)\n(DURATION {t_end - t_begin})\n(INSTANCE root\n   (NET\n")


GV = """module t (clk, a, b, sel);
input clk;
input [3:0] a;
input b, sel;
wire [1:0] w;
wire x, y, z, k0;
output [1:0] o;
assign k0 = 1'b1;
assign y = x;
GEN_AND2_D1 U0 ( .a1(a[0]), .a2(a[1]), .z(x) );
GEN_NOR2_D1 U1 ( .a1(y), .a2(b), .zn(w[0]) );
GEN_MUX2_D1 U2 ( .i0(w[0]), .i1(a[3]), .s(sel), .z(w[1]) );
GEN_NAND2_D1 U3 ( .a1(k0), .a2(w[1]), .zn(o[0]) );
GEN_XOR2_D1 U4 ( .a1(1'b0), .a2(a[2]), .z(z) );
GEN_INV_D1 U5 ( .i(z) );
endmodule
"""

SDF = """(DELAYFILE (TIMESCALE 1ps)
 (CELL (CELLTYPE "GEN_AND2_D1") (INSTANCE U0) (DELAY (ABSOLUTE (IOPATH a1 z (11:11:11) (13:13:13)) (IOPATH a2 z (17:17:17) (19:19:19)))))
 (CELL (CELLTYPE "GEN_NOR2_D1") (INSTANCE U1) (DELAY (ABSOLUTE (IOPATH a1 zn (5:5:5) (7:7:7)) (IOPATH a2 zn (9:9:9) (12:12:12)))))
 (CELL (CELLTYPE "GEN_MUX2_D1") (INSTANCE U2) (DELAY (ABSOLUTE (IOPATH i0 z (20:20:20) (21:21:21)) (IOPATH i1 z (22:22:22) (23:23:23))
    (IOPATH (posedge s) z (30:30:30) (31:31:31)) (IOPATH (negedge s) z (32:32:32) (33:33:33)))))
 (CELL (CELLTYPE "GEN_NAND2_D1") (INSTANCE U3) (DELAY (ABSOLUTE (IOPATH a1 zn (8:8:8) (9:9:9)) (IOPATH a2 zn (10:10:10) (14:14:14)))))
 (CELL (CELLTYPE "GEN_XOR2_D1") (INSTANCE U4) (DELAY (ABSOLUTE (IOPATH (posedge a1) z (4:4:4) (5:5:5)) (IOPATH (negedge a1) z (6:6:6) (7:7:7))
    (IOPATH (posedge a2) z (8:8:8) (9:9:9)) (IOPATH (negedge a2) z (10:10:10) (11:11:11)))))
 (CELL (CELLTYPE "GEN_INV_D1") (INSTANCE U5) (DELAY (ABSOLUTE (IOPATH i zn (3:3:3) (4:4:4)))))
)
"""

VCD = """$timescale 1ps $end
$scope module t $end
$var wire 4 ! a [3:0] $end
$var wire 1 " b $end
$var wire 1 # sel $end
$var wire 1 $ clk $end
$upscope $end
$enddefinitions $end
#0
$dumpvars
b0000 !
0"
x#
0$
$end
#100
b0011 !
1#
#130
b11 !
#150
b1z11 !
1"
#400
0"
b0 !
#420
1"
#425
0"
#600
b1111 !
0#
#700
bx10x !
#900
b1011 !
1#
"""


def test_cli_buses_aliases_constants(tools, tmp_path):
    files.write_vlib(tmp_path / "lib.vlib")
    (tmp_path / "d.gv").write_text(GV)
    (tmp_path / "d.sdf").write_text(SDF)
    (tmp_path / "d.vcd").write_text(VCD)
    recs = files.parse_saif(run_cli(tools, tmp_path, 50, 1000))
    # the VCD as the reference's parser reads it: bus bits keep only changes,
    # starting from Z; scalars keep every change
    bus = {0: "0000", 100: "0011", 130: "0011", 150: "1z11", 400: "0000", 600: "1111", 700: "x10x", 900: "1011"}
    code = {"0": 0, "1": 3, "x": 1, "z": 2}
    stim_of = {}
    for bit in range(4):
        ev, last = [], 2
        for t, s in bus.items():
            v = code[s[3 - bit]]
            if v != last:
                ev.append((t, v))
                last = v
        stim_of[f"a[{bit}]"] = ev
    stim_of["b"] = [(0, 0), (150, 3), (400, 0), (420, 3), (425, 0)]
    stim_of["sel"] = [(0, 1), (100, 3), (600, 0), (900, 3)]
    stim_of["clk"] = [(0, 0)]
    it, nl, saif = oracle_records(tmp_path, stim_of, 50, 1000)
    nid = {name: n for n, name in enumerate(it["nets"])}
    for name in ["a[0]", "a[3]", "b", "sel", "x", "w[0]", "w[1]", "o[0]", "z", "k0", "clk"]:
        assert recs[name] == tuple(int(v) for v in saif[nid[name]]), name
    assert recs["y"] == recs["x"]                  # assign alias reports its source
    assert recs["o[1]"] == (0, 0, 950)             # declared, never driven: all X
    assert recs["k0"] == (0, 950, 0)               # constant 1
    assert recs["U5[zn]"] == tuple(int(v) for v in saif[nid["U5[zn]"]])   # unconnected output


def simulate(tools, inter, vcd, t_begin, t_end, out, extra=()):
    r = subprocess.run([str(tools["gls_simulate"]), str(inter), str(vcd), str(t_begin), str(t_end), str(out),
                        *extra], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out.read_text()


def record_names(text):
    """NET record names of a flat SAIF file, in file order."""
    import re
    lines = text.splitlines()
    return [lines[k - 1].strip()[1:] for k, x in enumerate(lines) if re.match(r"\s*\(T0 \d+\)", x)]


def test_cli_reference_archive_and_saif_order(tools, tmp_path):
    """The reference's inter.dat (gls_process's default Boost text archive)
    simulates to the same SAIF as the native file; --saif-order=ref writes
    every record once, in the reference GPU tool's order and coverage (no
    nested instance records, the file ends after the NET list)."""
    files.write_vlib(tmp_path / "lib.vlib")
    (tmp_path / "d.gv").write_text(GV)
    (tmp_path / "d.sdf").write_text(SDF)
    (tmp_path / "d.vcd").write_text(VCD)
    for extra, name in (([], "a.dat"), (["--native"], "n.dat")):
        r = subprocess.run([str(tools["gls_process"]), *extra, str(tmp_path / "lib.vlib"), str(tmp_path / "d.gv"),
                            str(tmp_path / "d.sdf"), str(tmp_path / name)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
    assert (tmp_path / "a.dat").read_text().startswith("22 serialization::archive ")
    a = simulate(tools, tmp_path / "a.dat", tmp_path / "d.vcd", 50, 1000, tmp_path / "a.saif")
    n = simulate(tools, tmp_path / "n.dat", tmp_path / "d.vcd", 50, 1000, tmp_path / "n.saif")
    assert files.parse_saif(a) == files.parse_saif(n)
    r = simulate(tools, tmp_path / "a.dat", tmp_path / "d.vcd", 50, 1000, tmp_path / "r.saif", ["--saif-order=ref"])
    names = record_names(r)
    assert len(names) == len(set(names)), "a record printed twice"
    ref = files.parse_saif(r)
    flat = {k: v for k, v in files.parse_saif(a).items() if k != "U5[zn]"}   # the open output has no ref record
    assert ref == flat
    assert r.endswith("   )\n") and "INSTANCE U5" not in r
    # the reference order: nets as levels first read them, then constants,
    # unread gate outputs, unread VCD signals, aliases, undriven bus bits
    assert names.index("k0") > max(names.index(x) for x in ("a[0]", "a[1]", "w[1]"))
    assert names[-1] == "o[1]"
    # the same order from the native file
    r2 = simulate(tools, tmp_path / "n.dat", tmp_path / "d.vcd", 50, 1000, tmp_path / "r2.saif", ["--saif-order=ref"])
    assert record_names(r2) == names


def test_cli_hand_written_archive_matches_oracle(tools, tmp_path):
    """tests/golden/inter_small.dat (the reference's format, written by hand)
    simulates to oracle-identical SAIF: U1 = not(a) -> n1, U2 = nand(n1, k)
    -> y with k tied to 1, z an alias of n1, bus[1:0] undriven."""
    from pathlib import Path

    from gls.levelize import assemble
    gold = Path(__file__).resolve().parent / "golden" / "inter_small.dat"
    (tmp_path / "s.vcd").write_text("$timescale 1ps $end\n$scope module top $end\n$var wire 1 ! a $end\n"
                                    "$upscope $end\n$enddefinitions $end\n#0\n0!\n#100\n1!\n#104\n0!\n"
                                    "#300\n1!\n#700\nx!\n#800\n0!\n")
    text = simulate(tools, gold, tmp_path / "s.vcd", 0, 1000, tmp_path / "s.saif")
    recs = files.parse_saif(text)
    # the oracle on the same design: nets a=0, k=1, n1=2, y=3
    nl = assemble([("GEN_INV_D1", [0], [2], [(2, "i", "zn", 7, 9)]),
                   ("GEN_NAND2_D1", [2, 1], [3], [(2, "a1", "zn", 11, 13), (2, "a2", "zn", 15, 17)])], n_nets=4)
    st = stimulus({0: [(0, 0), (100, 3), (104, 0), (300, 3), (700, 1), (800, 0)], 1: [(0, 3)]})
    ow, osaif, _ = run_oracle(nl, st, 0, 1000)
    for name, n in (("a", 0), ("n1", 2), ("y", 3)):
        assert recs[name] == tuple(int(x) for x in osaif[n]), name
    assert recs["k"] == (0, 1000, 0)
    assert recs["z"] == recs["n1"]
    assert recs["bus[1]"] == recs["bus[0]"] == (0, 0, 1000)
    assert set(recs) == {"a", "n1", "y", "k", "z", "bus[1]", "bus[0]"}


def test_cli_binary_stimulus_gives_the_same_saif(tools, tmp_path):
    """gls_simulate on the binary stimulus that gls_vcd2stim writes (its
    GPU scan, and the host reader) and on the one gls.files.write_stim_bin
    writes: the same SAIF file as on the VCD, with and without the
    reference order; buses, aliases and constants included."""
    from gls import hostbuild
    tools = hostbuild.build()
    files.write_vlib(tmp_path / "lib.vlib")
    (tmp_path / "d.gv").write_text(GV)
    (tmp_path / "d.sdf").write_text(SDF)
    (tmp_path / "d.vcd").write_text(VCD)
    r = subprocess.run([str(tools["gls_process"]), str(tmp_path / "lib.vlib"), str(tmp_path / "d.gv"),
                        str(tmp_path / "d.sdf"), str(tmp_path / "a.dat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    for extra, name in (([], "g.stim"), (["--host-vcd"], "h.stim")):
        r = subprocess.run([str(tools["gls_vcd2stim"]), str(tmp_path / "d.vcd"), str(tmp_path / name), *extra],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
    assert (tmp_path / "g.stim").read_bytes() == (tmp_path / "h.stim").read_bytes()
    for order in ([], ["--saif-order=ref"]):
        v = simulate(tools, tmp_path / "a.dat", tmp_path / "d.vcd", 50, 1000, tmp_path / "v.saif", order)
        b = simulate(tools, tmp_path / "a.dat", tmp_path / "g.stim", 50, 1000, tmp_path / "b.saif", order)
        assert v == b
    # a generated design: the Python writer's file against the VCD
    cfg = synth.scaled(synth.CONFIGS["c1"], cells=800, cycles=200, depth=10)
    nl0 = synth.make_netlist(cfg, 9)
    st0 = synth.make_stimulus(cfg, nl0.ppi_nets, 10)
    files.write_gv(tmp_path / "e.gv", nl0)
    files.write_sdf(tmp_path / "e.sdf", nl0)
    files.write_vcd(tmp_path / "e.vcd", nl0, st0)
    files.write_stim_bin(tmp_path / "e.stim", nl0, st0)
    r = subprocess.run([str(tools["gls_process"]), str(tmp_path / "lib.vlib"), str(tmp_path / "e.gv"),
                        str(tmp_path / "e.sdf"), str(tmp_path / "e.dat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    v = simulate(tools, tmp_path / "e.dat", tmp_path / "e.vcd", 5_000, cfg.t_end, tmp_path / "ev.saif")
    b = simulate(tools, tmp_path / "e.dat", tmp_path / "e.stim", 5_000, cfg.t_end, tmp_path / "eb.saif")
    assert v == b
