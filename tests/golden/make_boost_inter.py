"""Hand-written inter.dat in the reference's format (a Boost text archive of
class `inter`, src/process.cpp:23-81) for a two-gate design, spelled out
token by token from the archive rules, independently of the C++ writer in
host/boost_inter.cpp.  `python tests/golden/make_boost_inter.py` rewrites
tests/golden/inter_small.dat; tests/test_boost_inter.py checks that the C++
reader reads it into EXPECTED_MODEL and that gls_process writes the same
bytes for SOURCES.

Archive rules used: header "22 serialization::archive 17"; a string is
"<length> <bytes>"; the first object of a class type is preceded by its
tracking flag and version ("0 0"); collections of arithmetic types have no
such prefix; a collection is "<count> 0 <items>"; a map item is a pair
(class) of key and value; a pointer is "<class number> [1 0 on first use]
<object number> <object>", class numbers counting class types in order of
first use from 0; floats and doubles in %.9e / %.17e.
"""
from __future__ import annotations

from pathlib import Path

SOURCES = {
    "small.vlib": """module GEN_INV_D1 (i, zn);
  input i;
  output zn;
  not (zn, i);
endmodule

module GEN_NAND2_D1 (a1, a2, zn);
  input a1, a2;
  output zn;
  nand (zn, a1, a2);
endmodule
""",
    "small.gv": """module top (a, y);
input a;
output y;
wire n1, k, z;
wire [1:0] bus;
assign k = 1'b1;
assign z = n1;
GEN_INV_D1 U1 ( .i(a), .zn(n1) );
GEN_NAND2_D1 U2 ( .a1(n1), .a2(k), .zn(y) );
endmodule
""",
    "small.sdf": """(DELAYFILE
 (TIMESCALE 1ps)
 (CELL (CELLTYPE "GEN_INV_D1") (INSTANCE U1)
  (DELAY (ABSOLUTE (IOPATH i zn (7:7:7) (9:9:9)))))
 (CELL (CELLTYPE "GEN_NAND2_D1") (INSTANCE U2)
  (DELAY (ABSOLUTE (IOPATH a1 zn (11:11:11) (13:13:13)) (IOPATH a2 zn (15:15:15) (17:17:17)))))
)
""",
}

# the simulation model the C++ reader must build (tests/test_boost_inter.py
# prints it the same way): U1 = not(a) -> n1, U2 = nand(n1, k) -> y with k
# tied to 1, z an alias of n1, bus[1:0] declared and undriven
EXPECTED_MODEL = """top top
level 0
inst U1 in a out n1 prog 7:0,1, arc 2 a n1 7 9
level 1
inst U2 in n1 k out y prog 5:0,1,2, arc 2 n1 y 11 13 arc 2 k y 15 17
const k 3
alias z n1
busbit bus[1]
busbit bus[0]
"""

CI = "0 0"            # class information of a class type's first object


def s(x: str) -> str:
    return f"{len(x)} {x}"


def coll(n: int) -> str:
    return f"{n} 0"   # count and item version


def pin(ptype, name, size=1, l=-1, r=-1, first=False):
    return " ".join(([CI] if first else []) + [s(ptype), s(name), str(size), str(l), str(r)])


def inv_module(first):
    # ModuleType GEN_INV_D1: name, ports, in_out_ports, supply1, supply0, function
    t = [CI] if first else []
    t += [s("GEN_INV_D1")]
    t += ([CI] if first else []) + [coll(2)]                       # map<string, Pin>
    t += ([CI] if first else []) + [s("i"), pin("input", "i", first=first)]   # pair<string, Pin>, Pin
    t += [s("zn"), pin("output", "zn")]
    t += ([CI] if first else []) + [coll(2), s("i"), s("zn")]     # in_out_ports: vector<string>
    t += [coll(0), coll(0)]                                        # supply1_vec, supply0_vec
    t += ([CI] if first else []) + [coll(1)]                       # vector<Function>
    t += ([CI] if first else []) + [s("not"), "7", coll(1), s("i")]   # Function: name, id, input_pins
    t += ([CI] if first else []) + [coll(0)]                       # input_data: vector<VCDBit>
    t += [coll(1), s("zn"), "0"]                                   # output_pins, output_data
    return t


def nand_module():
    t = [s("GEN_NAND2_D1"), coll(3)]
    t += [s("a1"), pin("input", "a1"), s("a2"), pin("input", "a2"), s("zn"), pin("output", "zn")]
    t += [coll(3), s("a1"), s("a2"), s("zn"), coll(0), coll(0)]
    t += [coll(1), s("nand"), "5", coll(2), s("a1"), s("a2"), coll(0), coll(1), s("zn"), "0"]
    return t


def archive() -> str:
    t = ["22 serialization::archive 17"]
    t += [CI]                                  # inter
    t += [CI]                                  # PreProcess
    # module_types: map<string, ModuleType>, sorted by name
    t += [CI, coll(2)]
    t += [CI, s("GEN_INV_D1")] + inv_module(first=True)          # pair<string, ModuleType> + value
    t += [s("GEN_NAND2_D1")] + nand_module()
    t += [coll(0)]                             # ignored_modules
    t += [s("top")]                            # top_module_name
    # instances: map<string, Instance>
    t += [CI, coll(2), CI, s("U1"), CI]        # map, pair<string, Instance>, Instance
    t += inv_module(first=False) + [s("U1")]   # type, name
    t += [CI, coll(1), CI, s("i"), s("a")]     # in_port_net: map<string, string>, pair<string, string>
    t += [coll(1), s("a")]                     # in_net
    t += [coll(1), s("zn"), s("n1")]           # out_port_net
    t += [coll(1), s("n1"), coll(0), coll(0)]  # out_net, unknown_in, unknown_out
    t += [coll(1), s("not"), "7", coll(1), s("a"), coll(0), coll(1), s("n1"), "0"]   # function_vec
    t += [CI, coll(1), coll(3), "7 0 1"]       # function_id_vec: vector<vector<int>>; vector<int> has no prefix
    t += [CI, coll(1), CI, "2", s("a"), s("n1"), "7.00000000000000000e+00", "9.00000000000000000e+00"]  # delays
    t += [coll(1), "-1", coll(1), s("a"), coll(1), "-1", coll(1), "0", coll(1), "0"]   # in_net_from_*
    t += [s("U2")] + nand_module() + [s("U2")]
    t += [coll(2), s("a1"), s("n1"), s("a2"), s("k")]
    t += [coll(2), s("n1"), s("k")]
    t += [coll(1), s("zn"), s("y")]
    t += [coll(1), s("y"), coll(0), coll(0)]
    t += [coll(1), s("nand"), "5", coll(2), s("n1"), s("k"), coll(0), coll(1), s("y"), "0"]
    t += [coll(1), coll(4), "5 0 1 2"]
    t += [coll(2), "2", s("n1"), s("y"), "1.10000000000000000e+01", "1.30000000000000000e+01",
          "2", s("k"), s("y"), "1.50000000000000000e+01", "1.70000000000000000e+01"]
    t += [coll(2), "0 -2", coll(2), s("U1"), s("k"), coll(2), "0 -2", coll(2), "0 3", coll(2), "0 0"]
    t += [coll(2), s("U1"), s("U2")]           # instance_name_vec
    # net_instance_map: map<string, vector<int>>
    t += [CI, coll(3), CI, s("a"), coll(1), "0", s("k"), coll(1), "1", s("n1"), coll(1), "1"]
    # out_net_from_id: map<string, int>
    t += [CI, coll(2), CI, s("n1"), "0", s("y"), "1"]
    # pins: map<string, Pin> (class known)
    t += [coll(6), s("a"), pin("input", "a"), s("bus"), pin("wire", "bus", 2, 1, 0), s("k"), pin("wire", "k"),
          s("n1"), pin("wire", "n1"), s("y"), pin("output", "y"), s("z"), pin("wire", "z")]
    t += [coll(7), s("a"), s("y"), s("n1"), s("k"), s("z"), s("bus[1]"), s("bus[0]")]   # pin_bits
    # pinbitValues: map<string, TimedValues*>; the pointer's class is the
    # 28th class type used (number 27), tracked: "27 1 0", object 0
    t += [CI, coll(1), CI, s("k"), "27 1 0 0", coll(1), CI, "0 3"]
    t += [coll(1), s("z"), s("n1")]            # assign_pairs
    t += [CI, coll(1), CI, s("k"), coll(3), "0 1 0"]   # Result: map<string, vector<u64>>
    t += [coll(2), coll(1), "0", coll(1), "1"]          # levels
    t += [coll(0)]                                      # initial_net_map (empty in the reference)
    t += [coll(2), "0 1", coll(2), "0 1"]               # data_in_num_start, data_out_num_start
    t += [coll(2), "0 1", coll(2), "1 2"]               # delay_start, delay_width
    t += [coll(2), "0 3", coll(2), "3 4"]               # functions_start, functions_width
    t += [coll(2), "1 2", coll(2), "1 1"]               # data_in_num, data_out_num
    t += [coll(2), "0 0", coll(2), "1 2"]               # val_num_start, delay_val_num
    t += [coll(2), "1 1", coll(2), "3 4"]               # functions_func_num, functions_val_num
    t += [coll(3), "2 2 2", coll(3), "0 0 1", coll(3), "0 0 0"]   # host_delay_edges, host_in_bit, host_out_bit
    t += [coll(3), "7.000000000e+00 1.100000000e+01 1.500000000e+01"]   # host_rise_val
    t += [coll(3), "9.000000000e+00 1.300000000e+01 1.700000000e+01"]   # host_fall_val
    t += [coll(7), "7 0 1 5 0 1 2"]                     # host_functions
    # OutMaps: vector<map<string, vector<unsigned>>>
    t += [CI, coll(2), CI, coll(1), CI, s("n1"), coll(2), "0 0", coll(1), s("y"), coll(2), "0 0"]
    return " ".join(t) + "\n"


if __name__ == "__main__":
    out = Path(__file__).resolve().parent / "inter_small.dat"
    out.write_text(archive())
    print(out)
