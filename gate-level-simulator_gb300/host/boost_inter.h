// inter.dat as the reference writes it: a Boost.Serialization text archive
// of class `inter` (src/process.cpp:23-81, written at :604-608 and read by
// the GPU tool at src/simulate.cu:1835-1844).
//
// The structs in namespace ref mirror the reference's archived types member
// for member, in their serialize() order, because the archive is nothing
// but those members in that order:
//   Pin          src/VCDTypes.h:126-137      TimedValue  :146-154
//   Delay        src/VCDTypes.h:174-185      ModuleType  :198-210
//   Function     src/Function.h:50-63        Instance    src/Instance.h:107-128
//   PreProcess   src/PreProcess.h:75-90      inter       src/process.cpp:54-79
// Boost is not available on this machine, so the archive grammar is
// implemented here from its published format (boost_inter.cpp); agreement
// with archives written by a real Boost build is unverified.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>
#include "design.h"

namespace glsh {
namespace ref {

struct Pin {
    std::string type, name;     // serialize order: type, name, size, lindex, rindex
    uint32_t size = 1;
    int lindex = -1, rindex = -1;
};

struct TimedValue {
    uint64_t t = 0;
    int value = 0;              // VCDBit: 0, X=1, Z=2, 1=3
};

struct Delay {
    int edge = 2;               // 0 posedge, 1 negedge, 2 both
    std::string in_bit, out_bit;   // the nets on the arc's input and output ports
    double rise = 1.0, fall = 1.0;
};

struct Function {
    std::string name;
    int id = 0;
    std::vector<std::string> input_pins;
    std::vector<int> input_data;    // VCDBit values (empty in archived designs)
    std::vector<std::string> output_pins;
    int output_data = 0;
};

struct ModuleType {
    std::string name;
    std::map<std::string, Pin> ports;
    std::vector<std::string> in_out_ports, supply1_vec, supply0_vec;
    std::vector<Function> function;
};

struct Instance {
    ModuleType type;
    std::string name;
    std::map<std::string, std::string> in_port_net;
    std::vector<std::string> in_net;
    std::map<std::string, std::string> out_port_net;
    std::vector<std::string> out_net, unknown_in, unknown_out;
    std::vector<Function> function_vec;
    std::vector<std::vector<int>> function_id_vec;
    std::vector<Delay> delays;
    std::vector<int> from_id;         // in_net_from_id: driver instance, -1 stimulus, -2 constant
    std::vector<std::string> from_info;
    std::vector<int> from_level, from_pos, from_out_order;
};

struct PreProcess {
    std::map<std::string, ModuleType> module_types;
    std::vector<std::string> ignored_modules;
    std::string top_module_name;
    std::map<std::string, Instance> instances;
    std::vector<std::string> instance_name_vec;
    std::map<std::string, std::vector<int>> net_instance_map;
    std::map<std::string, int> out_net_from_id;
    std::map<std::string, Pin> pins;
    std::vector<std::string> pin_bits;
    std::map<std::string, std::vector<TimedValue>> pinbit_values;   // archived through pointers
    std::map<std::string, std::string> assign_pairs;
    std::map<std::string, std::vector<uint64_t>> result;
};

struct Inter {
    PreProcess p;
    std::vector<std::vector<int>> levels;
    std::map<std::string, int> initial_net_map;
    std::vector<uint32_t> data_in_num_start, data_out_num_start, delay_start, delay_width, functions_start,
        functions_width;
    std::vector<int16_t> data_in_num, data_out_num;
    std::vector<uint32_t> val_num_start;
    std::vector<int16_t> delay_val_num, functions_func_num, functions_val_num, host_delay_edges, host_in_bit,
        host_out_bit;
    std::vector<float> host_rise_val, host_fall_val;
    std::vector<int16_t> host_functions;
    std::vector<std::map<std::string, std::vector<uint32_t>>> out_maps;
};

}  // namespace ref

// True when the bytes start like a Boost text archive.
bool is_boost_text_archive(const std::string &bytes);

// The archive text of an inter (library_version: the archive format version
// written in the header) and back.
std::string save_boost_inter(const ref::Inter &in, unsigned library_version = 17);
bool load_boost_inter(const std::string &text, ref::Inter &out, std::string *err);

// What `process` archives for a levelized design (src/process.cpp:196-608):
// the library's modules, every instance with its connections, function
// programs, delays and driver references, the level lists and the packed
// per-level arrays.
// pack = false leaves the packed per-level arrays empty (for pack_levels or
// pack_levels_gpu to fill).
void design_to_ref_inter(const Design &d, const Library &lib, ref::Inter &out, bool pack = true);
// The packed per-level arrays (src/process.cpp:423-566) from the levels and
// instances of `out`, on the host or on GPU `device` (gls_pack_levels;
// false with a message on a library error).
void pack_levels(ref::Inter &out);
bool pack_levels_gpu(ref::Inter &out, int device, std::string *err);
// The simulation model of an archived design: instances in level order
// with their function programs, arcs, constants, assign aliases and
// declared bus bits.
bool ref_inter_to_design(const ref::Inter &in, Design &d, std::string *err);

// The order in which the reference GPU tool writes SAIF records
// (src/simulate.cu:108-481, 1975-1980, 2151-2196, 2991-3000, 3289-3297).
// Its containers are libstdc++ unordered maps and sets; replaying the same
// insertions and erasures into the same container types gives the same
// iteration order.
struct SaifRecord {
    enum Kind { kNet, kConst, kUndriven } kind;
    std::string name;
    std::string source;      // kNet: the net whose counts are printed (an alias's source)
    uint64_t t0 = 0, t1 = 0; // kConst: the Result row (1 where the constant is 0 / 1)
};
struct VcdDecls {
    std::vector<std::pair<std::string, bool>> bits;   // declared bits in $var order, bus flag
};
std::vector<SaifRecord> saif_ref_order(const ref::Inter &in, const VcdDecls &vcd);

}  // namespace glsh
