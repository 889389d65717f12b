// Host-side design model of the gls command-line tools.
//
// `process` (gls_process) builds a Design from a Verilog cell library, a
// flat gate-level netlist and an SDF file, levelizes it and writes it to an
// inter.dat file; `simulate` (gls_simulate) reads it back, parses a VCD,
// runs libgls and writes SAIF.  This mirrors the reference's two-step flow
// (src/process.cpp:178-610, src/simulate.cu:1786-3315) with a native
// binary inter.dat instead of a Boost text archive.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

namespace glsh {

// A library module reduced to what simulation needs (ModuleType,
// src/VCDTypes.h:190-211): ports in declaration order and the function
// program in the reference's encoding (src/PreProcess.cpp:1194-1263) with
// pins numbered by port order: input k -> k, output k -> n_in + k,
// internal wires after, supply0 -> 16, supply1 -> 17.
struct Cell {
    std::string name;
    std::vector<std::string> inputs, outputs;
    struct Prim {
        uint8_t func;
        std::vector<uint8_t> pins;   // inputs, then the driven pin
    };
    std::vector<Prim> prims;
    // What the reference's ModuleType also records (kept for the Boost
    // inter.dat writer): every input / output / inout / wire / reg
    // declaration, the supply statements' tokens as its parser keeps them
    // (the keyword first, src/PreProcess.cpp:614-629) and the primitives by
    // port name.
    struct Decl {
        std::string name, type;
        int l = -1, r = -1;   // bus range, -1 for a scalar
    };
    std::vector<Decl> decls;
    std::vector<std::string> sup0_tokens, sup1_tokens;
    struct Func {
        std::string name;   // and, or, ..., udp_xbuf, udp_mux2
        int id;             // GLS_F_*
        std::vector<std::string> ins;
        std::string out;
    };
    std::vector<Func> funcs;
};

struct Arc {
    uint8_t edge;      // 0 posedge, 1 negedge, 2 both
    uint8_t in_pin;    // input port index
    uint8_t out_pin;   // output port index
    double rise, fall; // SDF units times the SDF TIMESCALE factor (ps)
};

struct Instance {
    std::string name;
    uint32_t cell;
    std::vector<uint32_t> pins;   // input nets then output nets (net ids)
    std::vector<Arc> arcs;
    uint32_t gv_index = 0;        // position in the netlist file (the reference's instance id)
    std::vector<uint32_t> conn;   // connected cell ports (pin indexes) in the order the netlist lists them
};

struct Design {
    std::string top;
    std::vector<std::string> net_names;
    std::unordered_map<std::string, uint32_t> net_id;
    std::vector<Cell> cells;
    std::vector<Instance> insts;              // in level order after levelize()
    std::vector<uint32_t> level_start;
    std::vector<std::pair<uint32_t, uint8_t>> constants;   // net, value (0 or 3)
    std::vector<std::pair<uint32_t, uint32_t>> aliases;    // assign left <- right
    std::vector<uint32_t> bus_bits;           // declared bus bits (reported even when undriven)
    std::vector<Cell::Decl> decls;            // the netlist's input / output / wire / inout declarations
    std::vector<std::string> ignored;         // library modules the front end skips
    std::vector<uint32_t> assign_consts;      // nets an assign ties to 1'b0 / 1'b1

    uint32_t net(const std::string &name);    // id of a net, created on first use
    int find_net(const std::string &name) const;
};

// The cell library: modules that simulation can evaluate, plus the names of
// modules the front end skips (sequential cells: udp_dff / udp_tlat /
// always blocks), whose outputs become stimulus nets.
struct Library {
    std::vector<Cell> cells;
    std::map<std::string, uint32_t> by_name;
    std::vector<std::string> ignored;
};

std::string read_file(const std::string &path, std::string *err);
bool parse_vlib(const std::string &text, Library &lib, std::string *err);
bool parse_gv(const std::string &text, const Library &lib, Design &d, std::string *err);
bool parse_sdf(const std::string &text, Design &d, const Library &lib, std::string *err);
bool levelize(Design &d, std::string *err);
// The levelization in two halves, for a levelizer elsewhere (gls_levelize on
// the GPU): every instance's distinct predecessors (the instances driving
// its input nets, through assign aliases), and the reordering of the
// instances by level.
void instance_preds(const Design &d, std::vector<uint64_t> &start, std::vector<uint32_t> &pred);
void apply_levels(Design &d, const std::vector<uint32_t> &order, const std::vector<uint32_t> &level_start);
bool write_inter(const std::string &path, const Design &d, std::string *err);
// Reads either format: the native one or the reference's Boost text archive.
bool read_inter(const std::string &path, Design &d, std::string *err);

}  // namespace glsh
