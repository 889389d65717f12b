// VCD stimulus reader and SAIF writer of the gls command-line tools.
#pragma once
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

namespace glsh {

// Change lists per bit name.  Scalars keep every change the file lists;
// bus bits keep only real changes, starting from Z as the reference's bus
// bit-blasting does (src/VCDParser.cpp:194-242).  A second change of one bit
// at the same time replaces the first.
struct VcdData {
    unsigned time_res = 1;
    std::string time_unit = "ps";
    std::unordered_map<std::string, size_t> index;   // bit name -> signal
    std::vector<std::string> names;
    std::vector<std::vector<uint64_t>> times;
    std::vector<std::vector<uint8_t>> values;        // 0, 1=X, 2=Z, 3
    // every declared bit in $var order, and whether its declaration is a bus
    // (the insertion order of the reference reader's InMaps_bus / InMaps_bit,
    // src/VCDParser.cpp:283-457)
    std::vector<std::pair<std::string, bool>> decl_bits;
};

bool parse_vcd(const std::string &text, VcdData &v, std::string *err);
// The same with the body scanned on GPU `device` (gls_vcd_scan): 1 when the
// GPU read the body, 0 when the host did (codes longer than 8 bytes, a body
// of 4 GB or more, a body the token-parallel scan reads differently, or a
// failed scan), -1 on an error in the header.
int parse_vcd_gpu(const std::string &text, VcdData &v, std::string *err, int device);

// Binary stimulus file: a VcdData as read from a VCD, stored so that a run
// loads it with a few large reads instead of parsing text.  Little endian:
//   "GLSSTIM1"
//   u32 time_res, u32 n_signals, u32 n_decl, u32 unit_len, char unit[unit_len]
//   per signal: u32 len, char name[len]
//   per declared bit: u32 len, char name[len], u8 bus
//   u64 start[n_signals + 1]          (first change of each signal)
//   u64 time[start[n_signals]]        (strictly increasing within a signal)
//   u8  value[start[n_signals]]       (0, 1=X, 2=Z, 3)
bool is_stim_bin(const std::string &bytes);
std::string save_stim_bin(const VcdData &v);
bool load_stim_bin(const std::string &bytes, VcdData &v, std::string *err);

}  // namespace glsh
