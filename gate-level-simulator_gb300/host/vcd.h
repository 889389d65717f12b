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

}  // namespace glsh
