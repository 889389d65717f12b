// ref_vcd_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own VCD reader -- VCDParser::init / parse / process
// of src/VCDParser.cpp:194-717, compiled from the reference sources by
// oracle/build.py -- the way its simulate tool calls it
// (src/simulate.cu:1971-1989), and prints every signal's change list as the
// tool then uses it: a bus bit's first `sizes` entries of times / values
// (src/simulate.cu:2171-2180), a scalar's list through hash_name_pair and
// hash_index_pair (:2184-2193).
//
// output: one line per declared bit, "@ name t:v t:v ...", names sorted
// (the reader writes progress lines of its own to stdout too).
//
// usage: ref_vcd <file.vcd> <dumpon> <dumpoff>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "VCDParser.h"

int main(int argc, char **argv)
{
    if (argc != 4) {
        fprintf(stderr, "usage: ref_vcd <file.vcd> <dumpon> <dumpoff>\n");
        return 2;
    }
    std::string path = argv[1];
    const VCDTime start = strtoull(argv[2], nullptr, 10), end = strtoull(argv[3], nullptr, 10);
    VCDParser parser;
    parser.init(path, end);
    if (!parser.parse(path, start, end)) {
        fprintf(stderr, "ref_vcd: parse failed\n");
        return 1;
    }
    parser.process();
    std::vector<std::string> lines;
    for (auto &name : parser.InMaps_bus) {
        std::string s = name;
        const unsigned n = parser.sizes[name];
        const auto &t = parser.times[name];
        const auto &v = parser.values[name];
        for (unsigned k = 0; k < n && k < t.size() && k < v.size(); ++k)
            s += " " + std::to_string(t[k]) + ":" + std::to_string(v[k]);
        lines.push_back(s);
    }
    for (auto &name : parser.InMaps_bit) {
        std::string s = name;
        auto h = parser.hash_name_pair.find(name);
        if (h != parser.hash_name_pair.end()) {
            auto ix = parser.hash_index_pair.find(h->second);
            if (ix != parser.hash_index_pair.end() && ix->second < parser.vec_times.size()) {
                const auto &t = parser.vec_times[ix->second];
                const auto &v = parser.vec_values[ix->second];
                for (size_t k = 0; k < t.size() && k < v.size(); ++k)
                    s += " " + std::to_string(t[k]) + ":" + std::to_string(v[k]);
            }
        }
        lines.push_back(s);
    }
    std::sort(lines.begin(), lines.end());
    for (auto &s : lines) printf("@ %s\n", s.c_str());   // the reader prints progress lines of its own
    return 0;
}
