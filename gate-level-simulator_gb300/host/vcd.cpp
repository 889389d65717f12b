// VCD reader of the gls command-line tools.
//
// Reads what the reference's VCDParser reads (src/VCDParser.cpp:283-717):
// $timescale, $var declarations (scalars and buses with [msb:lsb] ranges,
// bit-blasted into name[i]), #time lines, scalar changes and b<bits>
// vector changes.  Real values are ignored.  Short vector values are
// extended on the left as VCD specifies (the reference indexes the string
// as if it were full width).
#include "vcd.h"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cstring>
#include "gls.h"

namespace glsh {

namespace {

uint8_t code(char c)
{
    switch (c) {
    case '0': return 0;
    case '1': return 3;
    case 'x': case 'X': return 1;
    case 'z': case 'Z': return 2;
    default: return 255;
    }
}

struct Var {
    std::vector<size_t> bits;   // signal index per value-string position (msb first)
    bool bus;
};

struct Tok {
    const std::string &s;
    size_t i = 0;
    bool next(std::string &t)
    {
        while (i < s.size() && isspace((unsigned char)s[i])) ++i;
        if (i >= s.size()) return false;
        size_t j = i;
        while (j < s.size() && !isspace((unsigned char)s[j])) ++j;
        t.assign(s, i, j - i);
        i = j;
        return true;
    }
    void skip_to_end()
    {
        std::string t;
        while (next(t) && t != "$end") {}
    }
};

using Vars = std::unordered_map<std::string, std::vector<Var>>;   // code -> declarations

// the header up to and including "$enddefinitions ... $end"
bool parse_header(Tok &tk, VcdData &v, Vars &vars, std::string *err)
{
    auto signal = [&](const std::string &name) -> size_t {
        auto it = v.index.find(name);
        if (it != v.index.end()) return it->second;
        const size_t k = v.names.size();
        v.index.emplace(name, k);
        v.names.push_back(name);
        v.times.emplace_back();
        v.values.emplace_back();
        return k;
    };
    std::string t;
    for (;;) {
        if (!tk.next(t)) {
            if (err) *err = "VCD: no $enddefinitions";
            return false;
        }
        if (t == "$enddefinitions") { tk.skip_to_end(); return true; }
        if (t == "$timescale") {
            std::string a, all;
            while (tk.next(a) && a != "$end") all += a;
            size_t k = 0;
            while (k < all.size() && isdigit((unsigned char)all[k])) ++k;
            v.time_res = k ? (unsigned)atoi(all.substr(0, k).c_str()) : 1u;
            v.time_unit = all.substr(k);
            continue;
        }
        if (t == "$var") {
            std::vector<std::string> f;
            std::string a;
            while (tk.next(a) && a != "$end") f.push_back(a);
            if (f.size() < 4) {
                if (err) *err = "VCD: short $var";
                return false;
            }
            const int size = atoi(f[1].c_str());
            const std::string id = f[2];
            std::string ref = f[3];
            std::string range = f.size() > 4 ? f[4] : std::string();
            const size_t br = ref.find('[');
            if (range.empty() && br != std::string::npos) {
                range = ref.substr(br);
                ref = ref.substr(0, br);
            }
            Var var;
            var.bus = false;
            if (size <= 1) {
                std::string name = ref;
                if (!range.empty()) {
                    const std::string inner = range.substr(1, range.find(']') - 1);
                    const size_t c = inner.find(':');
                    name = ref + "[" + (c == std::string::npos ? inner : inner.substr(0, c)) + "]";
                }
                var.bits.push_back(signal(name));
            } else {
                int l = size - 1, r = 0;
                if (!range.empty()) {
                    const std::string inner = range.substr(1, range.find(']') - 1);
                    const size_t c = inner.find(':');
                    if (c != std::string::npos) {
                        l = atoi(inner.substr(0, c).c_str());
                        r = atoi(inner.substr(c + 1).c_str());
                    }
                }
                var.bus = true;
                for (int b = l;; b += (r > l ? 1 : -1)) {
                    var.bits.push_back(signal(ref + "[" + std::to_string(b) + "]"));
                    if (b == r) break;
                }
            }
            for (size_t b : var.bits) v.decl_bits.push_back({v.names[b], var.bus});
            vars[id].push_back(var);
            continue;
        }
        if (t[0] == '$') tk.skip_to_end();
    }
}

// appends changes: bus bits keep only real changes, starting from Z, and a
// later change at the same time replaces an earlier one
struct Sink {
    VcdData &v;
    std::vector<uint8_t> last;   // bus bits: the last value kept
    explicit Sink(VcdData &d) : v(d), last(d.names.size(), 2) {}
    void put(size_t k, uint8_t val, bool dedup, uint64_t now)
    {
        auto &tt = v.times[k];
        auto &vv = v.values[k];
        if (dedup) {
            if (val == last[k]) return;
            last[k] = val;
        }
        if (!tt.empty() && tt.back() == now) {
            vv.back() = val;
            return;
        }
        tt.push_back(now);
        vv.push_back(val);
    }
};

void parse_body(Tok &tk, VcdData &v, const Vars &vars)
{
    Sink sink(v);
    uint64_t now = 0;
    std::string t;
    while (tk.next(t)) {
        const char c = t[0];
        if (c == '#') {
            now = strtoull(t.c_str() + 1, nullptr, 10);
            continue;
        }
        if (c == '$') {
            if (t == "$comment") tk.skip_to_end();
            continue;   // $dumpvars / $dumpall / $dumpon / $dumpoff / $end
        }
        if (c == 'b' || c == 'B') {
            std::string id;
            if (!tk.next(id)) break;
            auto it = vars.find(id);
            if (it == vars.end()) continue;
            std::string bits = t.substr(1);
            for (const Var &var : it->second) {
                std::string full = bits;
                if (full.size() < var.bits.size()) {
                    const char pad = (full[0] == 'x' || full[0] == 'X') ? 'x' : (full[0] == 'z' || full[0] == 'Z') ? 'z' : '0';
                    full = std::string(var.bits.size() - full.size(), pad) + full;
                }
                const size_t off = full.size() - var.bits.size();
                for (size_t b = 0; b < var.bits.size(); ++b) {
                    const uint8_t val = code(full[off + b]);
                    if (val != 255) sink.put(var.bits[b], val, var.bus, now);
                }
            }
            continue;
        }
        if (c == 'r' || c == 'R') {
            std::string id;
            tk.next(id);
            continue;
        }
        const uint8_t val = code(c);
        if (val == 255) continue;
        auto it = vars.find(t.substr(1));
        if (it == vars.end()) continue;
        for (const Var &var : it->second)
            for (size_t k : var.bits) sink.put(k, val, var.bus, now);
    }
}

}  // namespace

bool parse_vcd(const std::string &s, VcdData &v, std::string *err)
{
    Tok tk{s};
    Vars vars;
    if (!parse_header(tk, v, vars, err)) return false;
    parse_body(tk, v, vars);
    return true;
}

int parse_vcd_gpu(const std::string &s, VcdData &v, std::string *err, int device)
{
    Tok tk{s};
    Vars vars;
    if (!parse_header(tk, v, vars, err)) return -1;
    // the code table: keys of at most 8 bytes, sorted
    std::vector<std::pair<uint64_t, const std::vector<Var> *>> codes;
    bool fits = true;
    for (const auto &kv : vars) {
        const std::string &id = kv.first;
        if (id.empty() || id.size() > 8) { fits = false; break; }
        uint64_t key = 0;
        for (size_t j = 0; j < id.size(); ++j) key |= (uint64_t)(uint8_t)id[j] << (8 * j);
        codes.emplace_back(key, &kv.second);
    }
    const size_t body = tk.i, n = s.size() - body;
    if (!fits || n >= 0xFFFF0000ull) {
        parse_body(tk, v, vars);
        return 0;
    }
    std::sort(codes.begin(), codes.end(),
              [](const std::pair<uint64_t, const std::vector<Var> *> &a,
                 const std::pair<uint64_t, const std::vector<Var> *> &b) { return a.first < b.first; });
    std::vector<uint64_t> key;
    std::vector<uint32_t> var_start(1, 0), bit_start(1, 0), bits;
    std::vector<uint8_t> bus;
    for (const auto &c : codes) {
        key.push_back(c.first);
        for (const Var &var : *c.second) {
            for (size_t b : var.bits) bits.push_back((uint32_t)b);
            bit_start.push_back((uint32_t)bits.size());
            bus.push_back(var.bus ? 1 : 0);
        }
        var_start.push_back((uint32_t)bus.size());
    }
    gls_vcd_ids ids{(uint32_t)key.size(), key.data(), var_start.data(), bit_start.data(), bits.data(), bus.data()};
    gls_vcd_changes ch;
    const int rc = gls_vcd_scan(device, s.data() + body, n, &ids, &ch);
    if (rc || ch.fallback) {
        // the host reader gives the same changes (also when the device has
        // no room for the scan's work space)
        gls_vcd_free(&ch);
        parse_body(tk, v, vars);
        return 0;
    }
    {   // room for every signal's changes up front: no regrowth while they go in
        std::vector<uint64_t> cnt(v.names.size(), 0);
        for (uint64_t r = 0; r < ch.n; ++r)
            if (ch.value[r] != 255) ++cnt[ch.signal[r]];
        for (size_t k = 0; k < cnt.size(); ++k) {
            v.times[k].reserve(v.times[k].size() + cnt[k]);
            v.values[k].reserve(v.values[k].size() + cnt[k]);
        }
    }
    Sink sink(v);
    for (uint64_t r = 0; r < ch.n; ++r)
        if (ch.value[r] != 255) sink.put(ch.signal[r], ch.value[r], ch.bus[r] != 0, ch.time[r]);
    gls_vcd_free(&ch);
    return 1;
}

}  // namespace glsh
