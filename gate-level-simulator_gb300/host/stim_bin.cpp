// Binary stimulus files (layout in vcd.h): written by gls_vcd2stim from a
// VCD, read by gls_simulate in place of the VCD.
#include <cstring>
#include "vcd.h"

namespace glsh {

namespace {
constexpr char kMagic[8] = {'G', 'L', 'S', 'S', 'T', 'I', 'M', '1'};

template <class T> void put(std::string &o, T x) { o.append(reinterpret_cast<const char *>(&x), sizeof x); }
void put_str(std::string &o, const std::string &s)
{
    put<uint32_t>(o, (uint32_t)s.size());
    o += s;
}

struct In {
    const std::string &b;
    size_t at = 8;
    bool ok = true;
    template <class T> T get()
    {
        T x{};
        if (!ok || b.size() - at < sizeof x) {
            ok = false;
            return x;
        }
        std::memcpy(&x, b.data() + at, sizeof x);
        at += sizeof x;
        return x;
    }
    std::string str()
    {
        const uint32_t n = get<uint32_t>();
        if (!ok || b.size() - at < n) {
            ok = false;
            return {};
        }
        std::string s = b.substr(at, n);
        at += n;
        return s;
    }
};
}  // namespace

bool is_stim_bin(const std::string &bytes)
{
    return bytes.size() >= 8 && std::memcmp(bytes.data(), kMagic, 8) == 0;
}

std::string save_stim_bin(const VcdData &v)
{
    std::string o(kMagic, 8);
    put<uint32_t>(o, v.time_res);
    put<uint32_t>(o, (uint32_t)v.names.size());
    put<uint32_t>(o, (uint32_t)v.decl_bits.size());
    put_str(o, v.time_unit);
    for (const auto &n : v.names) put_str(o, n);
    for (const auto &d : v.decl_bits) {
        put_str(o, d.first);
        put<uint8_t>(o, d.second ? 1 : 0);
    }
    uint64_t total = 0;
    put<uint64_t>(o, 0);
    for (const auto &t : v.times) {
        total += t.size();
        put<uint64_t>(o, total);
    }
    o.reserve(o.size() + total * 9);
    for (const auto &t : v.times) o.append(reinterpret_cast<const char *>(t.data()), t.size() * 8);
    for (const auto &x : v.values) o.append(reinterpret_cast<const char *>(x.data()), x.size());
    return o;
}

bool load_stim_bin(const std::string &bytes, VcdData &v, std::string *err)
{
    auto bad = [&](const char *what) {
        if (err) *err = std::string("binary stimulus: ") + what;
        return false;
    };
    if (!is_stim_bin(bytes)) return bad("not a GLSSTIM1 file");
    In in{bytes};
    v = VcdData();
    v.time_res = in.get<uint32_t>();
    const uint32_t ns = in.get<uint32_t>(), nd = in.get<uint32_t>();
    v.time_unit = in.str();
    if (!in.ok) return bad("truncated header");
    // every name takes at least its 4-byte length: bounds the counts by the file size
    if ((uint64_t)ns + nd > bytes.size() / 4) return bad("signal counts exceed the file");
    v.names.reserve(ns);
    for (uint32_t k = 0; k < ns && in.ok; ++k) {
        v.names.push_back(in.str());
        if (!v.index.emplace(v.names.back(), k).second) return bad("a signal name given twice");
    }
    v.decl_bits.reserve(nd);
    for (uint32_t k = 0; k < nd && in.ok; ++k) {
        std::string n = in.str();
        const uint8_t bus = in.get<uint8_t>();
        if (bus > 1) return bad("bus flag above 1");
        v.decl_bits.emplace_back(std::move(n), bus != 0);
    }
    if (!in.ok) return bad("truncated names");
    if ((bytes.size() - in.at) / 8 < (uint64_t)ns + 1) return bad("truncated change index");
    std::vector<uint64_t> start(ns + 1);
    std::memcpy(start.data(), bytes.data() + in.at, start.size() * 8);
    in.at += start.size() * 8;
    if (start[0] != 0) return bad("change index does not start at 0");
    for (uint32_t k = 0; k < ns; ++k)
        if (start[k + 1] < start[k]) return bad("change index not monotone");
    const uint64_t total = start[ns];
    if (total > (bytes.size() - in.at) / 9 || bytes.size() - in.at != total * 9)
        return bad("change arrays do not match the index");
    const char *tp = bytes.data() + in.at;
    const char *vp = tp + total * 8;
    v.times.resize(ns);
    v.values.resize(ns);
    for (uint32_t k = 0; k < ns; ++k) {
        const uint64_t a = start[k], n = start[k + 1] - a;
        v.times[k].resize(n);
        v.values[k].resize(n);
        std::memcpy(v.times[k].data(), tp + a * 8, n * 8);
        std::memcpy(v.values[k].data(), vp + a, n);
        for (uint64_t e = 0; e < n; ++e) {
            if (v.values[k][e] > 3) return bad("value above 3");
            if (e && v.times[k][e] <= v.times[k][e - 1]) return bad("times not strictly increasing");
        }
    }
    return true;
}

}  // namespace glsh
