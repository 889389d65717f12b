// Boost.Serialization text archive of the reference's `inter`: the grammar,
// the reference's archived content for a design, and the SAIF record order
// of the reference GPU tool.  See boost_inter.h.
//
// Archive grammar (Boost text_oarchive, the rules this file follows):
//   * header: the string "serialization::archive" (as "22 " + text), then
//     the library version number;
//   * every later item is one token after a single space; a string is its
//     length, a space and its bytes (so an empty string leaves two spaces);
//     integers and enums in decimal; float and double in scientific notation
//     with max_digits10 significant digits (9 and 17);
//   * a class object whose type is seen for the first time is preceded by
//     its tracking flag and class version ("0 0" here); class types are
//     numbered in the order of first use, which the archive does not write
//     except for pointers;
//   * collections of arithmetic types carry no class information; every
//     other collection (and std::pair, std::string excepted) is a class;
//   * a collection is its element count, its item version (0) and its
//     elements; a map's elements are pairs (first, second);
//   * a pointer is the class number of its target type, then (first time
//     that type is seen) tracking 1 and version 0, then the object number
//     (objects reached through pointers are counted from 0), then the
//     object; a null pointer is the class number -1.
#include "boost_inter.h"

#include <algorithm>
#include <cerrno>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>

namespace glsh {
namespace {

const char kSignature[] = "serialization::archive";

// ------------------------------------------------------------ type names
// Class types are told apart by name only, so the names must be unique per
// C++ type; they never appear in the archive.
template <class T> struct Key;
#define GLS_KEY(T, S)                                \
    template <> struct Key<T> {                      \
        static const std::string &get()              \
        {                                            \
            static const std::string k = S;          \
            return k;                                \
        }                                            \
    };
GLS_KEY(int, "int")
GLS_KEY(uint32_t, "unsigned")
GLS_KEY(int16_t, "short")
GLS_KEY(uint64_t, "u64")
GLS_KEY(float, "float")
GLS_KEY(double, "double")
GLS_KEY(std::string, "string")
GLS_KEY(ref::Pin, "Pin")
GLS_KEY(ref::TimedValue, "TimedValue")
GLS_KEY(ref::Delay, "Delay")
GLS_KEY(ref::Function, "Function")
GLS_KEY(ref::ModuleType, "ModuleType")
GLS_KEY(ref::Instance, "Instance")
GLS_KEY(ref::PreProcess, "PreProcess")
GLS_KEY(ref::Inter, "inter")
#undef GLS_KEY
template <class T> struct Key<std::vector<T>> {
    static const std::string &get()
    {
        static const std::string k = "vector<" + Key<T>::get() + ">";
        return k;
    }
};
template <class K, class V> struct Key<std::map<K, V>> {
    static const std::string &get()
    {
        static const std::string k = "map<" + Key<K>::get() + "," + Key<V>::get() + ">";
        return k;
    }
};
template <class K, class V> struct PairKey {
    static const std::string &get()
    {
        static const std::string k = "pair<" + Key<K>::get() + "," + Key<V>::get() + ">";
        return k;
    }
};
// Every type key is one static string: the registry tells types apart by
// the key's address.
const std::string kPinbitMap = "map<string,TimedValues*>";
const std::string kPinbitPair = "pair<string,TimedValues*>";
const std::string kTimedValues = "deque<TimedValue>";
const std::string kVectorVCDBit = "vector<VCDBit>";

// ------------------------------------------------------------ archives
struct Registry {
    std::unordered_map<const std::string *, int> id;   // class number by type key
    std::vector<char> tracked;                         // by class number
    // the class number of a type; *fresh is set on its first use, which
    // gives it the next number
    int use(const std::string &k, bool *fresh)
    {
        const auto it = id.find(&k);
        if (it != id.end()) {
            *fresh = false;
            return it->second;
        }
        const int c = (int)tracked.size();
        id.emplace(&k, c);
        tracked.push_back(0);
        *fresh = true;
        return c;
    }
    int find(const std::string &k) const
    {
        const auto it = id.find(&k);
        return it == id.end() ? -1 : it->second;
    }
};

struct Saver {
    static constexpr bool kLoad = false;
    std::string out;
    Registry reg;
    uint32_t next_object = 0;
    bool ok = true;

    void tok(const char *s)
    {
        if (!out.empty()) out.push_back(' ');
        out += s;
    }
    void i64(long long x)
    {
        char b[32];
        snprintf(b, sizeof b, "%lld", x);
        tok(b);
    }
    void u64(unsigned long long x)
    {
        char b[32];
        snprintf(b, sizeof b, "%llu", x);
        tok(b);
    }
    template <class T> void integer(T &x)
    {
        if (std::is_signed<T>::value) i64((long long)x);
        else u64((unsigned long long)x);
    }
    void real(float &x)
    {
        char b[64];
        snprintf(b, sizeof b, "%.9e", (double)x);
        tok(b);
    }
    void real(double &x)
    {
        char b[64];
        snprintf(b, sizeof b, "%.17e", x);
        tok(b);
    }
    void str(std::string &s)
    {
        u64(s.size());
        out.push_back(' ');
        out += s;
    }
    // class information of a type's first object
    void class_info(int, int tracking)
    {
        int t = tracking, v = 0;
        integer(t);
        integer(v);
    }
    bool tracked(int) const { return false; }
    void fail(const std::string &) { ok = false; }
};

struct Loader {
    static constexpr bool kLoad = true;
    const char *p, *e;
    Registry reg;
    bool ok = true;
    std::string err;
    std::vector<std::vector<ref::TimedValue>> objects;   // objects read through pointers, by number

    Loader(const std::string &s) : p(s.data()), e(s.data() + s.size()) {}
    void fail(const std::string &m)
    {
        if (ok) err = m;
        ok = false;
    }
    static bool space(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t'; }
    // the next token, in place: [*b, *n)
    bool word(const char *&b, const char *&n)
    {
        while (p < e && space(*p)) ++p;
        b = p;
        while (p < e && !space(*p)) ++p;
        n = p;
        if (b == n) fail("archive ends early");
        return ok;
    }
    template <class T> void integer(T &x)
    {
        const char *b, *n;
        if (!word(b, n)) return;
        const char *q = b;
        const bool neg = *q == '-';
        if (neg) {
            if (!std::is_signed<T>::value) return fail("negative count '" + std::string(b, n) + "'");
            ++q;
        }
        if (q == n || n - q > 20) return fail("bad integer '" + std::string(b, n) + "'");
        unsigned long long v = 0;
        for (; q < n; ++q) {
            const unsigned d = (unsigned)(*q - '0');
            if (d > 9 || v > (~0ull - d) / 10) return fail("bad integer '" + std::string(b, n) + "'");
            v = v * 10 + d;
        }
        x = neg ? (T)(-(long long)v) : (T)v;
    }
    template <class T> void real(T &x)
    {
        const char *b, *n;
        if (!word(b, n)) return;
        char *end = nullptr;
        const double v = strtod(b, &end);   // stops at the delimiter after the token
        if (end != n) return fail("bad number '" + std::string(b, n) + "'");
        x = (T)v;
    }
    void str(std::string &s)
    {
        uint64_t n = 0;
        integer(n);
        if (!ok) return;
        if (n > 0) {
            if (p >= e) return fail("archive ends early");
            ++p;   // the one delimiter before the bytes
            if ((uint64_t)(e - p) < n) return fail("string runs past the end of the archive");
            s.assign(p, (size_t)n);
            p += n;
        } else {
            s.clear();
        }
    }
    void class_info(int cid, int)
    {
        int tracking = 0, version = 0;
        integer(tracking);
        integer(version);
        reg.tracked[cid] = tracking != 0;
    }
    bool tracked(int cid) const { return reg.tracked[cid] != 0; }
    // a count that cannot exceed the bytes left (each element takes at least one)
    bool sane_count(uint64_t n)
    {
        if (n > (uint64_t)(e - p)) fail("collection count larger than the archive");
        return ok;
    }
};

template <class A, class F>
void object(A &a, const std::string &key, bool class_info, F &&body)
{
    if (!a.ok) return;
    bool fresh = false;
    const int cid = a.reg.use(key, &fresh);
    if (fresh && class_info) a.class_info(cid, 0);
    if (!a.ok) return;
    if (A::kLoad && a.tracked(cid)) {   // an archive that tracks this type numbers its objects
        uint32_t oid = 0;
        a.integer(oid);
    }
    body();
}

template <class A> void io(A &a, int &x) { a.integer(x); }
template <class A> void io(A &a, uint32_t &x) { a.integer(x); }
template <class A> void io(A &a, int16_t &x) { a.integer(x); }
template <class A> void io(A &a, uint64_t &x) { a.integer(x); }
template <class A> void io(A &a, float &x) { a.real(x); }
template <class A> void io(A &a, double &x) { a.real(x); }
template <class A> void io(A &a, std::string &x) { a.str(x); }

template <class A> void count_and_version(A &a, uint64_t &n)
{
    a.integer(n);
    uint32_t item_version = 0;
    a.integer(item_version);
    if constexpr (A::kLoad) {
        if (a.ok) a.sane_count(n);
    }
}

template <class A, class T> void io(A &a, std::vector<T> &v)
{
    object(a, Key<std::vector<T>>::get(), !std::is_arithmetic<T>::value, [&] {
        uint64_t n = v.size();
        count_and_version(a, n);
        if (!a.ok) return;
        if (A::kLoad) v.assign((size_t)n, T());
        for (auto &x : v) {
            io(a, x);
            if (!a.ok) return;
        }
    });
}

template <class A, class K, class V> void io(A &a, std::map<K, V> &m)
{
    const std::string &pair_key = PairKey<K, V>::get();
    object(a, Key<std::map<K, V>>::get(), true, [&] {
        uint64_t n = m.size();
        count_and_version(a, n);
        if (!a.ok) return;
        if (A::kLoad) {
            m.clear();
            for (uint64_t i = 0; i < n && a.ok; ++i) {
                K k{};
                V v{};
                object(a, pair_key, true, [&] {
                    io(a, k);
                    io(a, v);
                });
                m.emplace(std::move(k), std::move(v));
            }
        } else {
            for (auto &kv : m) {
                K k = kv.first;
                object(a, pair_key, true, [&] {
                    io(a, k);
                    io(a, kv.second);
                });
            }
        }
    });
}

template <class A> void io(A &a, ref::Pin &x)
{
    object(a, Key<ref::Pin>::get(), true, [&] {
        io(a, x.type);
        io(a, x.name);
        io(a, x.size);
        io(a, x.lindex);
        io(a, x.rindex);
    });
}
template <class A> void io(A &a, ref::TimedValue &x)
{
    object(a, Key<ref::TimedValue>::get(), true, [&] {
        io(a, x.t);
        io(a, x.value);
    });
}
template <class A> void io(A &a, ref::Delay &x)
{
    object(a, Key<ref::Delay>::get(), true, [&] {
        io(a, x.edge);
        io(a, x.in_bit);
        io(a, x.out_bit);
        io(a, x.rise);
        io(a, x.fall);
    });
}
template <class A> void io(A &a, ref::Function &x)
{
    object(a, Key<ref::Function>::get(), true, [&] {
        io(a, x.name);
        io(a, x.id);
        io(a, x.input_pins);
        // std::vector<VCDBit>: a collection of an enum is not one of the
        // arithmetic collections, so it carries class information
        object(a, kVectorVCDBit, true, [&] {
            uint64_t n = x.input_data.size();
            count_and_version(a, n);
            if (!a.ok) return;
            if (A::kLoad) x.input_data.assign((size_t)n, 0);
            for (auto &b : x.input_data) io(a, b);
        });
        io(a, x.output_pins);
        io(a, x.output_data);
    });
}
template <class A> void io(A &a, ref::ModuleType &x)
{
    object(a, Key<ref::ModuleType>::get(), true, [&] {
        io(a, x.name);
        io(a, x.ports);
        io(a, x.in_out_ports);
        io(a, x.supply1_vec);
        io(a, x.supply0_vec);
        io(a, x.function);
    });
}
template <class A> void io(A &a, ref::Instance &x)
{
    object(a, Key<ref::Instance>::get(), true, [&] {
        io(a, x.type);
        io(a, x.name);
        io(a, x.in_port_net);
        io(a, x.in_net);
        io(a, x.out_port_net);
        io(a, x.out_net);
        io(a, x.unknown_in);
        io(a, x.unknown_out);
        io(a, x.function_vec);
        io(a, x.function_id_vec);
        io(a, x.delays);
        io(a, x.from_id);
        io(a, x.from_info);
        io(a, x.from_level);
        io(a, x.from_pos);
        io(a, x.from_out_order);
    });
}

template <class F>
void load_pointed(Loader &l, std::vector<ref::TimedValue> &v, const std::string &k, F &&body)
{
    int cid = 0;
    l.integer(cid);
    if (!l.ok) return;
    if (cid == -1) {   // a null pointer: read as an empty list
        v.clear();
        return;
    }
    const int known = l.reg.find(k);
    if (known < 0) {
        if (cid != (int)l.reg.tracked.size()) return l.fail("unexpected class number " + std::to_string(cid));
        bool fresh = false;
        l.reg.use(k, &fresh);
        l.class_info(cid, 1);
    } else if (known != cid) {
        return l.fail("pointer class number " + std::to_string(cid) + " is not the TimedValues class");
    }
    if (!l.tracked(cid)) return body();
    uint32_t oid = 0;
    l.integer(oid);
    if (!l.ok) return;
    if (oid < l.objects.size()) {   // a second pointer to an object read before
        v = l.objects[oid];
        return;
    }
    if (oid != l.objects.size()) return l.fail("object number out of sequence");
    l.objects.emplace_back();
    body();
    if (l.ok) l.objects[oid] = v;
}

// map<string, TimedValues*>: every value is a pointer to a deque of
// TimedValue (a tracked class, since it is archived through pointers)
template <class A> void io_pointed(A &a, std::vector<ref::TimedValue> &v)
{
    const std::string &k = kTimedValues;
    auto body = [&] {
        uint64_t n = v.size();
        count_and_version(a, n);
        if (!a.ok) return;
        if (A::kLoad) v.assign((size_t)n, ref::TimedValue());
        for (auto &x : v) {
            io(a, x);
            if (!a.ok) return;
        }
    };
    if constexpr (!A::kLoad) {
        bool fresh = false;
        int cid = a.reg.use(k, &fresh);
        a.integer(cid);
        if (fresh) {
            a.reg.tracked[cid] = 1;
            a.class_info(cid, 1);
        }
        uint32_t oid = a.next_object++;
        a.integer(oid);
        body();
    } else {
        load_pointed(a, v, k, body);
    }
}

template <class A> void io_pinbits(A &a, std::map<std::string, std::vector<ref::TimedValue>> &m)
{
    object(a, kPinbitMap, true, [&] {
        uint64_t n = m.size();
        count_and_version(a, n);
        if (!a.ok) return;
        if (A::kLoad) {
            m.clear();
            for (uint64_t i = 0; i < n && a.ok; ++i) {
                std::string k;
                std::vector<ref::TimedValue> v;
                object(a, kPinbitPair, true, [&] {
                    io(a, k);
                    io_pointed(a, v);
                });
                m.emplace(std::move(k), std::move(v));
            }
        } else {
            for (auto &kv : m) {
                std::string k = kv.first;
                object(a, kPinbitPair, true, [&] {
                    io(a, k);
                    io_pointed(a, kv.second);
                });
            }
        }
    });
}

template <class A> void io(A &a, ref::PreProcess &x)
{
    object(a, Key<ref::PreProcess>::get(), true, [&] {
        io(a, x.module_types);
        io(a, x.ignored_modules);
        io(a, x.top_module_name);
        io(a, x.instances);
        io(a, x.instance_name_vec);
        io(a, x.net_instance_map);
        io(a, x.out_net_from_id);
        io(a, x.pins);
        io(a, x.pin_bits);
        io_pinbits(a, x.pinbit_values);
        io(a, x.assign_pairs);
        io(a, x.result);
    });
}
template <class A> void io(A &a, ref::Inter &x)
{
    object(a, Key<ref::Inter>::get(), true, [&] {
        io(a, x.p);
        io(a, x.levels);
        io(a, x.initial_net_map);
        io(a, x.data_in_num_start);
        io(a, x.data_out_num_start);
        io(a, x.delay_start);
        io(a, x.delay_width);
        io(a, x.functions_start);
        io(a, x.functions_width);
        io(a, x.data_in_num);
        io(a, x.data_out_num);
        io(a, x.val_num_start);
        io(a, x.delay_val_num);
        io(a, x.functions_func_num);
        io(a, x.functions_val_num);
        io(a, x.host_delay_edges);
        io(a, x.host_in_bit);
        io(a, x.host_out_bit);
        io(a, x.host_rise_val);
        io(a, x.host_fall_val);
        io(a, x.host_functions);
        io(a, x.out_maps);
    });
}

}  // namespace

bool is_boost_text_archive(const std::string &bytes)
{
    const std::string head = std::string("22 ") + kSignature;
    return bytes.compare(0, head.size(), head) == 0;
}

std::string save_boost_inter(const ref::Inter &in, unsigned library_version)
{
    Saver s;
    std::string sig = kSignature;
    s.str(sig);
    s.integer(library_version);
    ref::Inter copy = in;   // the generic code takes references
    io(s, copy);
    s.out.push_back('\n');
    return s.out;
}

bool load_boost_inter(const std::string &text, ref::Inter &out, std::string *err)
{
    Loader l(text);
    std::string sig;
    l.str(sig);
    if (l.ok && sig != kSignature) l.fail("not a Boost serialization archive");
    unsigned version = 0;
    l.integer(version);
    if (l.ok && version < 4) l.fail("archive library version " + std::to_string(version) + " predates item versions");
    out = ref::Inter();
    io(l, out);
    if (!l.ok) {
        if (err) *err = "inter.dat (Boost text archive): " + l.err;
        return false;
    }
    return true;
}

// ------------------------------------------------ design -> archived content
namespace {

int index_of(const std::vector<std::string> &v, const std::string &x)
{
    auto it = std::find(v.begin(), v.end(), x);
    return (int)(it - v.begin());   // v.size() when absent, as std::distance to end gives
}

ref::ModuleType module_of(const Cell &c)
{
    ref::ModuleType m;
    m.name = c.name;
    for (auto &d : c.decls) {
        ref::Pin p;
        p.type = d.type;
        p.name = d.name;
        p.lindex = d.l;
        p.rindex = d.r;
        p.size = d.l < 0 ? 1u : (uint32_t)(std::abs(d.l - d.r) + 1);
        m.ports[d.name] = p;
        if (d.type == "input" || d.type == "output" || d.type == "inout") m.in_out_ports.push_back(d.name);
    }
    m.supply1_vec = c.sup1_tokens;
    m.supply0_vec = c.sup0_tokens;
    for (auto &f : c.funcs) {
        ref::Function g;
        g.name = f.name;
        g.id = f.id;
        g.input_pins = f.ins;
        g.output_pins = {f.out};
        m.function.push_back(g);
    }
    return m;
}

}  // namespace

void design_to_ref_inter(const Design &d, const Library &lib, ref::Inter &out, bool pack)
{
    out = ref::Inter();
    ref::PreProcess &p = out.p;
    std::map<std::string, const Cell *> lib_cell;
    for (auto &c : lib.cells) {
        p.module_types[c.name] = module_of(c);
        lib_cell[c.name] = &c;
    }
    p.ignored_modules = d.ignored;
    p.top_module_name = d.top;
    const size_t n = d.insts.size();
    // instances by their netlist position (the reference's instance ids);
    // a design without those positions (read from the native format) numbers
    // its instances in level order
    std::vector<uint32_t> gv_of(n);
    {
        std::vector<char> seen(n, 0);
        bool perm = true;
        for (size_t k = 0; k < n && perm; ++k) {
            const uint32_t g = d.insts[k].gv_index;
            perm = g < n && !seen[g];
            if (perm) seen[g] = 1;
        }
        for (size_t k = 0; k < n; ++k) gv_of[k] = perm ? d.insts[k].gv_index : (uint32_t)k;
    }
    std::vector<const Instance *> by_gv(n, nullptr);
    std::vector<int> level_of(n, 0), pos_of(n, 0);
    for (size_t L = 0; L + 1 < d.level_start.size(); ++L)
        for (uint32_t k = d.level_start[L]; k < d.level_start[L + 1]; ++k) {
            const uint32_t g = gv_of[k];
            by_gv[g] = &d.insts[k];
            level_of[g] = (int)L;
            pos_of[g] = (int)(k - d.level_start[L]);
        }
    auto net = [&](uint32_t id) -> const std::string & { return d.net_names[id]; };
    // declared pins and bits
    for (auto &dc : d.decls) {
        ref::Pin pin;
        pin.type = dc.type;
        pin.name = dc.name;
        pin.lindex = dc.l;
        pin.rindex = dc.r;
        pin.size = dc.l < 0 ? 1u : (uint32_t)(std::abs(dc.l - dc.r) + 1);
        p.pins[dc.name] = pin;
        if (dc.l < 0) {
            p.pin_bits.push_back(dc.name);
        } else {
            for (int b = dc.l;; b += (dc.r > dc.l ? 1 : -1)) {
                p.pin_bits.push_back(dc.name + "[" + std::to_string(b) + "]");
                if (b == dc.r) break;
            }
        }
    }
    // a design read from the native format keeps neither the declarations
    // nor which constants an assign made: its declared bus bits stand for
    // the former, every constant but the two tie-offs for the latter
    if (d.decls.empty())
        for (uint32_t b : d.bus_bits) p.pin_bits.push_back(net(b));
    std::vector<uint32_t> assign_consts = d.assign_consts;
    if (assign_consts.empty())
        for (auto &c : d.constants)
            if (net(c.first) != "1'b0" && net(c.first) != "1'b1") assign_consts.push_back(c.first);
    std::vector<int8_t> constant(d.net_names.size(), -1);
    for (auto &c : d.constants) constant[c.first] = (int8_t)c.second;
    for (uint32_t ln : assign_consts) {
        ref::TimedValue tv;
        tv.value = constant[ln];
        p.pinbit_values[net(ln)] = {tv};
        p.result[net(ln)] = {tv.value == 3 ? 0ull : 1ull, tv.value == 3 ? 1ull : 0ull, 0ull};
    }
    for (auto &a : d.aliases) p.assign_pairs[net(a.first)] = net(a.second);
    // instances
    for (size_t g = 0; g < n; ++g) {
        const Instance &in = *by_gv[g];
        const Cell &cell = d.cells[in.cell];
        auto lcit = lib_cell.find(cell.name);   // absent: the record serves the SAIF order only
        const Cell &lc = lcit != lib_cell.end() ? *lcit->second : cell;
        ref::Instance r;
        if (lcit != lib_cell.end()) r.type = p.module_types[cell.name];
        r.name = in.name;
        const size_t ni = cell.inputs.size();
        std::vector<uint32_t> conn = in.conn;
        if (conn.empty())   // the native format keeps no port list: a port on its private open net was left open
            for (uint32_t k = 0; k < in.pins.size(); ++k) {
                const std::string &nm = net(in.pins[k]);
                const bool open = k < ni ? nm == "gls_open_input" : nm == in.name + "[" + cell.outputs[k - ni] + "]";
                if (!open) conn.push_back(k);
            }
        for (uint32_t port : conn) {
            const std::string &nm = net(in.pins[port]);
            if (port < ni) {
                r.in_port_net[cell.inputs[port]] = nm;
                r.in_net.push_back(nm);
                p.net_instance_map[nm].push_back((int)g);
                if (nm == "1'b0" || nm == "1'b1") {   // an instance pin tied off: a constant net
                    ref::TimedValue tv;
                    tv.value = nm == "1'b1" ? 3 : 0;
                    p.pinbit_values[nm] = {tv};
                    p.pins[nm] = ref::Pin{"wire", nm, 1, -1, -1};
                }
            } else {
                r.out_port_net[cell.outputs[port - ni]] = nm;
                r.out_net.push_back(nm);
                p.out_net_from_id[nm] = (int)g;
            }
        }
        for (auto &port : r.type.in_out_ports) {   // ports left open (src/PreProcess.cpp:1175-1183)
            if (!r.in_port_net.count(port) && !r.out_port_net.count(port)) r.unknown_out.push_back(port);
        }
        // function programs with ports replaced by nets (src/PreProcess.cpp:1184-1263)
        int pin_id = (int)(r.in_net.size() + r.out_net.size() + r.unknown_out.size());
        std::map<std::string, int> wires;
        auto in_list = [&](const std::vector<std::string> &v, const std::string &x) {
            return std::find(v.begin(), v.end(), x) != v.end();
        };
        for (auto &f : lc.funcs) {
            ref::Function fn;
            fn.name = f.name;
            fn.id = f.id;
            fn.input_pins = f.ins;
            fn.output_pins = {f.out};
            std::vector<int> row{f.id};
            for (size_t j = 0; j < fn.input_pins.size(); ++j) {
                const std::string cur = fn.input_pins[j];
                auto ip = r.in_port_net.find(cur);
                if (ip != r.in_port_net.end()) {
                    std::replace(fn.input_pins.begin(), fn.input_pins.end(), cur, ip->second);
                    row.push_back(index_of(r.in_net, ip->second));
                } else if (wires.count(cur)) {
                    row.push_back(wires[cur]);
                } else if (in_list(r.type.supply1_vec, cur)) {
                    row.push_back(17);
                } else if (in_list(r.type.supply0_vec, cur)) {
                    row.push_back(16);
                } else {
                    wires[cur] = pin_id;
                    row.push_back(pin_id++);
                }
            }
            {
                const std::string cur = fn.output_pins[0];
                auto op = r.out_port_net.find(cur);
                if (op != r.out_port_net.end()) {
                    fn.output_pins[0] = op->second;
                    row.push_back(index_of(r.out_net, op->second) + (int)r.in_net.size());
                } else if (wires.count(cur)) {
                    row.push_back(wires[cur]);
                } else if (in_list(r.type.supply1_vec, cur)) {
                    row.push_back(17);
                } else if (in_list(r.type.supply0_vec, cur)) {
                    row.push_back(16);
                } else {
                    wires[cur] = pin_id;
                    row.push_back(pin_id++);
                }
            }
            r.function_vec.push_back(fn);
            r.function_id_vec.push_back(row);
        }
        for (auto &a : in.arcs) {
            ref::Delay dl;
            dl.edge = a.edge;
            dl.in_bit = net(in.pins[a.in_pin]);
            // an output port left open is named by the port itself, as the
            // reference's SDF reader takes it from unknown_out
            const std::string &oport = cell.outputs[a.out_pin];
            const bool open_out = std::find(r.unknown_out.begin(), r.unknown_out.end(), oport) != r.unknown_out.end();
            dl.out_bit = open_out ? oport : net(in.pins[ni + a.out_pin]);
            dl.rise = a.rise;
            dl.fall = a.fall;
            r.delays.push_back(dl);
        }
        p.instance_name_vec.push_back(in.name);
        p.instances[in.name] = std::move(r);
    }
    // levels (instance ids in level order)
    for (size_t L = 0; L + 1 < d.level_start.size(); ++L) {
        std::vector<int> lv;
        for (uint32_t k = d.level_start[L]; k < d.level_start[L + 1]; ++k) lv.push_back((int)gv_of[k]);
        out.levels.push_back(lv);
    }
    auto inst = [&](int id) -> ref::Instance & { return p.instances.at(p.instance_name_vec[id]); };
    // where every input net comes from (src/process.cpp:276-372)
    std::map<std::string, int> initial_ids;
    auto initial = [&](const std::string &nm) {
        auto it = initial_ids.find(nm);
        if (it == initial_ids.end()) it = initial_ids.emplace(nm, (int)initial_ids.size()).first;
        return it->second;
    };
    auto from_driver = [&](ref::Instance &cur, int id, const std::string &nm) {
        const ref::Instance &drv = inst(id);
        const int order = drv.out_net.size() <= 1 ? 0 : index_of(drv.out_net, nm);
        cur.from_id.push_back(id);
        cur.from_info.push_back(p.instance_name_vec[id]);
        cur.from_level.push_back(level_of[id]);
        cur.from_pos.push_back(pos_of[id]);
        cur.from_out_order.push_back(order);
    };
    auto from = [&](ref::Instance &cur, int id, const std::string &info, int level, int pos) {
        cur.from_id.push_back(id);
        cur.from_info.push_back(info);
        cur.from_level.push_back(level);
        cur.from_pos.push_back(pos);
        cur.from_out_order.push_back(0);
    };
    for (size_t g = 0; g < n; ++g) {
        ref::Instance &cur = inst((int)g);
        for (const std::string &nm : cur.in_net) {
            auto drv = p.out_net_from_id.find(nm);
            auto pb = p.pinbit_values.find(nm);
            auto as = p.assign_pairs.find(nm);
            if (drv != p.out_net_from_id.end()) {
                from_driver(cur, drv->second, nm);
            } else if (pb != p.pinbit_values.end()) {
                from(cur, -2, nm, -2, pb->second.empty() ? 0 : pb->second[0].value);
            } else if (as != p.assign_pairs.end()) {
                const std::string &src = as->second;
                auto d2 = p.out_net_from_id.find(src);
                auto p2 = p.pinbit_values.find(src);
                if (d2 != p.out_net_from_id.end()) from_driver(cur, d2->second, src);
                else if (p2 != p.pinbit_values.end()) from(cur, -2, src, -2, p2->second.empty() ? 0 : p2->second[0].value);
                else from(cur, -1, src, -1, initial(src));
            } else {
                from(cur, -1, nm, -1, initial(nm));
            }
        }
    }
    // outputs per level, first position of each net (src/process.cpp:252-274)
    out.out_maps.assign(out.levels.size(), {});
    for (size_t L = 0; L < out.levels.size(); ++L)
        for (size_t j = 0; j < out.levels[L].size(); ++j) {
            const ref::Instance &cur = inst(out.levels[L][j]);
            for (size_t k = 0; k < cur.out_net.size(); ++k)
                if (!out.out_maps[L].count(cur.out_net[k]))
                    out.out_maps[L][cur.out_net[k]] = {(uint32_t)j, (uint32_t)k};
        }
    if (pack) pack_levels(out);
}

// The packed per-level arrays of an archived design (src/process.cpp:423-566).
void pack_levels(ref::Inter &out)
{
    ref::PreProcess &p = out.p;
    auto inst = [&](int id) -> ref::Instance & { return p.instances.at(p.instance_name_vec[id]); };
    size_t n = 0;   // instances over all levels
    for (auto &lv : out.levels) n += lv.size();
    const size_t nl = out.levels.size();
    out.data_in_num_start.assign(nl, 0);
    out.data_out_num_start.assign(nl, 0);
    out.delay_start.assign(nl, 0);
    out.delay_width.assign(nl, 0);
    out.functions_start.assign(nl, 0);
    out.functions_width.assign(nl, 0);
    out.data_in_num.assign(n, 0);
    out.data_out_num.assign(n, 0);
    out.val_num_start.assign(n, 0);
    out.delay_val_num.assign(n, 0);
    out.functions_func_num.assign(n, 0);
    out.functions_val_num.assign(n, 0);
    uint32_t sum = 0, dstart = 0, fstart = 0;
    for (size_t L = 0; L < nl; ++L) {
        const auto &lv = out.levels[L];
        uint32_t val_w = 0, dw = 0, fw = 0;
        out.data_in_num_start[L] = out.data_out_num_start[L] = sum;
        out.functions_start[L] = fstart;
        out.delay_start[L] = dstart;
        for (size_t j = 0; j < lv.size(); ++j) {
            const ref::Instance &cur = inst(lv[j]);
            out.data_in_num[j + sum] = (int16_t)cur.in_net.size();
            out.data_out_num[j + sum] = (int16_t)cur.out_net.size();
            out.val_num_start[j + sum] = val_w;
            val_w += (uint32_t)cur.in_net.size();
            out.delay_val_num[j + sum] = (int16_t)cur.delays.size();
            dw = std::max(dw, (uint32_t)cur.delays.size());
            uint32_t width = 0;
            for (auto &row : cur.function_id_vec) width = std::max(width, (uint32_t)row.size());
            fw = std::max(fw, width * (uint32_t)cur.function_id_vec.size());
            out.functions_func_num[j + sum] = (int16_t)cur.function_id_vec.size();
            out.functions_val_num[j + sum] = (int16_t)width;
        }
        sum += (uint32_t)lv.size();
        dstart += (uint32_t)lv.size() * dw;
        fstart += (uint32_t)lv.size() * fw;
        out.delay_width[L] = dw;
        out.functions_width[L] = fw;
    }
    out.host_delay_edges.assign(dstart, 0);
    out.host_in_bit.assign(dstart, 0);
    out.host_out_bit.assign(dstart, 0);
    out.host_rise_val.assign(dstart, 0.f);
    out.host_fall_val.assign(dstart, 0.f);
    out.host_functions.assign(fstart, 0);
    for (size_t L = 0; L < nl; ++L) {
        const auto &lv = out.levels[L];
        const uint32_t ds = out.delay_start[L], dw = out.delay_width[L], fs = out.functions_start[L],
                       fw = out.functions_width[L];
        for (size_t j = 0; j < lv.size(); ++j) {
            const ref::Instance &cur = inst(lv[j]);
            for (size_t k = 0; k < dw; ++k) {
                const size_t at = ds + j * dw + k;
                if (k < cur.delays.size()) {
                    const ref::Delay &dl = cur.delays[k];
                    out.host_delay_edges[at] = (int16_t)dl.edge;
                    out.host_in_bit[at] = (int16_t)index_of(cur.in_net, dl.in_bit);
                    out.host_out_bit[at] = (int16_t)index_of(cur.out_net, dl.out_bit);
                    out.host_rise_val[at] = (float)dl.rise;
                    out.host_fall_val[at] = (float)dl.fall;
                } else {
                    out.host_delay_edges[at] = out.host_in_bit[at] = out.host_out_bit[at] = -1;
                    out.host_rise_val[at] = out.host_fall_val[at] = -1.0f;
                }
            }
            const size_t h = cur.function_id_vec.size();
            const size_t w = h ? fw / h : 0;
            for (size_t r2 = 0; r2 < h; ++r2)
                for (size_t k = 0; k < w; ++k)
                    out.host_functions[fs + j * fw + r2 * w + k] =
                        (int16_t)(k < cur.function_id_vec[r2].size() ? cur.function_id_vec[r2][k] : -1);
            for (size_t k = w * h; k < fw; ++k) out.host_functions[fs + j * fw + k] = -1;
        }
    }
}

// ------------------------------------------------ archived content -> design
bool ref_inter_to_design(const ref::Inter &in, Design &d, std::string *err)
{
    d = Design();
    const ref::PreProcess &p = in.p;
    d.top = p.top_module_name;
    {   // about one net per instance output plus the declared bits: no rehash while the names go in
        const size_t nets = p.out_net_from_id.size() + p.pin_bits.size() + p.net_instance_map.size() + 16;
        d.net_id.reserve(nets);
        d.net_names.reserve(nets);
    }
    for (const std::string &b : p.pin_bits) {
        const uint32_t id = d.net(b);
        if (b.find('[') != std::string::npos) d.bus_bits.push_back(id);
    }
    std::map<std::string, uint32_t> cell_of;   // one cell per distinct program shape
    d.level_start.push_back(0);
    uint32_t gv = 0;
    for (const auto &lv : in.levels) {
        for (int id : lv) {
            if (id < 0 || (size_t)id >= p.instance_name_vec.size()) {
                if (err) *err = "inter.dat: level list names instance " + std::to_string(id) + " out of range";
                return false;
            }
            auto it = p.instances.find(p.instance_name_vec[id]);
            if (it == p.instances.end()) {
                if (err) *err = "inter.dat: instance " + p.instance_name_vec[id] + " missing";
                return false;
            }
            const ref::Instance &r = it->second;
            const size_t ni = r.in_net.size(), no = r.out_net.size(), nu = r.unknown_out.size();
            // a port left open that a primitive drives becomes an extra
            // output named inst[port]; its internal wire number maps to it
            std::map<int, int> remap;
            for (size_t f = 0; f < r.function_id_vec.size() && f < r.function_vec.size(); ++f) {
                const auto &row = r.function_id_vec[f];
                if (row.empty() || r.function_vec[f].output_pins.empty()) continue;
                const int u = index_of(r.unknown_out, r.function_vec[f].output_pins[0]);
                if ((size_t)u < nu) remap[row.back()] = (int)(ni + no + u);
            }
            Cell c;
            c.name = r.type.name;
            for (size_t k = 0; k < ni; ++k) c.inputs.push_back("i" + std::to_string(k));
            for (size_t k = 0; k < no + nu; ++k) c.outputs.push_back("o" + std::to_string(k));
            std::string sig = c.name + "|" + std::to_string(ni) + "|" + std::to_string(no + nu);
            for (const auto &row : r.function_id_vec) {
                if (row.size() < 2 || row[0] < 0 || row[0] > 9) {
                    if (err) *err = "inter.dat: instance " + r.name + " has a malformed function program";
                    return false;
                }
                Cell::Prim pr;
                pr.func = (uint8_t)row[0];
                sig += "|" + std::to_string(row[0]);
                for (size_t k = 1; k < row.size(); ++k) {
                    int q = row[k];
                    auto rm = remap.find(q);
                    if (rm != remap.end()) q = rm->second;
                    if (q < 0 || q > 31) {
                        if (err) *err = "inter.dat: instance " + r.name + " has a pin number out of range";
                        return false;
                    }
                    pr.pins.push_back((uint8_t)q);
                    sig += "," + std::to_string(q);
                }
                c.prims.push_back(pr);
            }
            auto ci = cell_of.find(sig);
            if (ci == cell_of.end()) {
                ci = cell_of.emplace(sig, (uint32_t)d.cells.size()).first;
                d.cells.push_back(c);
            }
            Instance x;
            x.name = r.name;
            x.cell = ci->second;
            x.gv_index = (uint32_t)id;
            for (auto &nm : r.in_net) x.pins.push_back(d.net(nm));
            for (auto &nm : r.out_net) x.pins.push_back(d.net(nm));
            for (auto &port : r.unknown_out) x.pins.push_back(d.net(r.name + "[" + port + "]"));
            for (size_t k = 0; k < x.pins.size(); ++k) x.conn.push_back((uint32_t)k);
            for (const ref::Delay &dl : r.delays) {
                const int ip = index_of(r.in_net, dl.in_bit);
                int op = index_of(r.out_net, dl.out_bit);
                if ((size_t)op >= no) op = (int)no + index_of(r.unknown_out, dl.out_bit);
                if ((size_t)ip >= ni || (size_t)op >= no + nu || dl.edge < 0 || dl.edge > 2) continue;
                Arc a;
                a.edge = (uint8_t)dl.edge;
                a.in_pin = (uint8_t)ip;
                a.out_pin = (uint8_t)op;
                a.rise = dl.rise;
                a.fall = dl.fall;
                x.arcs.push_back(a);
            }
            d.insts.push_back(std::move(x));
            ++gv;
        }
        d.level_start.push_back((uint32_t)d.insts.size());
    }
    if (gv != p.instances.size() && err) *err = "";   // instances outside every level are not simulated
    for (auto &kv : p.pinbit_values)
        if (!kv.second.empty()) d.constants.push_back({d.net(kv.first), (uint8_t)(kv.second[0].value & 3)});
    for (auto &kv : p.assign_pairs) d.aliases.push_back({d.net(kv.first), d.net(kv.second)});
    for (auto &kv : p.result) d.assign_consts.push_back(d.net(kv.first));
    d.ignored = p.ignored_modules;
    return true;
}

// ------------------------------------------------------- SAIF record order
std::vector<SaifRecord> saif_ref_order(const ref::Inter &in, const VcdDecls &vcd)
{
    const ref::PreProcess &p = in.p;
    std::vector<SaifRecord> recs;
    auto net_rec = [&](const std::string &name, const std::string &src) {
        SaifRecord r;
        r.kind = SaifRecord::kNet;
        r.name = name;
        r.source = src;
        recs.push_back(r);
    };
    // the reader's declared signals (src/VCDParser.cpp:360-450)
    std::unordered_set<std::string> in_bus, in_bit;
    std::unordered_set<std::string> bus_sizes;   // parser.sizes: the bus bit names
    for (auto &b : vcd.bits) {
        if (b.second) {
            in_bus.insert(b.first);
            bus_sizes.insert(b.first);
        } else {
            in_bit.insert(b.first);
        }
    }
    // declared bus bits (src/simulate.cu:1975-1980)
    std::unordered_set<std::string> pin_bits_set;
    for (auto &b : p.pin_bits)
        if (b.find('[') != std::string::npos) pin_bits_set.insert(b);
    auto drop_bit = [&](const std::string &nm) {
        if (nm.find('[') != std::string::npos) pin_bits_set.erase(nm);
    };
    std::unordered_set<std::string> result, other;
    std::vector<std::map<std::string, std::vector<uint32_t>>> out_maps = in.out_maps;
    for (size_t L = 0; L < in.levels.size(); ++L) {
        // first-seen input nets of the level, in instance and pin order
        std::unordered_map<std::string, char> temp;
        for (int id : in.levels[L]) {
            const ref::Instance &r = p.instances.at(p.instance_name_vec[id]);
            for (size_t k = 0; k < r.in_net.size(); ++k) {
                const std::string &nm = r.in_net[k];
                const int from = k < r.from_id.size() ? r.from_id[k] : -1;
                if (from != -2 && !result.count(nm)) {
                    result.insert(nm);
                    temp[nm] = 1;
                }
                if (from == -1) {
                    const std::string &src = k < r.from_info.size() ? r.from_info[k] : nm;
                    if (bus_sizes.count(src)) in_bus.erase(nm);
                    else in_bit.erase(nm);
                } else if (from >= 0 && k < r.from_level.size() && (size_t)r.from_level[k] < out_maps.size()) {
                    out_maps[r.from_level[k]].erase(nm);
                }
            }
        }
        for (auto &kv : temp) {
            drop_bit(kv.first);
            net_rec(kv.first, kv.first);
        }
        if (L + 1 == in.levels.size()) {
            for (auto &kv : p.result) {   // constants (std::map: name order)
                drop_bit(kv.first);
                SaifRecord r;
                r.kind = SaifRecord::kConst;
                r.name = kv.first;
                r.t0 = kv.second.size() > 0 ? kv.second[0] : 0;
                r.t1 = kv.second.size() > 1 ? kv.second[1] : 0;
                recs.push_back(r);
            }
        }
    }
    for (auto &om : out_maps)   // gate outputs no gate reads
        for (auto &kv : om) {
            drop_bit(kv.first);
            net_rec(kv.first, kv.first);
            other.insert(kv.first);
        }
    for (auto *set : {&in_bus, &in_bit})   // stimulus nets no gate reads
        for (auto &nm : *set) {
            drop_bit(nm);
            net_rec(nm, nm);
            other.insert(nm);
        }
    for (auto &kv : p.assign_pairs) {   // assign aliases (std::map: name order)
        const std::string &l = kv.first, &r = kv.second;
        if (result.count(l) || other.count(l) || p.result.count(l)) continue;
        drop_bit(l);
        if (result.count(r) || other.count(r)) {
            net_rec(l, r);
        } else if (p.result.count(r)) {
            SaifRecord c;
            c.kind = SaifRecord::kConst;
            c.name = l;
            const auto &v = p.result.at(r);
            c.t0 = v.size() > 0 ? v[0] : 0;
            c.t1 = v.size() > 1 ? v[1] : 0;
            recs.push_back(c);
        } else {
            SaifRecord u;   // the reference prints the name with no counts
            u.kind = SaifRecord::kNet;
            u.name = l;
            recs.push_back(u);
        }
    }
    for (auto &nm : pin_bits_set) {   // declared bus bits nothing printed
        SaifRecord u;
        u.kind = SaifRecord::kUndriven;
        u.name = nm;
        recs.push_back(u);
    }
    return recs;
}

}  // namespace glsh
