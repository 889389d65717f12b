// Front end of the gls command-line tools: Verilog cell library, flat
// gate-level netlist, SDF, levelization and the inter.dat file.
//
// The parsers follow the subset the reference's front end reads
// (src/PreProcess.cpp: parse_vlib 42-648, parse_gv 650-1274, parse_sdf
// 1276-1464), written as a small tokenizer instead of line splitting, so a
// statement may span lines and carry comments.
#include "design.h"
#include "boost_inter.h"

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <set>
#include <sstream>

namespace glsh {

uint32_t Design::net(const std::string &name)
{
    auto it = net_id.find(name);
    if (it != net_id.end()) return it->second;
    const uint32_t id = (uint32_t)net_names.size();
    net_names.push_back(name);
    net_id.emplace(name, id);
    return id;
}

int Design::find_net(const std::string &name) const
{
    auto it = net_id.find(name);
    return it == net_id.end() ? -1 : (int)it->second;
}

std::string read_file(const std::string &path, std::string *err)
{
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) {
        if (err) *err = "cannot open " + path;
        return std::string();
    }
    // one read into a buffer of the file's size (files reach gigabytes)
    const std::streamoff n = f.tellg();
    std::string s;
    if (n > 0) {
        s.resize((size_t)n);
        f.seekg(0);
        if (!f.read(&s[0], n)) {
            if (err) *err = "cannot read " + path;
            return std::string();
        }
    }
    return s;
}

namespace {

// ------------------------------------------------------------- tokenizer
struct Lexer {
    const std::string &s;
    size_t i = 0;
    explicit Lexer(const std::string &t) : s(t) {}

    void skip_ws()
    {
        for (;;) {
            while (i < s.size() && isspace((unsigned char)s[i])) ++i;
            if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '/') {
                while (i < s.size() && s[i] != '\n') ++i;
                continue;
            }
            if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '*') {
                size_t e = s.find("*/", i + 2);
                i = e == std::string::npos ? s.size() : e + 2;
                continue;
            }
            if (i < s.size() && s[i] == '`') {   // compiler directive: skip the line
                while (i < s.size() && s[i] != '\n') ++i;
                continue;
            }
            break;
        }
    }
    // identifiers (with escaped names), numbers with base (1'b0), single
    // punctuation characters
    bool next(std::string &tok)
    {
        skip_ws();
        if (i >= s.size()) return false;
        const char c = s[i];
        if (c == '\\') {   // escaped identifier runs to white space
            size_t j = i + 1;
            while (j < s.size() && !isspace((unsigned char)s[j])) ++j;
            tok = s.substr(i + 1, j - i - 1);
            i = j;
            return true;
        }
        if (isalnum((unsigned char)c) || c == '_' || c == '$' || c == '\'') {
            size_t j = i;
            while (j < s.size() && (isalnum((unsigned char)s[j]) || s[j] == '_' || s[j] == '$' || s[j] == '\''))
                ++j;
            tok = s.substr(i, j - i);
            i = j;
            return true;
        }
        tok = std::string(1, c);
        ++i;
        return true;
    }
    bool peek(std::string &tok)
    {
        const size_t save = i;
        const bool ok = next(tok);
        i = save;
        return ok;
    }
};

bool block_word(const std::string &t)
{
    return t == "module" || t == "endmodule" || t == "primitive" || t == "endprimitive" || t == "specify" ||
           t == "endspecify" || t == "table" || t == "endtable" || t == "begin" || t == "end";
}

// The next statement: tokens up to and without ';'.  Block keywords
// (module, endmodule, begin, end, ...) also end a statement, so blocks that
// close without a semicolon do not swallow the next declaration.  False at
// end of input.
bool statement(Lexer &L, std::vector<std::string> &toks)
{
    toks.clear();
    std::string t;
    for (;;) {
        const size_t save = L.i;
        if (!L.next(t)) break;
        if (t == ";") return true;
        if (block_word(t)) {
            if (!toks.empty() && t != "module" && t != "primitive" && t != "specify" && t != "table") {
                L.i = save;
                return true;
            }
            if (!toks.empty()) {
                L.i = save;
                return true;
            }
            toks.push_back(t);
            if (t != "module" && t != "primitive") return true;   // a lone keyword statement
            continue;
        }
        toks.push_back(t);
    }
    return !toks.empty();
}

const char *kGateNames[] = {"and", "or", "xor", "xnor", "nor", "nand", "buf", "not"};

int gate_id(const std::string &t)
{
    for (int k = 0; k < 8; ++k)
        if (t == kGateNames[k]) return k;
    if (t == "udp_xbuf") return 8;
    if (t == "udp_mux2") return 9;
    return -1;
}

// ---------------------------------------------------------------- vlib
struct ModBuild {
    Cell cell;
    std::vector<std::string> wires;
    std::set<std::string> sup0, sup1;
    struct P {
        int func;
        std::string out;
        std::vector<std::string> ins;
    };
    std::vector<P> prims;
    bool ignored = false;
};

bool finish_module(ModBuild &m, Library &lib, std::string *err)
{
    if (m.ignored) {
        lib.ignored.push_back(m.cell.name);
        return true;
    }
    Cell &c = m.cell;
    std::vector<std::string> wires;
    auto pin = [&](const std::string &n) -> int {
        if (n == "1'b0" || m.sup0.count(n)) return 16;
        if (n == "1'b1" || m.sup1.count(n)) return 17;
        for (size_t k = 0; k < c.inputs.size(); ++k)
            if (c.inputs[k] == n) return (int)k;
        for (size_t k = 0; k < c.outputs.size(); ++k)
            if (c.outputs[k] == n) return (int)(c.inputs.size() + k);
        for (size_t k = 0; k < wires.size(); ++k)
            if (wires[k] == n) return (int)(c.inputs.size() + c.outputs.size() + k);
        wires.push_back(n);
        return (int)(c.inputs.size() + c.outputs.size() + wires.size() - 1);
    };
    for (auto &p : m.prims) {
        Cell::Prim pr;
        pr.func = (uint8_t)p.func;
        for (auto &n : p.ins) pr.pins.push_back((uint8_t)pin(n));
        pr.pins.push_back((uint8_t)pin(p.out));
        if (c.inputs.size() + c.outputs.size() + wires.size() > 16) {
            if (err) *err = "module " + c.name + ": more than 16 pins and wires";
            return false;
        }
        c.prims.push_back(pr);
    }
    lib.by_name[c.name] = (uint32_t)lib.cells.size();
    lib.cells.push_back(c);
    return true;
}

}  // namespace

bool parse_vlib(const std::string &text, Library &lib, std::string *err)
{
    Lexer L(text);
    std::vector<std::string> st;
    while (statement(L, st)) {
        if (st.empty()) continue;
        if (st[0] == "primitive") {   // UDP definitions: skip to endprimitive
            while (statement(L, st) && !(st.size() == 1 && st[0] == "endprimitive")) {}
            continue;
        }
        if (st[0] != "module") continue;
        if (st.size() < 2) {
            if (err) *err = "module without a name";
            return false;
        }
        ModBuild m;
        m.cell.name = st[1];
        bool done = false;
        while (!done && statement(L, st)) {
            if (st.empty()) continue;
            const std::string &k = st[0];
            if (k == "endmodule") { done = true; break; }
            if (k == "specify") {
                while (statement(L, st) && !(st.size() == 1 && st[0] == "endspecify")) {}
                continue;
            }
            if (k == "input" || k == "output" || k == "inout" || k == "wire" || k == "reg" || k == "supply0" ||
                k == "supply1") {
                size_t a = 1;
                int l = -1, r = -1;
                if (a < st.size() && st[a] == "[") {   // ranges are not used by the cells, only recorded
                    if (a + 3 < st.size()) {
                        l = atoi(st[a + 1].c_str());
                        r = st[a + 2] == ":" ? atoi(st[a + 3].c_str()) : l;
                    }
                    while (a < st.size() && st[a] != "]") ++a;
                    ++a;
                }
                if (k == "supply0") m.cell.sup0_tokens.push_back(k);
                if (k == "supply1") m.cell.sup1_tokens.push_back(k);
                for (; a < st.size(); ++a) {
                    if (st[a] == ",") continue;
                    if (k == "input") m.cell.inputs.push_back(st[a]);
                    else if (k == "output") m.cell.outputs.push_back(st[a]);
                    else if (k == "inout") m.cell.inputs.push_back(st[a]);
                    else if (k == "supply0") { m.sup0.insert(st[a]); m.cell.sup0_tokens.push_back(st[a]); }
                    else if (k == "supply1") { m.sup1.insert(st[a]); m.cell.sup1_tokens.push_back(st[a]); }
                    if (k != "supply0" && k != "supply1") m.cell.decls.push_back({st[a], k, l, r});
                }
                continue;
            }
            if (k == "udp_dff" || k == "udp_tlat" || k == "always") {
                m.ignored = true;
                continue;
            }
            const int f = gate_id(k);
            if (f >= 0) {
                // name? ( out , in , ... )
                size_t a = 1;
                while (a < st.size() && st[a] != "(") ++a;
                std::vector<std::string> args;
                for (++a; a < st.size() && st[a] != ")"; ++a)
                    if (st[a] != ",") args.push_back(st[a]);
                if (args.size() < 2) {
                    if (err) *err = "module " + m.cell.name + ": primitive " + k + " needs an output and inputs";
                    return false;
                }
                ModBuild::P p;
                p.func = f;
                p.out = args[0];
                p.ins.assign(args.begin() + 1, args.end());
                m.prims.push_back(p);
                m.cell.funcs.push_back({k, f, p.ins, p.out});
                continue;
            }
            // other statements (instances of unknown UDPs, tables, ...) are ignored
        }
        if (!finish_module(m, lib, err)) return false;
    }
    return true;
}

// ------------------------------------------------------------------ gv
namespace {

// Expand a port expression into bit nets: name, name[i], name[a:b],
// {e, e, ...}, 1'b0 / 1'b1.  Whole-bus names expand with the declared range.
bool expand(const std::vector<std::string> &t, size_t &a, size_t end, Design &d,
            const std::map<std::string, std::pair<int, int>> &ranges, std::vector<std::string> &bits,
            std::string *err)
{
    if (a >= end) return true;
    if (t[a] == "{") {
        ++a;
        while (a < end && t[a] != "}") {
            if (t[a] == ",") { ++a; continue; }
            if (!expand(t, a, end, d, ranges, bits, err)) return false;
        }
        ++a;
        return true;
    }
    const std::string name = t[a++];
    if (name == "1'b0" || name == "1'b1") {
        bits.push_back(name);
        return true;
    }
    if (a < end && t[a] == "[") {
        int l = atoi(t[a + 1].c_str());
        int r = l;
        a += 2;
        if (a < end && t[a] == ":") {
            r = atoi(t[a + 1].c_str());
            a += 2;
        }
        ++a;   // ]
        if (l == r) bits.push_back(name + "[" + std::to_string(l) + "]");
        else
            for (int k = l;; k += (r > l ? 1 : -1)) {
                bits.push_back(name + "[" + std::to_string(k) + "]");
                if (k == r) break;
            }
        return true;
    }
    auto it = ranges.find(name);
    if (it != ranges.end()) {
        const int l = it->second.first, r = it->second.second;
        for (int k = l;; k += (r > l ? 1 : -1)) {
            bits.push_back(name + "[" + std::to_string(k) + "]");
            if (k == r) break;
        }
        return true;
    }
    bits.push_back(name);
    return true;
}

}  // namespace

bool parse_gv(const std::string &text, const Library &lib, Design &d, std::string *err)
{
    Lexer L(text);
    std::vector<std::string> st;
    std::map<std::string, std::pair<int, int>> ranges;
    std::map<std::string, uint32_t> design_cell;   // library cell -> design cell index
    const uint32_t c0 = d.net("1'b0"), c1 = d.net("1'b1");
    d.constants.push_back({c0, 0});
    d.constants.push_back({c1, 3});
    bool in_module = false;
    std::set<std::string> ignored(lib.ignored.begin(), lib.ignored.end());
    d.ignored = lib.ignored;
    while (statement(L, st)) {
        if (st.empty()) continue;
        const std::string &k = st[0];
        if (k == "module") {
            if (st.size() > 1) d.top = st[1];
            in_module = true;
            continue;
        }
        if (k == "endmodule") break;
        if (!in_module) continue;
        if (k == "input" || k == "output" || k == "wire" || k == "inout") {
            size_t a = 1;
            int l = -1, r = -1;
            if (a < st.size() && st[a] == "[") {
                l = atoi(st[a + 1].c_str());
                r = atoi(st[a + 3].c_str());
                a += 5;
            }
            for (; a < st.size(); ++a) {
                if (st[a] == ",") continue;
                d.decls.push_back({st[a], k, l, r});
                if (l >= 0) {
                    ranges[st[a]] = {l, r};
                    for (int b = l;; b += (r > l ? 1 : -1)) {
                        d.bus_bits.push_back(d.net(st[a] + "[" + std::to_string(b) + "]"));
                        if (b == r) break;
                    }
                } else {
                    d.net(st[a]);
                }
            }
            continue;
        }
        if (k == "assign") {
            size_t eq = 1;
            while (eq < st.size() && st[eq] != "=") ++eq;
            std::vector<std::string> lhs, rhs;
            size_t a = 1;
            if (!expand(st, a, eq, d, ranges, lhs, err)) return false;
            a = eq + 1;
            if (!expand(st, a, st.size(), d, ranges, rhs, err)) return false;
            if (lhs.size() != rhs.size()) {
                if (err) *err = "assign with different widths";
                return false;
            }
            for (size_t b = 0; b < lhs.size(); ++b) {
                const uint32_t ln = d.net(lhs[b]);
                if (rhs[b] == "1'b0") d.constants.push_back({ln, 0});
                else if (rhs[b] == "1'b1") d.constants.push_back({ln, 3});
                else d.aliases.push_back({ln, d.net(rhs[b])});
                if (rhs[b] == "1'b0" || rhs[b] == "1'b1") d.assign_consts.push_back(ln);
            }
            continue;
        }
        // instance:  CELL NAME ( .port(expr), ... )
        if (st.size() < 3) continue;
        auto lit = lib.by_name.find(k);
        if (lit == lib.by_name.end()) {
            if (!ignored.count(k)) fprintf(stderr, "WARNING: skip unknown module %s\n", k.c_str());
            continue;   // sequential cells: their outputs are driven by the stimulus
        }
        const Cell &cell = lib.cells[lit->second];
        Instance in;
        in.name = st[1];
        in.gv_index = (uint32_t)d.insts.size();
        auto dc = design_cell.find(cell.name);
        if (dc == design_cell.end()) {
            dc = design_cell.emplace(cell.name, (uint32_t)d.cells.size()).first;
            d.cells.push_back(cell);
        }
        in.cell = dc->second;
        std::vector<int> pins(cell.inputs.size() + cell.outputs.size(), -1);
        size_t a = 2;
        if (st[a] == "#") {   // parameters are not supported by the cells
            if (err) *err = "instance " + in.name + ": parameters are not supported";
            return false;
        }
        ++a;   // (
        while (a < st.size() && st[a] != ")") {
            if (st[a] == ",") { ++a; continue; }
            if (st[a] != ".") {
                if (err) *err = "instance " + in.name + ": only named port connections are supported";
                return false;
            }
            const std::string port = st[a + 1];
            a += 3;   // . port (
            size_t e = a;
            int depth = 1;
            while (e < st.size()) {
                if (st[e] == "(") ++depth;
                if (st[e] == ")" && --depth == 0) break;
                ++e;
            }
            std::vector<std::string> bits;
            size_t q = a;
            if (!expand(st, q, e, d, ranges, bits, err)) return false;
            a = e + 1;
            int p = -1;
            for (size_t k2 = 0; k2 < cell.inputs.size(); ++k2)
                if (cell.inputs[k2] == port) p = (int)k2;
            for (size_t k2 = 0; k2 < cell.outputs.size(); ++k2)
                if (cell.outputs[k2] == port) p = (int)(cell.inputs.size() + k2);
            if (p < 0) {
                if (err) *err = "instance " + in.name + ": cell " + cell.name + " has no port " + port;
                return false;
            }
            if (bits.size() > 1) {
                if (err) *err = "instance " + in.name + ": multi-bit connection on port " + port;
                return false;
            }
            if (bits.empty()) continue;   // .port() left open
            pins[p] = (int)d.net(bits[0]);
            in.conn.push_back((uint32_t)p);
        }
        for (size_t p = 0; p < pins.size(); ++p) {
            if (pins[p] >= 0) continue;
            if (p < cell.inputs.size()) {
                pins[p] = (int)d.net("gls_open_input");   // reads X, as an unknown net does
            } else {   // an unconnected output keeps a private net, named inst[port] as in the reference
                pins[p] = (int)d.net(in.name + "[" + cell.outputs[p - cell.inputs.size()] + "]");
            }
        }
        for (int p : pins) in.pins.push_back((uint32_t)p);
        d.insts.push_back(in);
    }
    return true;
}

// ----------------------------------------------------------------- sdf
namespace {

struct SNode {
    std::string atom;
    std::vector<SNode> kids;
    bool list = false;
};

bool sparse(const std::string &s, size_t &i, SNode &out)
{
    while (i < s.size() && isspace((unsigned char)s[i])) ++i;
    if (i >= s.size()) return false;
    if (s[i] == '(') {
        out.list = true;
        ++i;
        for (;;) {
            while (i < s.size() && isspace((unsigned char)s[i])) ++i;
            if (i >= s.size()) return false;
            if (s[i] == ')') { ++i; return true; }
            SNode k;
            if (!sparse(s, i, k)) return false;
            out.kids.push_back(std::move(k));
        }
    }
    if (s[i] == '"') {
        size_t j = s.find('"', i + 1);
        if (j == std::string::npos) return false;
        out.atom = s.substr(i + 1, j - i - 1);
        i = j + 1;
        return true;
    }
    size_t j = i;
    while (j < s.size() && !isspace((unsigned char)s[j]) && s[j] != '(' && s[j] != ')') ++j;
    out.atom = s.substr(i, j - i);
    i = j;
    return true;
}

std::string upper(std::string x)
{
    for (auto &c : x) c = (char)toupper((unsigned char)c);
    return x;
}

// (r:t:m) -> the second non-empty field, as the reference's
// Split(value, ":")[1] takes it (src/PreProcess.cpp:1352-1400): the typical
// value, or the max when the typical field is empty; a single value (t) is
// taken as it is.  False when the list is empty.
bool delay_value(const SNode &n, double &v)
{
    if (!n.list || n.kids.empty()) return false;
    const std::string a = n.kids[0].atom;
    std::vector<std::string> f;
    size_t p = 0;
    while (p <= a.size()) {
        size_t q = a.find(':', p);
        if (q == std::string::npos) q = a.size();
        if (q > p) f.push_back(a.substr(p, q - p));
        p = q + 1;
    }
    if (f.empty()) return false;
    v = atof((f.size() >= 2 ? f[1] : f[0]).c_str());
    return true;
}

void walk_iopaths(const SNode &n, std::vector<const SNode *> &out)
{
    if (!n.list) return;
    if (!n.kids.empty() && !n.kids[0].list && upper(n.kids[0].atom) == "IOPATH") {
        out.push_back(&n);
        return;
    }
    for (auto &k : n.kids) walk_iopaths(k, out);
}

}  // namespace

bool parse_sdf(const std::string &text, Design &d, const Library &lib, std::string *err)
{
    (void)lib;
    SNode root;
    size_t i = 0;
    if (!sparse(text, i, root)) {
        if (err) *err = "SDF: malformed S-expression";
        return false;
    }
    double factor = 1.0;   // delays are kept in ps, as the reference does (src/PreProcess.cpp:1277-1318)
    std::unordered_map<std::string, uint32_t> inst_of;
    for (uint32_t k = 0; k < d.insts.size(); ++k) inst_of[d.insts[k].name] = k;
    for (auto &n : root.kids) {
        if (!n.list || n.kids.empty()) continue;
        const std::string head = upper(n.kids[0].atom);
        if (head == "TIMESCALE") {
            std::string ts;
            for (size_t k = 1; k < n.kids.size(); ++k) ts += n.kids[k].atom;
            if (ts == "1ns") factor = 1e3;
            else if (ts == "1ps") factor = 1.0;
            else if (ts == "1us") factor = 1e6;
            else if (ts == "1ms") factor = 1e9;
            else if (ts == "1s") factor = 1e12;
            else if (ts == "100ps") factor = 100.0;
            else if (ts == "10ps") factor = 10.0;
            else fprintf(stderr, "WARNING: SDF timescale %s not supported, using 1ps\n", ts.c_str());
            continue;
        }
        if (head != "CELL") continue;
        std::string iname;
        for (auto &k : n.kids)
            if (k.list && !k.kids.empty() && upper(k.kids[0].atom) == "INSTANCE" && k.kids.size() > 1)
                iname = k.kids[1].atom;
        auto it = inst_of.find(iname);
        if (it == inst_of.end()) continue;   // cells the netlist skipped
        Instance &in = d.insts[it->second];
        const Cell &cell = d.cells[in.cell];
        std::vector<const SNode *> paths;
        walk_iopaths(n, paths);
        for (const SNode *p : paths) {
            // (IOPATH in out (r) (f)) or (IOPATH (posedge in) out (r) (f))
            if (p->kids.size() < 4) continue;
            Arc arc;
            std::string port;
            const SNode &src = p->kids[1];
            if (src.list) {
                if (src.kids.size() < 2) continue;
                const std::string e = upper(src.kids[0].atom);
                arc.edge = e == "POSEDGE" ? 0 : (e == "NEGEDGE" ? 1 : 2);
                port = src.kids[1].atom;
            } else {
                arc.edge = 2;
                port = src.atom;
            }
            const std::string oport = p->kids[2].atom;
            int ip = -1, op = -1;
            for (size_t k = 0; k < cell.inputs.size(); ++k)
                if (cell.inputs[k] == port) ip = (int)k;
            for (size_t k = 0; k < cell.outputs.size(); ++k)
                if (cell.outputs[k] == oport) op = (int)k;
            if (ip < 0 || op < 0) continue;   // the reference leaves such arcs unmatched
            double r = 0, f = 0;
            if (!delay_value(p->kids[3], r)) continue;
            f = r;
            if (p->kids.size() > 4) delay_value(p->kids[4], f);
            arc.in_pin = (uint8_t)ip;
            arc.out_pin = (uint8_t)op;
            arc.rise = r * factor;
            arc.fall = f * factor;
            in.arcs.push_back(arc);
        }
    }
    return true;
}

// ------------------------------------------------------------- levelize
// Kahn levels as TopologyOrder computes them (src/process.cpp:90-176):
// an edge runs from an instance to every instance reading one of its
// output nets; each level takes, in instance order, every instance whose
// predecessors are all placed.  Reads through assign aliases count.
void instance_preds(const Design &d, std::vector<uint64_t> &start, std::vector<uint32_t> &pred)
{
    const size_t n = d.insts.size();
    std::vector<uint32_t> alias_to(d.net_names.size());
    for (uint32_t k = 0; k < alias_to.size(); ++k) alias_to[k] = k;
    for (auto &a : d.aliases) alias_to[a.first] = a.second;
    auto resolve = [&](uint32_t net) {
        for (int hop = 0; hop < 64 && alias_to[net] != net; ++hop) net = alias_to[net];
        return net;
    };
    std::vector<int> driver(d.net_names.size(), -1);
    for (size_t i = 0; i < n; ++i) {
        const Cell &c = d.cells[d.insts[i].cell];
        for (size_t o = 0; o < c.outputs.size(); ++o) driver[d.insts[i].pins[c.inputs.size() + o]] = (int)i;
    }
    start.assign(1, 0);
    pred.clear();
    std::vector<uint32_t> ps;
    for (size_t i = 0; i < n; ++i) {
        const Cell &c = d.cells[d.insts[i].cell];
        ps.clear();
        for (size_t p = 0; p < c.inputs.size(); ++p) {
            const int drv = driver[resolve(d.insts[i].pins[p])];
            if (drv >= 0) ps.push_back((uint32_t)drv);
        }
        std::sort(ps.begin(), ps.end());
        ps.erase(std::unique(ps.begin(), ps.end()), ps.end());
        pred.insert(pred.end(), ps.begin(), ps.end());
        start.push_back(pred.size());
    }
}

void apply_levels(Design &d, const std::vector<uint32_t> &order, const std::vector<uint32_t> &level_start)
{
    std::vector<Instance> sorted;
    sorted.reserve(order.size());
    for (uint32_t i : order) sorted.push_back(std::move(d.insts[i]));
    d.insts = std::move(sorted);
    d.level_start = level_start;
}

bool levelize(Design &d, std::string *err)
{
    const size_t n = d.insts.size();
    std::vector<uint64_t> start;
    std::vector<uint32_t> pred;
    instance_preds(d, start, pred);
    // successors and in-degrees, then one frontier per level
    std::vector<uint64_t> sstart(n + 1, 0);
    for (uint32_t p : pred) ++sstart[p + 1];
    for (size_t i = 0; i < n; ++i) sstart[i + 1] += sstart[i];
    std::vector<uint32_t> succ(pred.size());
    std::vector<uint64_t> fill(sstart.begin(), sstart.end() - 1);
    std::vector<uint32_t> indeg(n);
    for (size_t i = 0; i < n; ++i) {
        indeg[i] = (uint32_t)(start[i + 1] - start[i]);
        for (uint64_t e = start[i]; e < start[i + 1]; ++e) succ[fill[pred[e]]++] = (uint32_t)i;
    }
    std::vector<uint32_t> order, level_start(1, 0), q;
    order.reserve(n);
    for (size_t i = 0; i < n; ++i)
        if (indeg[i] == 0) q.push_back((uint32_t)i);
    while (!q.empty()) {
        order.insert(order.end(), q.begin(), q.end());
        level_start.push_back((uint32_t)order.size());
        std::vector<uint32_t> next;
        for (uint32_t i : q)
            for (uint64_t e = sstart[i]; e < sstart[i + 1]; ++e)
                if (--indeg[succ[e]] == 0) next.push_back(succ[e]);
        std::sort(next.begin(), next.end());   // a level in instance order
        q.swap(next);
    }
    if (order.size() < n) {
        if (err) *err = "combinational loop: the netlist cannot be levelized";
        return false;
    }
    apply_levels(d, order, level_start);
    return true;
}

// --------------------------------------------------------------- inter.dat
// Native binary inter.dat: "GLSINTR1" then length-prefixed sections.
namespace {

struct W {
    std::string b;
    void u8(uint8_t x) { b.push_back((char)x); }
    void u32(uint32_t x) { b.append(reinterpret_cast<const char *>(&x), 4); }
    void f64(double x) { b.append(reinterpret_cast<const char *>(&x), 8); }
    void str(const std::string &s)
    {
        u32((uint32_t)s.size());
        b += s;
    }
};

struct R {
    const std::string &b;
    size_t i = 0;
    bool ok = true;
    explicit R(const std::string &x) : b(x) {}
    bool need(size_t n)
    {
        if (i + n > b.size()) ok = false;
        return ok;
    }
    uint8_t u8()
    {
        if (!need(1)) return 0;
        return (uint8_t)b[i++];
    }
    uint32_t u32()
    {
        uint32_t x = 0;
        if (!need(4)) return 0;
        memcpy(&x, b.data() + i, 4);
        i += 4;
        return x;
    }
    double f64()
    {
        double x = 0;
        if (!need(8)) return 0;
        memcpy(&x, b.data() + i, 8);
        i += 8;
        return x;
    }
    std::string str()
    {
        const uint32_t n = u32();
        if (!need(n)) return std::string();
        std::string s = b.substr(i, n);
        i += n;
        return s;
    }
};

}  // namespace

bool write_inter(const std::string &path, const Design &d, std::string *err)
{
    W w;
    w.b = "GLSINTR1";
    w.str(d.top);
    w.u32((uint32_t)d.net_names.size());
    for (auto &s : d.net_names) w.str(s);
    w.u32((uint32_t)d.cells.size());
    for (auto &c : d.cells) {
        w.str(c.name);
        w.u32((uint32_t)c.inputs.size());
        for (auto &s : c.inputs) w.str(s);
        w.u32((uint32_t)c.outputs.size());
        for (auto &s : c.outputs) w.str(s);
        w.u32((uint32_t)c.prims.size());
        for (auto &p : c.prims) {
            w.u8(p.func);
            w.u8((uint8_t)p.pins.size());
            for (uint8_t q : p.pins) w.u8(q);
        }
    }
    w.u32((uint32_t)d.insts.size());
    for (auto &in : d.insts) {
        w.str(in.name);
        w.u32(in.cell);
        w.u32((uint32_t)in.pins.size());
        for (uint32_t p : in.pins) w.u32(p);
        w.u32((uint32_t)in.arcs.size());
        for (auto &a : in.arcs) {
            w.u8(a.edge);
            w.u8(a.in_pin);
            w.u8(a.out_pin);
            w.f64(a.rise);
            w.f64(a.fall);
        }
    }
    w.u32((uint32_t)d.level_start.size());
    for (uint32_t x : d.level_start) w.u32(x);
    w.u32((uint32_t)d.constants.size());
    for (auto &c : d.constants) {
        w.u32(c.first);
        w.u8(c.second);
    }
    w.u32((uint32_t)d.aliases.size());
    for (auto &a : d.aliases) {
        w.u32(a.first);
        w.u32(a.second);
    }
    w.u32((uint32_t)d.bus_bits.size());
    for (uint32_t x : d.bus_bits) w.u32(x);
    std::ofstream f(path, std::ios::binary);
    if (!f) {
        if (err) *err = "cannot write " + path;
        return false;
    }
    f.write(w.b.data(), (std::streamsize)w.b.size());
    return (bool)f;
}

bool read_inter(const std::string &path, Design &d, std::string *err)
{
    std::string e2;
    const std::string b = read_file(path, &e2);
    if (b.empty()) {
        if (err) *err = e2.empty() ? "empty " + path : e2;
        return false;
    }
    if (is_boost_text_archive(b)) {   // the reference's own format
        ref::Inter in;
        return load_boost_inter(b, in, err) && ref_inter_to_design(in, d, err);
    }
    if (b.compare(0, 8, "GLSINTR1") != 0) {
        if (err) *err = path + " is neither a gls inter.dat nor a Boost text archive";
        return false;
    }
    R r(b);
    r.i = 8;
    d = Design();
    d.top = r.str();
    const uint32_t nn = r.u32();
    for (uint32_t k = 0; k < nn && r.ok; ++k) d.net(r.str());
    const uint32_t nc = r.u32();
    for (uint32_t k = 0; k < nc && r.ok; ++k) {
        Cell c;
        c.name = r.str();
        const uint32_t ni = r.u32();
        for (uint32_t q = 0; q < ni && r.ok; ++q) c.inputs.push_back(r.str());
        const uint32_t no = r.u32();
        for (uint32_t q = 0; q < no && r.ok; ++q) c.outputs.push_back(r.str());
        const uint32_t np = r.u32();
        for (uint32_t q = 0; q < np && r.ok; ++q) {
            Cell::Prim p;
            p.func = r.u8();
            const uint8_t k2 = r.u8();
            for (uint8_t z = 0; z < k2; ++z) p.pins.push_back(r.u8());
            c.prims.push_back(p);
        }
        d.cells.push_back(c);
    }
    const uint32_t ni = r.u32();
    for (uint32_t k = 0; k < ni && r.ok; ++k) {
        Instance in;
        in.name = r.str();
        in.cell = r.u32();
        const uint32_t np = r.u32();
        for (uint32_t q = 0; q < np && r.ok; ++q) in.pins.push_back(r.u32());
        const uint32_t na = r.u32();
        for (uint32_t q = 0; q < na && r.ok; ++q) {
            Arc a;
            a.edge = r.u8();
            a.in_pin = r.u8();
            a.out_pin = r.u8();
            a.rise = r.f64();
            a.fall = r.f64();
            in.arcs.push_back(a);
        }
        if (in.cell >= d.cells.size()) r.ok = false;
        d.insts.push_back(in);
    }
    const uint32_t nl = r.u32();
    for (uint32_t k = 0; k < nl && r.ok; ++k) d.level_start.push_back(r.u32());
    const uint32_t ncst = r.u32();
    for (uint32_t k = 0; k < ncst && r.ok; ++k) {
        const uint32_t net = r.u32();
        d.constants.push_back({net, r.u8()});
    }
    const uint32_t nal = r.u32();
    for (uint32_t k = 0; k < nal && r.ok; ++k) {
        const uint32_t a = r.u32();
        d.aliases.push_back({a, r.u32()});
    }
    const uint32_t nb = r.u32();
    for (uint32_t k = 0; k < nb && r.ok; ++k) d.bus_bits.push_back(r.u32());
    if (!r.ok) {
        if (err) *err = path + ": truncated or corrupt inter.dat";
        return false;
    }
    return true;
}

}  // namespace glsh
