// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own serial simulator core -- SimulateInst, Process,
// Calculate, AddDelay, CheckDelay, RunFunction, GetValueAt, calc and the CPU
// DumpSaif of src/simulate.cpp:37-1506, compiled from the reference sources
// by oracle/build.py -- on a case file (oracle/casefile.py), with the
// level loop of src/simulate.cpp:1569-1668.
//
// The reference's `main` does not compile against its own VCDParser, so this
// driver replaces it: it builds the Instance objects that `process` would
// have archived (names n<id> for nets, U<i> for instances), feeds every
// instance the change lists of its input nets, and writes the output
// waveforms plus the reference's SAIF file.
//
// usage: ref_sim <case> <result> <saif_out> [--calc fixed|literal]
//                [--threads N] [--repeat R]
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <thread>
#include "simulate.h"

// defined in the extracted core (src/simulate.cpp)
void SimulateInst(Instance inst, std::map<std::string, TimedValues*> bitValues,
                  std::unordered_map<std::string, TimedValues*>& _out_value, VCDTimeUnit time_unit);
void DumpSaif(std::unordered_map<std::string, TimedValues*> val_map,
              std::unordered_map<std::string, TimedValues*> out_value,
              std::map<std::string, TimedValues> pinbitValues, std::string saif_out,
              VCDTimeUnit time_unit, unsigned time_res, std::string root_name, VCDTime start, VCDTime end);
// the shipped calc of src/simulate.cpp:382, renamed by the extraction recipe
void gls_ref_calc_literal(std::string name, std::vector<VCDBit> input_data, VCDBit &output_data);

static bool g_literal = false;

// 4-state Verilog primitive semantics (the ref-fixed mode): Z reads as X.
static VCDBit fixed_calc(const std::string &name, const std::vector<VCDBit> &in)
{
    bool any0 = false, any1 = false, anyx = false;
    int par = 0;
    for (VCDBit b : in) {
        if (b == VCD_0) any0 = true;
        else if (b == VCD_1) { any1 = true; par ^= 1; }
        else anyx = true;
    }
    if (name == "and") return any0 ? VCD_0 : anyx ? VCD_X : VCD_1;
    if (name == "nand") return any0 ? VCD_1 : anyx ? VCD_X : VCD_0;
    if (name == "or") return any1 ? VCD_1 : anyx ? VCD_X : VCD_0;
    if (name == "nor") return any1 ? VCD_0 : anyx ? VCD_X : VCD_1;
    if (name == "xor") return anyx ? VCD_X : (par ? VCD_1 : VCD_0);
    if (name == "xnor") return anyx ? VCD_X : (par ? VCD_0 : VCD_1);
    if (name == "buf") return (in[0] == VCD_0 || in[0] == VCD_1) ? in[0] : VCD_X;
    if (name == "not") return in[0] == VCD_0 ? VCD_1 : in[0] == VCD_1 ? VCD_0 : VCD_X;
    if (name == "udp_xbuf") {
        if (in.size() != 2 || in[1] != VCD_1) return VCD_X;
        return in[0] == VCD_0 ? VCD_0 : VCD_1;
    }
    if (name == "udp_mux2") {
        if (in.size() != 3) return VCD_X;
        bool a01 = in[0] == VCD_0 || in[0] == VCD_1, b01 = in[1] == VCD_0 || in[1] == VCD_1;
        if (in[2] == VCD_0) return a01 ? in[0] : VCD_X;
        if (in[2] == VCD_1) return b01 ? in[1] : VCD_X;
        return (a01 && in[0] == in[1]) ? in[0] : VCD_X;
    }
    return VCD_X;
}

void calc(std::string name, std::vector<VCDBit> input_data, VCDBit &output_data)
{
    if (g_literal) gls_ref_calc_literal(name, input_data, output_data);
    else output_data = fixed_calc(name, input_data);
}

static const char *kFuncName[] = {"and", "or", "xor", "xnor", "nor", "nand", "buf", "not", "udp_xbuf", "udp_mux2"};

struct CellRec {
    int n_in, n_out;
    std::vector<std::pair<int, std::vector<int>>> prims;
};

static FILE *g_in;
static void rd(void *p, size_t n)
{
    if (fread(p, 1, n, g_in) != n) { fprintf(stderr, "ref_sim: truncated case\n"); exit(2); }
}
template <typename T> static T rdv() { T x; rd(&x, sizeof x); return x; }

static std::string net_name(uint32_t n) { return "n" + std::to_string(n); }

int main(int argc, char **argv)
{
    if (argc < 4) { fprintf(stderr, "usage: ref_sim <case> <result> <saif> [--calc fixed|literal] [--threads N] [--repeat R]\n"); return 2; }
    int threads = 1, repeat = 1;
    for (int i = 4; i < argc; ++i) {
        if (!strcmp(argv[i], "--calc") && i + 1 < argc) g_literal = !strcmp(argv[++i], "literal");
        else if (!strcmp(argv[i], "--threads") && i + 1 < argc) threads = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--repeat") && i + 1 < argc) repeat = atoi(argv[++i]);
    }
    g_in = fopen(argv[1], "rb");
    if (!g_in) { fprintf(stderr, "ref_sim: cannot open case\n"); return 2; }
    char magic[8];
    rd(magic, 8);
    if (memcmp(magic, "GLSCASE1", 8)) { fprintf(stderr, "ref_sim: bad magic\n"); return 2; }
    uint32_t n_nets = rdv<uint32_t>();
    uint32_t n_cells = rdv<uint32_t>();
    std::vector<CellRec> cells(n_cells);
    for (auto &c : cells) {
        c.n_in = rdv<uint8_t>(); c.n_out = rdv<uint8_t>();
        int np = rdv<uint8_t>();
        for (int p = 0; p < np; ++p) {
            int f = rdv<uint8_t>(), n = rdv<uint8_t>();
            std::vector<int> pins(n);
            for (int k = 0; k < n; ++k) pins[k] = rdv<uint8_t>();
            c.prims.push_back({f, pins});
        }
    }
    uint32_t n_inst = rdv<uint32_t>();
    std::vector<Instance> insts(n_inst);
    std::vector<uint32_t> level(n_inst);
    for (uint32_t i = 0; i < n_inst; ++i) {
        uint32_t cid = rdv<uint32_t>();
        level[i] = rdv<uint32_t>();
        const CellRec &c = cells[cid];
        Instance &in = insts[i];
        in.name = "U" + std::to_string(i);
        std::vector<uint32_t> pins(c.n_in + c.n_out);
        for (auto &p : pins) p = rdv<uint32_t>();
        for (int k = 0; k < c.n_in; ++k) in.in_net.push_back(net_name(pins[k]));
        for (int k = 0; k < c.n_out; ++k) in.out_net.push_back(net_name(pins[c.n_in + k]));
        in.type.name = "cell" + std::to_string(cid);
        in.type.supply1_vec.push_back("gls_supply1");
        in.type.supply0_vec.push_back("gls_supply0");
        // function program with pins renamed as parse_gv does (src/PreProcess.cpp:1199-1263)
        std::vector<Function> fv;
        for (auto &pr : c.prims) {
            Function f(kFuncName[pr.first], pr.first);
            for (size_t k = 0; k < pr.second.size(); ++k) {
                int q = pr.second[k];
                std::string nm;
                if (q < c.n_in) nm = in.in_net[q];
                else if (q < c.n_in + c.n_out) nm = in.out_net[q - c.n_in];
                else if (q == 16) nm = "gls_supply0";
                else if (q == 17) nm = "gls_supply1";
                else nm = "gls_w" + std::to_string(q);
                if (k + 1 < pr.second.size()) f.set_in(nm); else f.set_out(nm);
            }
            fv.push_back(f);
        }
        in.set_function(fv);
        uint16_t na = rdv<uint16_t>();
        for (int a = 0; a < na; ++a) {
            Delay d;
            d.edge = rdv<uint8_t>();
            int ip = rdv<uint8_t>(), op = rdv<uint8_t>();
            (void)rdv<uint8_t>();
            d.rise_val = rdv<double>();
            d.fall_val = rdv<double>();
            d.in_bit = in.in_net[ip];
            d.out_bit = in.out_net[op];
            in.set_delay(d);
        }
    }
    uint32_t n_stim = rdv<uint32_t>();
    std::unordered_map<std::string, TimedValues*> val_map;
    std::vector<uint32_t> stim_nets;
    for (uint32_t s = 0; s < n_stim; ++s) {
        uint32_t net = rdv<uint32_t>(), n = rdv<uint32_t>();
        std::vector<uint64_t> t(n);
        std::vector<uint8_t> v(n);
        if (n) { rd(t.data(), 8 * n); rd(v.data(), n); }
        TimedValues *tv = new TimedValues();
        for (uint32_t e = 0; e < n; ++e) tv->push_back(TimedValue{t[e], (VCDBit)v[e]});
        val_map[net_name(net)] = tv;
        stim_nets.push_back(net);
    }
    uint64_t t_begin = rdv<uint64_t>(), t_end = rdv<uint64_t>();
    fclose(g_in);

    std::unordered_map<std::string, TimedValues*> out_value;
    auto t0 = std::chrono::steady_clock::now();
    for (int rep = 0; rep < repeat; ++rep) {
        out_value.clear();
        uint32_t i = 0;
        while (i < n_inst) {
            uint32_t j = i;
            while (j < n_inst && level[j] == level[i]) ++j;
            // bitValues of every instance of the level (src/simulate.cpp:1617-1664)
            std::vector<std::map<std::string, TimedValues*>> bv(j - i);
            for (uint32_t k = i; k < j; ++k)
                for (const std::string &nm : insts[k].in_net) {
                    auto it = val_map.find(nm);
                    if (it != val_map.end()) bv[k - i][nm] = it->second;
                    else {
                        auto jt = out_value.find(nm);
                        if (jt == out_value.end()) { fprintf(stderr, "ref_sim: net %s has no waveform\n", nm.c_str()); return 3; }
                        bv[k - i][nm] = jt->second;
                    }
                }
            int nt = std::max(1, std::min<int>(threads, (int)(j - i)));
            std::vector<std::unordered_map<std::string, TimedValues*>> local(nt);
            std::atomic<uint32_t> next(i);
            auto work = [&](int tid) {
                for (;;) {
                    uint32_t k = next++;
                    if (k >= j) break;
                    SimulateInst(insts[k], bv[k - i], local[tid], TIME_PS);
                }
            };
            std::vector<std::thread> th;
            for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
            work(0);
            for (auto &t : th) t.join();
            for (auto &m : local) for (auto &kv : m) out_value[kv.first] = kv.second;
            i = j;
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    fprintf(stderr, "ref_sim: simulate %.6f s\n", std::chrono::duration<double>(t1 - t0).count());

    FILE *f = fopen(argv[2], "wb");
    if (!f) return 2;
    fwrite("GLSRES01", 1, 8, f);
    fwrite(&n_nets, 4, 1, f);
    for (uint32_t n = 0; n < n_nets; ++n) {
        std::string nm = net_name(n);
        TimedValues *tv = nullptr;
        auto it = val_map.find(nm);
        if (it != val_map.end()) tv = it->second;
        else {
            auto jt = out_value.find(nm);
            if (jt != out_value.end()) tv = jt->second;
        }
        uint64_t cnt = tv ? tv->size() : UINT64_MAX;
        fwrite(&cnt, 8, 1, f);
        if (!tv) continue;
        for (auto &e : *tv) { uint64_t t = e.t; fwrite(&t, 8, 1, f); }
        for (auto &e : *tv) { uint8_t v = (uint8_t)e.value; fwrite(&v, 1, 1, f); }
    }
    for (uint32_t n = 0; n < n_nets; ++n) {
        uint64_t r[3] = {UINT64_MAX, UINT64_MAX, UINT64_MAX};
        fwrite(r, 8, 3, f);   // SAIF comes from the reference's own DumpSaif file
    }
    fclose(f);
    std::map<std::string, TimedValues> pinbit;
    DumpSaif(val_map, out_value, pinbit, argv[3], TIME_PS, 1, "root", t_begin, t_end);
    return 0;
}
