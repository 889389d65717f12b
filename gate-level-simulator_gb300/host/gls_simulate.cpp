// gls_simulate <inter.dat> <vcd|stim> <dumpon_time> <dumpoff_time> <out.saif>
//              [--calc fixed|literal] [--device N] [--host-vcd]
//              [--saif-order=ref|net]
//
// The `simulate` step of the reference (src/simulate.cu:1786-3315) on
// libgls: read the levelized design (the reference's Boost text archive or
// the tools' native inter.dat) and the VCD stimulus, simulate every level on
// the GPU, write T0 / T1 / TX of every net over [dumpon_time, dumpoff_time)
// as SAIF.  Times are in the VCD time unit.
//
// Net coverage follows the reference GPU tool: nets read by gates and VCD
// nets, gate outputs, constants, assign aliases (with their source's
// counts) and declared bus bits nothing drives (all X).  By default records
// are written in net order; --saif-order=ref writes them in the order (and
// with the coverage and ending) of the reference GPU tool, whose hash
// containers it replays (host/boost_inter.cpp, saif_ref_order).
//
// The VCD body is scanned on the GPU (gls_vcd_scan) unless --host-vcd is
// given; both read the same changes.  A binary stimulus file written by
// gls_vcd2stim (it starts "GLSSTIM1") may stand in for the VCD: its change
// lists are loaded as they are.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include "boost_inter.h"
#include "design.h"
#include "gls.h"
#include "vcd.h"

using namespace glsh;

namespace {

// T0 / T1 / TX of a change list over (start, end] from X, as the reference
// integrates a VCD signal (src/simulate.cu:265-330)
void saif_of_changes(const std::vector<uint64_t> &t, const std::vector<uint8_t> &v, uint64_t start, uint64_t end,
                     uint64_t c[3])
{
    uint64_t acc[4] = {0, 0, 0, 0};   // by value: 0, X, Z, 1
    uint64_t last = start;
    uint8_t state = 1;
    for (size_t k = 0; k < t.size(); ++k) {
        if (t[k] <= start) {
            state = v[k];
            continue;
        }
        if (t[k] > end) break;
        acc[state & 3] += t[k] - last;
        last = t[k];
        state = v[k];
    }
    if (last < end) acc[state & 3] += end - last;
    c[0] = acc[0];
    c[1] = acc[3];
    c[2] = acc[1] + acc[2];
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 6) {
        printf("[USAGE] ./gls_simulate [intermediate_file] vcd_path dumpon_time(ps) dumpoff_time(ps) saif_out\n");
        return 255;
    }
    int calc = GLS_CALC_FIXED, device = 0;
    bool host_vcd = false, ref_order = false;
    for (int k = 6; k < argc; ++k) {
        if (!strcmp(argv[k], "--calc") && k + 1 < argc) calc = !strcmp(argv[++k], "literal") ? GLS_CALC_LITERAL : GLS_CALC_FIXED;
        else if (!strcmp(argv[k], "--device") && k + 1 < argc) device = atoi(argv[++k]);
        else if (!strcmp(argv[k], "--host-vcd")) host_vcd = true;
        else if (!strcmp(argv[k], "--saif-order=ref")) ref_order = true;
        else if (!strcmp(argv[k], "--saif-order=net")) ref_order = false;
    }
    std::ofstream outf(argv[5]);
    if (!outf) {
        printf("File %s Open Error!\nExit!\n", argv[5]);
        return 255;
    }
    const unsigned long long t_begin = strtoull(argv[3], nullptr, 10), t_end = strtoull(argv[4], nullptr, 10);
    if (t_end <= t_begin) {
        printf("dumpoff_time must be greater than dumpon_time\n");
        return 255;
    }
    using clk = std::chrono::steady_clock;
    const auto t_start = clk::now();
    auto ms_since = [](clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); };
    std::string err;
    Design d;
    ref::Inter archived;   // the reference's content of the design (for --saif-order=ref)
    {
        const std::string bytes = read_file(argv[1], &err);
        bool ok;
        if (is_boost_text_archive(bytes)) {
            ok = load_boost_inter(bytes, archived, &err) && ref_inter_to_design(archived, d, &err);
        } else {
            ok = read_inter(argv[1], d, &err);
            if (ok && ref_order) design_to_ref_inter(d, Library(), archived);
        }
        if (!ok) {
            printf("ERROR: %s\n", err.c_str());
            return 255;
        }
    }
    const double ms_design = ms_since(t_start);
    const auto t_vcd = clk::now();
    VcdData vcd;
    const std::string vtext = read_file(argv[2], &err);
    if (vtext.empty() ||
        (is_stim_bin(vtext) ? !load_stim_bin(vtext, vcd, &err)
                            : (host_vcd ? !parse_vcd(vtext, vcd, &err) : parse_vcd_gpu(vtext, vcd, &err, device) < 0))) {
        printf("Parse Failed. %s\n", err.c_str());
        return 1;
    }
    const uint32_t n_nets = (uint32_t)d.net_names.size();
    // assign aliases: a read of the left side reads the right side
    std::vector<uint32_t> alias_to(n_nets);
    for (uint32_t k = 0; k < n_nets; ++k) alias_to[k] = k;
    for (auto &a : d.aliases) alias_to[a.first] = a.second;
    auto resolve = [&](uint32_t n) {
        for (int hop = 0; hop < 64 && alias_to[n] != n; ++hop) n = alias_to[n];
        return n;
    };
    // the C ABI netlist
    std::vector<gls_cell> cells;
    std::vector<gls_prim> prims;
    for (auto &c : d.cells) {
        gls_cell gc;
        memset(&gc, 0, sizeof gc);
        gc.n_in = (uint8_t)c.inputs.size();
        gc.n_out = (uint8_t)c.outputs.size();
        gc.n_prim = (uint8_t)c.prims.size();
        gc.prim_start = (uint32_t)prims.size();
        for (auto &p : c.prims) {
            gls_prim gp;
            memset(&gp, 0, sizeof gp);
            gp.func = p.func;
            gp.n_pins = (uint8_t)p.pins.size();
            for (size_t q = 0; q < p.pins.size() && q < 14; ++q) gp.pins[q] = p.pins[q];
            prims.push_back(gp);
        }
        cells.push_back(gc);
    }
    if (prims.empty()) prims.push_back(gls_prim{});
    std::vector<uint32_t> inst_cell, pin_start(1, 0), pin_net, arc_start(1, 0);
    std::vector<gls_arc> arcs;
    std::vector<uint8_t> driven(n_nets, 0), read(n_nets, 0);
    for (auto &in : d.insts) {
        const Cell &c = d.cells[in.cell];
        inst_cell.push_back(in.cell);
        for (size_t p = 0; p < in.pins.size(); ++p) {
            uint32_t net = in.pins[p];
            if (p < c.inputs.size()) {
                net = resolve(net);
                read[net] = 1;
            } else {
                driven[net] = 1;
            }
            pin_net.push_back(net);
        }
        pin_start.push_back((uint32_t)pin_net.size());
        for (auto &a : in.arcs) {
            gls_arc ga;
            memset(&ga, 0, sizeof ga);
            ga.edge = a.edge;
            ga.in_pin = a.in_pin;
            ga.out_pin = a.out_pin;
            ga.rise = a.rise;
            ga.fall = a.fall;
            arcs.push_back(ga);
        }
        arc_start.push_back((uint32_t)arcs.size());
    }
    if (arcs.empty()) arcs.push_back(gls_arc{});
    gls_netlist nl = {n_nets, (uint32_t)cells.size(), cells.data(), (uint32_t)prims.size(), prims.data(),
                      (uint32_t)inst_cell.size(), (uint32_t)(d.level_start.size() - 1), d.level_start.data(),
                      inst_cell.data(), pin_start.data(), pin_net.data(), arc_start.data(), arcs.data()};
    // stimulus: VCD nets (not driven by a gate) and constants
    std::vector<int8_t> constant(n_nets, -1);
    for (auto &c : d.constants) constant[c.first] = (int8_t)c.second;
    std::vector<uint32_t> st_net;
    std::vector<uint64_t> st_start(1, 0);
    std::vector<uint32_t> st_time;
    std::vector<uint8_t> st_val;
    std::vector<uint8_t> in_stim(n_nets, 0);
    for (uint32_t n = 0; n < n_nets; ++n) {
        if (driven[n]) continue;
        auto it = vcd.index.find(d.net_names[n]);
        if (it != vcd.index.end()) {
            const auto &tt = vcd.times[it->second];
            const auto &vv = vcd.values[it->second];
            for (size_t e = 0; e < tt.size(); ++e) {
                if (tt[e] > (1u << 30) - 2) {
                    printf("ERROR: VCD time %llu of %s exceeds 2^30-2\n", (unsigned long long)tt[e], d.net_names[n].c_str());
                    return 255;
                }
                st_time.push_back((uint32_t)tt[e]);
                st_val.push_back(vv[e]);
            }
        } else if (constant[n] >= 0) {
            st_time.push_back(0);
            st_val.push_back((uint8_t)constant[n]);
        } else if (read[n]) {
            printf("error: net %s has no waveform (neither VCD, gate output nor constant)\n", d.net_names[n].c_str());
            return 255;
        } else {
            continue;
        }
        st_net.push_back(n);
        st_start.push_back(st_time.size());
        in_stim[n] = 1;
    }
    gls_stimulus st = {(uint32_t)st_net.size(), st_net.data(), st_start.data(), st_time.data(), st_val.data()};
    gls_opts o;
    memset(&o, 0, sizeof o);
    o.device = device;
    o.calc_mode = calc;
    o.delay_factor = 1.0;
    gls_ctx *ctx = nullptr;
    int rc = gls_create(&o, &ctx);
    if (rc) {
        printf("ERROR: no usable CUDA device (gls_create %d)\n", rc);
        return 255;
    }
    const double ms_stim = ms_since(t_vcd);
    const auto t_run = clk::now();
    uint32_t win = 0;
    if ((rc = gls_load_netlist(ctx, &nl)) || (rc = gls_add_window(ctx, &st, t_begin, t_end, &win)) || (rc = gls_run(ctx))) {
        printf("ERROR: %s\n", gls_last_error(ctx));
        gls_destroy(ctx);
        return 255;
    }
    std::vector<uint64_t> t0(n_nets), t1(n_nets), tx(n_nets);
    gls_saif_counts(ctx, win, t0.data(), t1.data(), tx.data());
    gls_stats stats;
    gls_stats_get(ctx, &stats);
    gls_destroy(ctx);
    const double ms_run = ms_since(t_run);
    const auto t_saif = clk::now();
    // SAIF text, format of src/simulate.cu:457-481
    const unsigned long long dur = t_end - t_begin;
    outf << "(TIMESCALE " << vcd.time_res << " " << vcd.time_unit << ")\n";
    outf << "(DURATION " << dur << ")\n";
    outf << "(INSTANCE root\n   (NET\n";
    auto rec = [&](const std::string &name, uint64_t a, uint64_t b, uint64_t c, const char *ind) {
        outf << ind << "(" << name << "\n" << ind << "   (T0 " << a << ") (T1 " << b << ") (TX " << c << ")\n" << ind << ")\n";
    };
    if (ref_order) {
        // the records in the reference GPU tool's order and coverage: nets
        // as levels first read them, constants, unread gate outputs, unread
        // VCD signals (their counts from the VCD itself when the design has
        // no such net), assign aliases, then undriven declared bus bits; the
        // file ends after the NET list, as the reference's does
        VcdDecls decls;
        decls.bits = vcd.decl_bits;
        for (const SaifRecord &r : saif_ref_order(archived, decls)) {
            if (r.kind == SaifRecord::kConst) {
                rec(r.name, r.t0 ? dur : 0, r.t1 ? dur : 0, 0, "      ");
                continue;
            }
            if (r.kind == SaifRecord::kUndriven) {
                rec(r.name, 0, 0, dur, "      ");
                continue;
            }
            const int id = r.source.empty() ? -1 : d.find_net(r.source);
            if (id >= 0 && t0[resolve((uint32_t)id)] != UINT64_MAX) {
                const uint32_t s = resolve((uint32_t)id);
                rec(r.name, t0[s], t1[s], tx[s], "      ");
                continue;
            }
            auto v = r.source.empty() ? vcd.index.end() : vcd.index.find(r.source);
            if (v != vcd.index.end()) {
                uint64_t c[3];
                saif_of_changes(vcd.times[v->second], vcd.values[v->second], t_begin, t_end, c);
                rec(r.name, c[0], c[1], c[2], "      ");
                continue;
            }
            outf << "      (" << r.name << "\n      )\n";   // the reference prints no counts here
        }
        outf << "   )\n";
        outf.close();
        printf("simulated %zu instances in %zu levels: %llu gate-events, %llu output events, %.3f ms on the GPU\n",
               d.insts.size(), d.level_start.size() - 1, (unsigned long long)stats.gate_events,
               (unsigned long long)stats.output_events, stats.kernel_ms);
        return 0;
    }
    std::vector<uint8_t> done(n_nets, 0);
    std::vector<uint32_t> nested;   // unconnected outputs named inst[port]
    for (uint32_t n = 0; n < n_nets; ++n) {
        if (t0[n] == UINT64_MAX) continue;
        const std::string &nm = d.net_names[n];
        if (nm == "1'b0" || nm == "1'b1") continue;
        const size_t br = nm.find('[');
        if (br != std::string::npos && !isdigit((unsigned char)nm[br + 1])) {
            nested.push_back(n);
            continue;
        }
        rec(nm, t0[n], t1[n], tx[n], "      ");
        done[n] = 1;
    }
    for (auto &a : d.aliases) {
        if (done[a.first]) continue;
        const uint32_t src = resolve(a.first);
        if (t0[src] == UINT64_MAX) continue;
        rec(d.net_names[a.first], t0[src], t1[src], tx[src], "      ");
        done[a.first] = 1;
    }
    for (uint32_t n : d.bus_bits) {
        if (done[n] || t0[n] != UINT64_MAX) continue;
        rec(d.net_names[n], 0, 0, dur, "      ");
        done[n] = 1;
    }
    outf << "   )\n";
    for (uint32_t n : nested) {
        const std::string &nm = d.net_names[n];
        const size_t br = nm.find('[');
        outf << "   (INSTANCE " << nm.substr(0, br) << "\n      (NET\n";
        rec(nm.substr(br + 1, nm.size() - br - 2), t0[n], t1[n], tx[n], "         ");
        outf << "      )\n   )\n";
    }
    outf << ")\n";
    outf.close();
    printf("simulated %zu instances in %zu levels: %llu gate-events, %llu output events, %.3f ms on the GPU\n",
           d.insts.size(), d.level_start.size() - 1, (unsigned long long)stats.gate_events,
           (unsigned long long)stats.output_events, stats.kernel_ms);
    printf("timing (ms): design %.1f, stimulus %.1f, simulate %.1f (GPU kernels %.1f), SAIF %.1f, total %.1f\n",
           ms_design, ms_stim, ms_run, stats.kernel_ms, ms_since(t_saif), ms_since(t_start));
    return 0;
}
