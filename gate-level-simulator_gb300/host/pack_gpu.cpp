// pack_levels_gpu: the packed per-level arrays of an archived design
// (src/process.cpp:423-566) computed by gls_pack_levels on the GPU.  The
// host only flattens every instance's counts, arcs (their nets as positions
// in the instance's net lists) and function rows in level order.
#include <algorithm>
#include "boost_inter.h"
#include "gls.h"

namespace glsh {

bool pack_levels_gpu(ref::Inter &out, int device, std::string *err)
{
    ref::PreProcess &p = out.p;
    auto inst = [&](int id) -> const ref::Instance & { return p.instances.at(p.instance_name_vec[id]); };
    auto pos = [](const std::vector<std::string> &v, const std::string &x) {
        return (int16_t)(std::find(v.begin(), v.end(), x) - v.begin());   // the list's length when absent
    };
    const uint32_t nl = (uint32_t)out.levels.size();
    std::vector<uint32_t> level_start(nl + 1, 0);
    for (uint32_t L = 0; L < nl; ++L) level_start[L + 1] = level_start[L] + (uint32_t)out.levels[L].size();
    const uint32_t n = level_start[nl];
    std::vector<uint16_t> n_in(n), n_out(n);
    std::vector<uint32_t> arc_start(n + 1, 0), row_start(n + 1, 0), entry_start(1, 0);
    std::vector<gls_pack_arc> arcs;
    std::vector<int16_t> entries;
    uint32_t i = 0;
    for (uint32_t L = 0; L < nl; ++L)
        for (int id : out.levels[L]) {
            const ref::Instance &c = inst(id);
            n_in[i] = (uint16_t)c.in_net.size();
            n_out[i] = (uint16_t)c.out_net.size();
            for (const ref::Delay &d : c.delays)
                arcs.push_back({(int16_t)d.edge, pos(c.in_net, d.in_bit), pos(c.out_net, d.out_bit), 0, (float)d.rise,
                                (float)d.fall});
            for (const auto &row : c.function_id_vec) {
                for (int x : row) entries.push_back((int16_t)x);
                entry_start.push_back((uint32_t)entries.size());
            }
            arc_start[i + 1] = (uint32_t)arcs.size();
            row_start[i + 1] = (uint32_t)entry_start.size() - 1;
            ++i;
        }
    gls_pack_in in{nl, n, level_start.data(), n_in.data(), n_out.data(), arc_start.data(), arcs.data(),
                   row_start.data(), entry_start.data(), entries.data()};
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
    gls_pack_out o{};
    o.data_in_num_start = out.data_in_num_start.data();
    o.data_out_num_start = out.data_out_num_start.data();
    o.delay_start = out.delay_start.data();
    o.delay_width = out.delay_width.data();
    o.functions_start = out.functions_start.data();
    o.functions_width = out.functions_width.data();
    o.data_in_num = out.data_in_num.data();
    o.data_out_num = out.data_out_num.data();
    o.val_num_start = out.val_num_start.data();
    o.delay_val_num = out.delay_val_num.data();
    o.functions_func_num = out.functions_func_num.data();
    o.functions_val_num = out.functions_val_num.data();
    int rc = gls_pack_levels(device, &in, &o);   // sizes the padded tables
    if (rc == GLS_EOVERFLOW) {
        out.host_delay_edges.assign(o.delay_total, 0);
        out.host_in_bit.assign(o.delay_total, 0);
        out.host_out_bit.assign(o.delay_total, 0);
        out.host_rise_val.assign(o.delay_total, 0.f);
        out.host_fall_val.assign(o.delay_total, 0.f);
        out.host_functions.assign(o.functions_total, 0);
        o.delay_edges = out.host_delay_edges.data();
        o.in_bit = out.host_in_bit.data();
        o.out_bit = out.host_out_bit.data();
        o.rise_val = out.host_rise_val.data();
        o.fall_val = out.host_fall_val.data();
        o.functions = out.host_functions.data();
        o.delay_cap = o.delay_total;
        o.functions_cap = o.functions_total;
        rc = gls_pack_levels(device, &in, &o);
    } else if (rc == GLS_OK) {   // no padded entries at all
        out.host_delay_edges.clear();
        out.host_in_bit.clear();
        out.host_out_bit.clear();
        out.host_rise_val.clear();
        out.host_fall_val.clear();
        out.host_functions.clear();
    }
    if (rc != GLS_OK) {
        if (err) *err = "gls_pack_levels failed with status " + std::to_string(rc);
        return false;
    }
    return true;
}

}  // namespace glsh
