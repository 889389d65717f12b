// gls_process [--gpu-levelize] [--gpu-pack] [--native] <vlib> <gv> <sdf> <inter.dat>
//
// The `process` step of the reference (src/process.cpp:178-610): read the
// Verilog cell library, the flat gate-level netlist and the SDF file,
// levelize the instance graph and write the levelized design to inter.dat
// as the reference does, a Boost text archive of its `inter` class
// (host/boost_inter.cpp); --native writes the tools' own binary format
// instead (host/design.cpp).  With --gpu-levelize the levels are computed
// on GPU 0 (gls_levelize), with --gpu-pack the archive's packed per-level
// arrays (gls_pack_levels); the file is the same.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include "boost_inter.h"
#include "design.h"
#include "gls.h"

int main(int argc, char **argv)
{
    bool gpu = false, gpu_pack = false, native = false;
    std::vector<char *> pos;
    for (int k = 1; k < argc; ++k) {
        if (!strcmp(argv[k], "--gpu-levelize")) gpu = true;
        else if (!strcmp(argv[k], "--gpu-pack")) gpu_pack = true;
        else if (!strcmp(argv[k], "--native")) native = true;
        else pos.push_back(argv[k]);
    }
    if (pos.size() != 4) {
        printf("[USAGE] ./gls_process [--gpu-levelize] [--gpu-pack] [--native] vlib_path gv_path sdf_path "
               "intermediate_file\n");
        return 255;
    }
    argv = pos.data() - 1;
    using namespace glsh;
    std::string err;
    Library lib;
    Design d;
    const std::string vlib = read_file(argv[1], &err);
    if (vlib.empty() || !parse_vlib(vlib, lib, &err)) {
        printf("ERROR: %s\n", err.empty() ? "empty cell library" : err.c_str());
        return 255;
    }
    printf("INFO: vlib file's parsing done! (%zu modules, %zu skipped)\n", lib.cells.size(), lib.ignored.size());
    const std::string gv = read_file(argv[2], &err);
    if (gv.empty() || !parse_gv(gv, lib, d, &err)) {
        printf("ERROR: %s\n", err.empty() ? "empty netlist" : err.c_str());
        return 255;
    }
    printf("INFO: gate level file's parsing done! (%zu instances, %zu nets)\n", d.insts.size(), d.net_names.size());
    const std::string sdf = read_file(argv[3], &err);
    if (!sdf.empty() && !parse_sdf(sdf, d, lib, &err)) {
        printf("ERROR: %s\n", err.c_str());
        return 255;
    }
    printf("INFO: SDF file's parsing done!\n");
    if (gpu) {
        std::vector<uint64_t> start;
        std::vector<uint32_t> pred;
        instance_preds(d, start, pred);
        const uint32_t n = (uint32_t)d.insts.size();
        std::vector<uint32_t> order(n ? n : 1), level_start(n + 1);
        uint32_t n_levels = 0;
        const int rc = gls_levelize(0, n, start.data(), pred.data(), order.data(), level_start.data(), &n_levels);
        if (rc == GLS_EINVAL) {
            printf("ERROR: combinational loop: the netlist cannot be levelized\n");
            return 255;
        }
        if (rc) {
            printf("ERROR: GPU levelization failed (code %d)\n", rc);
            return 255;
        }
        order.resize(n);
        level_start.resize(n_levels + 1);
        apply_levels(d, order, level_start);
    } else if (!levelize(d, &err)) {
        printf("ERROR: %s\n", err.c_str());
        return 255;
    }
    printf("levels size: %zu\n", d.level_start.size() - 1);
    if (native) {
        if (!write_inter(argv[4], d, &err)) {
            printf("ERROR: %s\n", err.c_str());
            return 255;
        }
    } else {
        ref::Inter in;
        design_to_ref_inter(d, lib, in, false);
        const auto t0 = std::chrono::steady_clock::now();
        if (gpu_pack) {
            if (!pack_levels_gpu(in, 0, &err)) {
                printf("ERROR: %s\n", err.c_str());
                return 255;
            }
        } else {
            pack_levels(in);
        }
        printf("INFO: level packing done on the %s (%.1f ms)\n", gpu_pack ? "GPU" : "host",
               std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
        std::ofstream f(argv[4], std::ios::binary);
        const std::string text = save_boost_inter(in);
        f.write(text.data(), (std::streamsize)text.size());
        if (!f) {
            printf("ERROR: cannot write %s\n", argv[4]);
            return 255;
        }
    }
    printf("store database into %s\n", argv[4]);
    return 0;
}
