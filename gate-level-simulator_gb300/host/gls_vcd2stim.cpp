// gls_vcd2stim <in.vcd> <out.glsstim> [--device N] [--host-vcd]
//
// Convert a VCD stimulus into the tools' binary stimulus file (layout in
// vcd.h): the change lists gls_simulate would read from the VCD, which it
// then loads without parsing text.  The VCD body is scanned on the GPU
// (gls_vcd_scan) unless --host-vcd is given.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include "design.h"
#include "vcd.h"

using namespace glsh;

int main(int argc, char **argv)
{
    if (argc < 3) {
        printf("[USAGE] ./gls_vcd2stim vcd_path out_path [--device N] [--host-vcd]\n");
        return 255;
    }
    int device = 0;
    bool host_vcd = false;
    for (int k = 3; k < argc; ++k) {
        if (!strcmp(argv[k], "--device") && k + 1 < argc) device = atoi(argv[++k]);
        else if (!strcmp(argv[k], "--host-vcd")) host_vcd = true;
    }
    std::string err;
    const std::string text = read_file(argv[1], &err);
    VcdData v;
    if (text.empty() || (host_vcd ? !parse_vcd(text, v, &err) : parse_vcd_gpu(text, v, &err, device) < 0)) {
        printf("Parse Failed. %s\n", err.c_str());
        return 1;
    }
    const std::string out = save_stim_bin(v);
    std::ofstream f(argv[2], std::ios::binary);
    if (!f || !f.write(out.data(), (std::streamsize)out.size())) {
        printf("File %s Open Error!\nExit!\n", argv[2]);
        return 255;
    }
    return 0;
}
