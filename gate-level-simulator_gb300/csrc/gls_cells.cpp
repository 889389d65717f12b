// Cell truth tables for the device kernels.
//
// A gate output is evaluated on the GPU by one table lookup.  The table of
// output `o` of a cell is built here by running the cell's primitive program
// on every combination of 4-state input values, the way RunFunction
// (src/simulate.cpp:1203-1363) runs it per simulated time step: primitives
// in order, intermediate wires remembered, supply pins constant, unknown
// pins X, stop at the first primitive that drives `o`.
//
// Two primitive semantics are offered:
//   GLS_CALC_FIXED    4-state Verilog gate primitives, Z read as X; the UDPs
//                     follow their tables (udp_xbuf, udp_mux2 of
//                     examples/GENERIC_STD_CELL.vlib:2-11, 57-69).
//   GLS_CALC_LITERAL  the shipped calc of src/simulate.cpp:382-870 step for
//                     step, including its 1^x inversion under the
//                     0 / X=1 / Z=2 / 1=3 encoding.
#include <cstdint>
#include <cstring>
#include "gls.h"

namespace {

constexpr uint8_t V0 = 0, VX = 1, VZ = 2, V1 = 3;

uint8_t eval_fixed(int f, const uint8_t *in, int n)
{
    bool any0 = false, any1 = false, anyx = false;
    int par = 0;
    for (int i = 0; i < n; ++i) {
        if (in[i] == V0) any0 = true;
        else if (in[i] == V1) { any1 = true; par ^= 1; }
        else anyx = true;
    }
    switch (f) {
    case GLS_F_AND: return any0 ? V0 : (anyx ? VX : V1);
    case GLS_F_NAND: return any0 ? V1 : (anyx ? VX : V0);
    case GLS_F_OR: return any1 ? V1 : (anyx ? VX : V0);
    case GLS_F_NOR: return any1 ? V0 : (anyx ? VX : V1);
    case GLS_F_XOR: return anyx ? VX : (par ? V1 : V0);
    case GLS_F_XNOR: return anyx ? VX : (par ? V0 : V1);
    case GLS_F_BUF: return (in[0] == V0 || in[0] == V1) ? in[0] : VX;
    case GLS_F_NOT: return in[0] == V0 ? V1 : (in[0] == V1 ? V0 : VX);
    case GLS_F_UDP_XBUF:
        // rows "0 1 : 0", "1 1 : 1", "x 1 : 1"; everything else x
        if (n != 2 || in[1] != V1) return VX;
        return in[0] == V0 ? V0 : V1;
    case GLS_F_UDP_MUX2: {
        // rows select i0 when s=0, i1 when s=1, and agree when s=x
        if (n != 3) return VX;
        const bool a01 = in[0] == V0 || in[0] == V1, b01 = in[1] == V0 || in[1] == V1;
        if (in[2] == V0) return a01 ? in[0] : VX;
        if (in[2] == V1) return b01 ? in[1] : VX;
        return (a01 && in[0] == in[1]) ? in[0] : VX;
    }
    default: return VX;
    }
}

bool is_and(int f) { return f == GLS_F_AND || f == GLS_F_NAND; }
bool is_or(int f) { return f == GLS_F_OR || f == GLS_F_NOR; }

// first two inputs of the n-ary gates in the shipped calc
int literal_head(int f, uint8_t a, uint8_t b)
{
    const bool ax = a == VX || a == VZ, bx = b == VX || b == VZ;
    if (is_and(f)) {
        if (!ax && !bx) return a & b;
        return ax ? (b == V0 ? V0 : VX) : (a == V0 ? V0 : VX);
    }
    if (is_or(f)) {
        if (!ax && !bx) return a | b;
        return ax ? (b == V1 ? V1 : VX) : (a == V1 ? V1 : VX);
    }
    if (!ax && !bx) return a ^ b;
    if (a == VX || b == VX) return VX;
    if (a == VZ) return b == VZ ? V0 : VX;
    return VX;
}

// fold of each further input in the shipped calc (its switch on tmp)
int literal_fold(int f, int tmp, uint8_t x)
{
    if (is_and(f)) {
        switch (tmp) {
        case 0: return V0;
        case 1: return x == VZ ? VX : x;
        case 2: case 3: return x == V0 ? V0 : VX;
        default: return VX;
        }
    }
    if (is_or(f)) {
        switch (tmp) {
        case 0: return x == VZ ? VX : x;
        case 1: return V1;
        case 2: case 3: return x == V1 ? V1 : VX;
        default: return VX;
        }
    }
    switch (tmp) {
    case 0: return x == VZ ? VX : x;
    case 1: return (x == V0 || x == V1) ? (tmp ^ x) : VX;
    case 2: return VX;
    case 3: return x == VZ ? V0 : VX;
    default: return VX;
    }
}

uint8_t eval_literal(int f, const uint8_t *in, int n)
{
    switch (f) {
    case GLS_F_AND: case GLS_F_OR: case GLS_F_XOR: case GLS_F_XNOR: case GLS_F_NOR: case GLS_F_NAND: {
        if (n < 2) return VX;
        int tmp = literal_head(f, in[0], in[1]);
        for (int i = 2; i < n; ++i) tmp = literal_fold(f, tmp, in[i]);
        if (f == GLS_F_XNOR || f == GLS_F_NOR || f == GLS_F_NAND) tmp = (tmp == 0 || tmp == 1) ? (1 ^ tmp) : VX;
        return (uint8_t)tmp;
    }
    case GLS_F_BUF: return in[0] == VZ ? VX : in[0];
    case GLS_F_NOT: return (in[0] == V0 || in[0] == V1) ? (uint8_t)(1 ^ in[0]) : VX;
    case GLS_F_UDP_XBUF: return in[1] == V1 ? (in[0] == VX ? V1 : in[0]) : VX;
    case GLS_F_UDP_MUX2:
        if (in[2] == V0) return in[0];
        if (in[2] == V1) return in[1];
        if (in[2] == VX) return in[0] == in[1] ? in[0] : VX;
        return VX;
    default: return VX;
    }
}

}  // namespace

extern "C" int gls_cell_lut(const gls_cell *cell, const gls_prim *prims, int out, int calc_mode,
                            uint8_t *lut, uint32_t lut_cap)
{
    if (!cell || !prims || !lut) return GLS_EINVAL;
    if (cell->n_in > 6 || out < 0 || out >= cell->n_out) return GLS_EINVAL;
    if (calc_mode != GLS_CALC_FIXED && calc_mode != GLS_CALC_LITERAL) return GLS_EINVAL;
    const uint32_t entries = 1u << (2 * cell->n_in);
    if (lut_cap < entries) return GLS_EINVAL;
    const int out_pin = cell->n_in + out;
    for (int p = 0; p < cell->n_prim; ++p) {
        const gls_prim &pr = prims[cell->prim_start + p];
        if (pr.n_pins < 2 || pr.n_pins > 14 || pr.func > GLS_F_UDP_MUX2) return GLS_EINVAL;
    }
    for (uint32_t idx = 0; idx < entries; ++idx) {
        uint8_t val[256];
        bool have[256];
        std::memset(have, 0, sizeof have);
        uint8_t result = VX;
        for (int p = 0; p < cell->n_prim; ++p) {
            const gls_prim &pr = prims[cell->prim_start + p];
            const int ni = pr.n_pins - 1;
            uint8_t in[14];
            for (int j = 0; j < ni; ++j) {
                const int q = pr.pins[j];
                if (q < cell->n_in) in[j] = (uint8_t)((idx >> (2 * q)) & 3u);
                else if (have[q]) in[j] = val[q];
                else if (q == GLS_PIN_SUPPLY1) in[j] = V1;
                else if (q == GLS_PIN_SUPPLY0) in[j] = V0;
                else in[j] = VX;
            }
            const uint8_t r = calc_mode == GLS_CALC_LITERAL ? eval_literal(pr.func, in, ni)
                                                            : eval_fixed(pr.func, in, ni);
            const int q = pr.pins[ni];
            if (q == out_pin) { result = r; break; }
            val[q] = r;
            have[q] = true;
        }
        lut[idx] = result;
    }
    return GLS_OK;
}
