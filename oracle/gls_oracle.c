/*
 * gls_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's serial gate-level simulator
 * (YiwiSun/gate-level-simulator, src/simulate.cpp).  It is the checker for
 * the CUDA path: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg may run it, never the product path.
 *
 * Parity is pinned: tests/test_oracle.py checks this restatement against the
 * reference's own functions compiled from the reference sources
 * (oracle/build.py -> oracle/_ref/ref_sim) and against the committed
 * golden vectors in tests/golden/.
 *
 * Functions and the reference lines they restate:
 *   calc_fixed / calc_literal   src/simulate.cpp:382-870   (calc)
 *   run_function                src/simulate.cpp:1203-1363 (RunFunction)
 *   check_delay                 src/simulate.cpp:1178-1201 (CheckDelay)
 *   add_delay                   src/simulate.cpp:1012-1176 (AddDelay)
 *   get_value_at                src/simulate.cpp:1459-1506 (GetValueAt)
 *   simulate_output             src/simulate.cpp:872-1011  (SimulateInst +
 *                               Process 1365-1457 + Calculate 919-1011)
 *   saif_integral               src/simulate.cpp:102-163   (DumpSaif loop)
 *   level loop                  src/simulate.cpp:1569-1668
 *
 * Input: a case file (format in oracle/casefile.py).  Output: a result file
 * with every computed net's waveform and its T0/T1/TX counts.
 *
 * usage: gls_oracle <case> <result> [--calc fixed|literal] [--factor F]
 *                   [--threads N] [--insts a:b]   (simulate only that
 *                   instance range; inputs must then come from stimulus)
 *                   [--keep nets.bin]  (write the waveforms of only these
 *                   nets: u32 count, then u32 net ids; every other net's
 *                   list is freed after the last level that reads it, once
 *                   its SAIF counts are taken -- a run over a large design
 *                   then holds only the lists still to be read)
 *                   [--verify-lookup]  (also run GetValueAt's binary search
 *                   at every step and stop if it disagrees with the cursor
 *                   values the simulation uses)
 *
 * Asserts of the reference are treated as compiled with NDEBUG: an input
 * edge that is neither rise nor fall counts as posedge
 * (src/simulate.cpp:1058-1065), exactly like the reference's else-branch.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <float.h>

enum { V0 = 0, VX = 1, VZ = 2, V1 = 3 };
enum { F_AND = 0, F_OR, F_XOR, F_XNOR, F_NOR, F_NAND, F_BUF, F_NOT, F_UDP_XBUF, F_UDP_MUX2 };
#define PIN_SUPPLY0 16
#define PIN_SUPPLY1 17

typedef struct { uint8_t func, npins; uint8_t pins[16]; } Prim;
typedef struct { uint8_t n_in, n_out, n_prim; Prim *prims; } Cell;
typedef struct { uint8_t edge, in_pin, out_pin; double rise, fall; } Arc;
typedef struct {
    uint32_t cell, level;
    uint32_t *in, *out;
    uint16_t n_arcs;
    Arc *arcs;
} Inst;
typedef struct { uint64_t n, cap; uint64_t *t; uint8_t *v; int valid; } Wave;

static uint32_t g_n_nets, g_n_cells, g_n_inst;
static Cell *g_cells;
static Inst *g_inst;
static Wave *g_wave;
static uint64_t g_t_begin, g_t_end;
static int g_literal = 0;
static double g_factor = 1.0;
static int g_verify_lookup = 0;

static void die(const char *m) { fprintf(stderr, "gls_oracle: %s\n", m); exit(2); }

/* ---------------------------------------------------------------- reading */
static FILE *g_in;
static void rd(void *p, size_t n) { if (fread(p, 1, n, g_in) != n) die("truncated case file"); }
static uint8_t rd8(void) { uint8_t x; rd(&x, 1); return x; }
static uint16_t rd16(void) { uint16_t x; rd(&x, 2); return x; }
static uint32_t rd32(void) { uint32_t x; rd(&x, 4); return x; }
static uint64_t rd64(void) { uint64_t x; rd(&x, 8); return x; }
static double rdf(void) { double x; rd(&x, 8); return x; }

static void wave_push(Wave *w, uint64_t t, uint8_t v)
{
    if (w->n == w->cap) {
        w->cap = w->cap ? w->cap * 2 : 16;
        w->t = realloc(w->t, w->cap * 8);
        w->v = realloc(w->v, w->cap);
        if (!w->t || !w->v) die("out of memory");
    }
    w->t[w->n] = t; w->v[w->n] = v; w->n++;
}

static void read_case(const char *path)
{
    g_in = fopen(path, "rb");
    if (!g_in) die("cannot open case file");
    char magic[8]; rd(magic, 8);
    if (memcmp(magic, "GLSCASE1", 8)) die("bad case magic");
    g_n_nets = rd32();
    g_n_cells = rd32();
    g_cells = calloc(g_n_cells, sizeof(Cell));
    for (uint32_t c = 0; c < g_n_cells; ++c) {
        Cell *cl = &g_cells[c];
        cl->n_in = rd8(); cl->n_out = rd8(); cl->n_prim = rd8();
        cl->prims = calloc(cl->n_prim, sizeof(Prim));
        for (int p = 0; p < cl->n_prim; ++p) {
            cl->prims[p].func = rd8();
            cl->prims[p].npins = rd8();
            if (cl->prims[p].npins > 16 || cl->prims[p].npins < 2) die("bad primitive");
            rd(cl->prims[p].pins, cl->prims[p].npins);
        }
    }
    g_n_inst = rd32();
    g_inst = calloc(g_n_inst, sizeof(Inst));
    for (uint32_t i = 0; i < g_n_inst; ++i) {
        Inst *in = &g_inst[i];
        in->cell = rd32(); in->level = rd32();
        if (in->cell >= g_n_cells) die("bad cell id");
        Cell *cl = &g_cells[in->cell];
        in->in = malloc(sizeof(uint32_t) * (cl->n_in ? cl->n_in : 1));
        in->out = malloc(sizeof(uint32_t) * (cl->n_out ? cl->n_out : 1));
        for (int k = 0; k < cl->n_in; ++k) in->in[k] = rd32();
        for (int k = 0; k < cl->n_out; ++k) in->out[k] = rd32();
        in->n_arcs = rd16();
        in->arcs = calloc(in->n_arcs ? in->n_arcs : 1, sizeof(Arc));
        for (int a = 0; a < in->n_arcs; ++a) {
            in->arcs[a].edge = rd8(); in->arcs[a].in_pin = rd8();
            in->arcs[a].out_pin = rd8(); (void)rd8();
            in->arcs[a].rise = rdf(); in->arcs[a].fall = rdf();
        }
    }
    g_wave = calloc(g_n_nets, sizeof(Wave));
    uint32_t n_stim = rd32();
    for (uint32_t s = 0; s < n_stim; ++s) {
        uint32_t net = rd32();
        uint32_t n = rd32();
        if (net >= g_n_nets) die("bad stimulus net");
        Wave *w = &g_wave[net];
        w->n = w->cap = n;
        w->t = malloc(8 * (n ? n : 1));
        w->v = malloc(n ? n : 1);
        for (uint32_t e = 0; e < n; ++e) w->t[e] = rd64();
        rd(w->v, n);
        w->valid = 1;
    }
    g_t_begin = rd64();
    g_t_end = rd64();
    fclose(g_in);
}

/* ------------------------------------------------------------------- calc */
/* 4-state Verilog primitive semantics (the "ref-fixed" calc mode): Z on an
 * input is an unknown; udp_xbuf / udp_mux2 follow their UDP tables in
 * examples/GENERIC_STD_CELL.vlib:2-11 and :57-69. */
static uint8_t inv(uint8_t v) { return v == V0 ? V1 : v == V1 ? V0 : VX; }
static uint8_t calc_fixed(int f, const uint8_t *in, int n)
{
    int any0 = 0, any1 = 0, anyx = 0, par = 0;
    for (int i = 0; i < n; ++i) {
        if (in[i] == V0) any0 = 1;
        else if (in[i] == V1) { any1 = 1; par ^= 1; }
        else anyx = 1;
    }
    switch (f) {
    case F_AND:  return any0 ? V0 : anyx ? VX : V1;
    case F_NAND: return any0 ? V1 : anyx ? VX : V0;
    case F_OR:   return any1 ? V1 : anyx ? VX : V0;
    case F_NOR:  return any1 ? V0 : anyx ? VX : V1;
    case F_XOR:  return anyx ? VX : (par ? V1 : V0);
    case F_XNOR: return anyx ? VX : (par ? V0 : V1);
    case F_BUF:  return (in[0] == V0 || in[0] == V1) ? in[0] : VX;
    case F_NOT:  return inv(in[0]);
    case F_UDP_XBUF:
        if (n != 2 || in[1] != V1) return VX;
        return in[0] == V0 ? V0 : V1;
    case F_UDP_MUX2: {
        if (n != 3) return VX;
        uint8_t a = in[0], b = in[1], s = in[2];
        int a01 = (a == V0 || a == V1), b01 = (b == V0 || b == V1);
        if (s == V0) return a01 ? a : VX;
        if (s == V1) return b01 ? b : VX;
        return (a01 && a == b) ? a : VX;
    }
    }
    return VX;
}

/* The shipped calc of src/simulate.cpp:382-870 (the "ref-literal" mode),
 * restated operation by operation, including its 1^x inversion under the
 * 0/X=1/Z=2/1=3 encoding. */
static int lit_first_two(int f, uint8_t a, uint8_t b)
{
    int ax = (a == VX || a == VZ), bx = (b == VX || b == VZ);
    switch (f) {
    case F_AND: case F_NAND:
        if (!ax && !bx) return a & b;
        if (ax) return b == V0 ? V0 : VX;
        return a == V0 ? V0 : VX;
    case F_OR: case F_NOR:
        if (!ax && !bx) return a | b;
        if (ax) return b == V1 ? V1 : VX;
        return a == V1 ? V1 : VX;
    default: /* xor, xnor */
        if (!ax && !bx) return a ^ b;
        if (a == VX || b == VX) return VX;
        if (a == VZ) return b == VZ ? V0 : VX;
        return a == VZ ? V0 : VX;
    }
}
static int lit_step(int f, int tmp, uint8_t x)
{
    switch (f) {
    case F_AND: case F_NAND:
        if (tmp == 0) return V0;
        if (tmp == 1) return x == VZ ? VX : x;
        if (tmp == 2 || tmp == 3) return x == V0 ? V0 : VX;
        return VX;
    case F_OR: case F_NOR:
        if (tmp == 0) return x == VZ ? VX : x;
        if (tmp == 1) return V1;
        if (tmp == 2 || tmp == 3) return x == V1 ? V1 : VX;
        return VX;
    default: /* xor, xnor */
        if (tmp == 0) return x == VZ ? VX : x;
        if (tmp == 1) return (x == V0 || x == V1) ? (tmp ^ x) : VX;
        if (tmp == 2) return VX;
        if (tmp == 3) return x == VZ ? V0 : VX;
        return VX;
    }
}
static uint8_t calc_literal(int f, const uint8_t *in, int n)
{
    int tmp;
    switch (f) {
    case F_AND: case F_OR: case F_XOR: case F_XNOR: case F_NOR: case F_NAND:
        tmp = lit_first_two(f, in[0], in[1]);
        for (int i = 2; i < n; ++i) tmp = lit_step(f, tmp, in[i]);
        if (f == F_XNOR || f == F_NOR || f == F_NAND)
            tmp = (tmp == 0 || tmp == 1) ? (1 ^ tmp) : VX;
        return (uint8_t)tmp;
    case F_BUF: return in[0] == VZ ? VX : in[0];
    case F_NOT: return (in[0] == V0 || in[0] == V1) ? (uint8_t)(1 ^ in[0]) : VX;
    case F_UDP_XBUF:
        if (in[1] == V1) return in[0] == VX ? V1 : in[0];
        return VX;
    case F_UDP_MUX2:
        if (in[2] == V0) return in[0];
        if (in[2] == V1) return in[1];
        if (in[2] == VX) return in[0] == in[1] ? in[0] : VX;
        return VX;
    }
    return VX;
}

/* RunFunction: evaluate the cell's primitives in order and return at the
 * first one that drives output `o`; intermediate wires and other outputs are
 * remembered by pin, supply pins are constants, anything unknown reads X. */
static uint8_t run_function(const Cell *cl, const uint8_t *pin_val, int o)
{
    uint8_t val[32]; uint8_t have[32];
    memset(have, 0, sizeof have);
    int out_pin = cl->n_in + o;
    for (int p = 0; p < cl->n_prim; ++p) {
        const Prim *pr = &cl->prims[p];
        uint8_t in[16];
        int ni = pr->npins - 1;
        for (int j = 0; j < ni; ++j) {
            int q = pr->pins[j];
            if (q < cl->n_in) in[j] = pin_val[q];
            else if (q < 32 && have[q]) in[j] = val[q];
            else if (q == PIN_SUPPLY1) in[j] = V1;
            else if (q == PIN_SUPPLY0) in[j] = V0;
            else in[j] = VX;
        }
        uint8_t r = g_literal ? calc_literal(pr->func, in, ni) : calc_fixed(pr->func, in, ni);
        int q = pr->pins[ni];
        if (q == out_pin) return r;
        if (q < 32) { val[q] = r; have[q] = 1; }
    }
    return VX; /* no primitive drives the output: undefined in the reference */
}

/* CheckDelay: 1 rise, 2 fall, 3 X->Z, 4 Z->X, 0 unchanged. */
static int check_delay(uint8_t pre, uint8_t cur)
{
    if ((pre == V0 && cur != V0) || (cur == V1 && pre != V1)) return 1;
    if ((pre == V1 && cur != V1) || (cur == V0 && pre != V0)) return 2;
    if (pre == VX && cur == VZ) return 3;
    if (pre == VZ && cur == VX) return 4;
    return 0;
}

static double pick(const Arc *a, int s)
{
    switch (s) {
    case 1: return a->rise;
    case 2: return a->fall;
    case 3: return a->rise > a->fall ? a->rise : a->fall;
    case 4: return a->rise < a->fall ? a->rise : a->fall;
    }
    return 1.0;
}

/* GetValueAt: binary search for time t in a net's change list; cur is the
 * value at t, last the value just before an event at exactly t. */
static void get_value_at(const Wave *w, uint64_t t, uint8_t *cur, uint8_t *last)
{
    *cur = VX; *last = VX;
    if (w->n == 0) return;
    uint64_t beg = 0, end = w->n, mid = beg + (end - beg) / 2;
    while (mid != end) {
        if (w->t[mid] < t) {
            *cur = w->v[mid]; *last = w->v[mid];
            beg = mid + 1; mid = beg + (end - beg) / 2;
        } else if (w->t[mid] > t) {
            end = mid; mid = beg + (end - beg) / 2;
        } else {
            *cur = w->v[mid];
            if (mid != 0) *last = w->v[mid - 1];
            break;
        }
    }
}

/* ---------------------------------------------------------- per output */
static void simulate_output(const Inst *in, int o, Wave *outw)
{
    const Cell *cl = &g_cells[in->cell];
    /* distinct input nets (bitValues is a map keyed by net) */
    uint32_t nets[16]; int m = 0;
    for (int p = 0; p < cl->n_in; ++p) {
        int seen = 0;
        for (int j = 0; j < m; ++j) if (nets[j] == in->in[p]) seen = 1;
        if (!seen) nets[m++] = in->in[p];
    }
    const Wave *w[16];
    for (int j = 0; j < m; ++j) {
        w[j] = &g_wave[nets[j]];
        if (!w[j]->valid) die("input net has no waveform (level order broken)");
        for (uint64_t e = 1; e < w[j]->n; ++e)
            if (w[j]->t[e] <= w[j]->t[e - 1]) die("input waveform times not strictly increasing");
    }
    outw->n = 0;
    wave_push(outw, 0, VX);
    outw->valid = 1;
    uint8_t pre = VX;
    uint64_t cursor[16] = {0};
    for (;;) {
        /* Process: next distinct time over all input nets */
        uint64_t t = UINT64_MAX; int any = 0;
        for (int j = 0; j < m; ++j)
            if (cursor[j] < w[j]->n && w[j]->t[cursor[j]] < t) { t = w[j]->t[cursor[j]]; any = 1; }
        if (!any) break;
        uint32_t chg = 0;
        for (int j = 0; j < m; ++j)
            if (cursor[j] < w[j]->n && w[j]->t[cursor[j]] == t) { chg |= 1u << j; cursor[j]++; }
        /* cur / last value of every input pin.  GetValueAt's binary search
         * finds, for a net with an event at t, that event's value and the one
         * before it (X for a first event), else the value of the last event
         * before t (X if none) for both; the cursors, just moved past the
         * events at t, give the same values directly. */
        uint8_t cur_net[16], last_net[16], pin_val[16];
        for (int j = 0; j < m; ++j) {
            const uint64_t c = cursor[j];
            if ((chg >> j) & 1u) {
                cur_net[j] = w[j]->v[c - 1];
                last_net[j] = c >= 2 ? w[j]->v[c - 2] : VX;
            } else {
                cur_net[j] = last_net[j] = c ? w[j]->v[c - 1] : VX;
            }
            if (g_verify_lookup) {
                uint8_t vc, vl;
                get_value_at(w[j], t, &vc, &vl);
                if (vc != cur_net[j] || vl != last_net[j]) die("cursor values disagree with GetValueAt");
            }
        }
        for (int p = 0; p < cl->n_in; ++p)
            for (int j = 0; j < m; ++j) if (nets[j] == in->in[p]) pin_val[p] = cur_net[j];
        uint8_t F = run_function(cl, pin_val, o);
        int s = check_delay(pre, F);
        if (s == 0) continue;
        /* related delays: arcs of this output whose input net changed */
        const Arc *rel[64]; int nrel = 0; int rel_slot[64];
        for (int a = 0; a < in->n_arcs; ++a) {
            const Arc *arc = &in->arcs[a];
            if (arc->out_pin != o) continue;
            uint32_t net = in->in[arc->in_pin];
            for (int j = 0; j < m; ++j)
                if (nets[j] == net && ((chg >> j) & 1)) {
                    if (nrel < 64) { rel_slot[nrel] = j; rel[nrel++] = arc; }
                }
        }
        int num_in = __builtin_popcount(chg);
        double dv = 1.0;
        if (nrel == 0) dv = 1.0;
        else if (num_in == 1) {
            if (nrel == 1) dv = pick(rel[0], s);
            else {
                int j = rel_slot[0];
                int is = check_delay(last_net[j], cur_net[j]);
                int edge = (is == 2) ? 1 : 0;
                for (int r = 0; r < nrel; ++r)
                    if (rel[r]->edge == edge) { dv = pick(rel[r], s); break; }
            }
        } else {
            double mn = DBL_MAX;
            for (int r = 0; r < nrel; ++r) {
                const Arc *arc = rel[r];
                if (arc->edge == 2) { double x = pick(arc, s); if (x < mn) mn = x; }
                else {
                    int j = rel_slot[r];
                    int is = check_delay(last_net[j], cur_net[j]);
                    int edge = (is == 2) ? 1 : 0;
                    if (edge == arc->edge) { double x = pick(arc, s); if (x < mn) mn = x; }
                }
            }
            dv = (mn == DBL_MAX) ? 1.0 : mn;
        }
        uint64_t out_t = t + (uint64_t)(dv * g_factor);
        /* inertial update of the output list (Calculate 991-1009) */
        uint64_t lt = outw->t[outw->n - 1]; uint8_t lv = outw->v[outw->n - 1];
        while (lt >= out_t) {
            if (outw->n <= 1) { outw->n--; break; }
            outw->n--;
            lt = outw->t[outw->n - 1]; lv = outw->v[outw->n - 1];
        }
        if (lv != F) wave_push(outw, out_t, F);
        if (outw->n == 0) die("output list emptied (zero delay at time 0 with equal value)");
        pre = outw->v[outw->n - 1];
    }
}

/* ------------------------------------------------------------ threading */
static uint32_t g_lo, g_hi;
static volatile uint32_t g_next;
static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;

static void *worker(void *arg)
{
    (void)arg;
    for (;;) {
        pthread_mutex_lock(&g_mu);
        uint32_t i = g_next++;
        pthread_mutex_unlock(&g_mu);
        if (i >= g_hi) break;
        const Inst *in = &g_inst[i];
        const Cell *cl = &g_cells[in->cell];
        for (int o = 0; o < cl->n_out; ++o) simulate_output(in, o, &g_wave[in->out[o]]);
    }
    return NULL;
}

/* ------------------------------------------------------ lean mode (--keep) */
static uint8_t *g_keep;          /* per net: 1 = write its waveform */
static int32_t *g_free_after;    /* per net: level after which its list is dropped (-1: at once) */
static uint64_t (*g_saif)[3];    /* per net: counts taken before a list is dropped */
static uint8_t *g_saif_done;

static void saif_integral(const Wave *w, uint64_t start, uint64_t end, uint64_t r[3]);

static void drop_list(uint32_t n)
{
    Wave *w = &g_wave[n];
    if (!w->valid || g_saif_done[n]) return;
    saif_integral(w, g_t_begin, g_t_end, g_saif[n]);
    g_saif_done[n] = 1;
    if (g_keep[n]) return;
    free(w->t); free(w->v);
    w->t = NULL; w->v = NULL; w->n = w->cap = 0;
}

/* ----------------------------------------------------------------- SAIF */
static void saif_integral(const Wave *w, uint64_t start, uint64_t end, uint64_t r[3])
{
    uint64_t t0 = 0, t1 = 0, tx = 0, tz = 0, last_time = start;
    uint8_t st = VX;
    for (uint64_t e = 0; e < w->n; ++e) {
        uint64_t ct = w->t[e];
        if (ct <= start) { st = w->v[e]; continue; }
        if (ct > end) break;
        uint64_t d = ct - last_time;
        if (st == VX) tx += d; else if (st == V0) t0 += d; else if (st == V1) t1 += d; else tz += d;
        last_time = ct; st = w->v[e];
    }
    if (last_time < end) {
        uint64_t d = end - last_time;
        if (st == VX) tx += d; else if (st == V0) t0 += d; else if (st == V1) t1 += d; else tz += d;
    }
    r[0] = t0; r[1] = t1; r[2] = tx + tz;
}

int main(int argc, char **argv)
{
    if (argc < 3) die("usage: gls_oracle <case> <result> [--calc fixed|literal] [--factor F] [--threads N] [--insts a:b] "
                      "[--keep nets.bin] [--verify-lookup]");
    int threads = 1;
    long lo = -1, hi = -1;
    const char *keep_path = NULL;
    for (int i = 3; i < argc; ++i) {
        if (!strcmp(argv[i], "--calc") && i + 1 < argc) g_literal = !strcmp(argv[++i], "literal");
        else if (!strcmp(argv[i], "--factor") && i + 1 < argc) g_factor = atof(argv[++i]);
        else if (!strcmp(argv[i], "--threads") && i + 1 < argc) threads = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--insts") && i + 1 < argc) {
            if (sscanf(argv[++i], "%ld:%ld", &lo, &hi) != 2) die("bad --insts");
        } else if (!strcmp(argv[i], "--keep") && i + 1 < argc) keep_path = argv[++i];
        else if (!strcmp(argv[i], "--verify-lookup")) g_verify_lookup = 1;
        else die("unknown option");
    }
    read_case(argv[1]);
    if (threads < 1) threads = 1;
    if (lo < 0) { lo = 0; hi = g_n_inst; }
    if (hi > (long)g_n_inst) hi = g_n_inst;
    const int lean = keep_path != NULL;
    if (lean) {
        g_keep = calloc(g_n_nets, 1);
        g_free_after = malloc(sizeof(int32_t) * g_n_nets);
        g_saif = calloc(g_n_nets, sizeof *g_saif);
        g_saif_done = calloc(g_n_nets, 1);
        if (!g_keep || !g_free_after || !g_saif || !g_saif_done) die("out of memory");
        FILE *kf = fopen(keep_path, "rb");
        if (!kf) die("cannot open --keep file");
        uint32_t nk;
        if (fread(&nk, 4, 1, kf) != 1) die("truncated --keep file");
        for (uint32_t k = 0; k < nk; ++k) {
            uint32_t n;
            if (fread(&n, 4, 1, kf) != 1) die("truncated --keep file");
            if (n >= g_n_nets) die("bad net in --keep file");
            g_keep[n] = 1;
        }
        fclose(kf);
        /* a list is dropped after the last level that reads it; one that no
         * simulated instance reads, after the level that makes it */
        for (uint32_t n = 0; n < g_n_nets; ++n) g_free_after[n] = -1;
        for (long k = lo; k < hi; ++k) {
            const Inst *in = &g_inst[k];
            const Cell *cl = &g_cells[in->cell];
            for (int q = 0; q < cl->n_in; ++q)
                if ((int32_t)in->level > g_free_after[in->in[q]]) g_free_after[in->in[q]] = (int32_t)in->level;
            for (int q = 0; q < cl->n_out; ++q)
                if ((int32_t)in->level > g_free_after[in->out[q]]) g_free_after[in->out[q]] = (int32_t)in->level;
        }
        for (uint32_t n = 0; n < g_n_nets; ++n)
            if (g_free_after[n] < 0) drop_list(n);
    }
    /* level loop: instances are stored in level order */
    uint32_t i = (uint32_t)lo;
    while (i < (uint32_t)hi) {
        uint32_t j = i;
        while (j < (uint32_t)hi && g_inst[j].level == g_inst[i].level) ++j;
        g_lo = i; g_hi = j; g_next = i;
        pthread_t th[256];
        int nt = threads > 256 ? 256 : threads;
        for (int k = 0; k < nt; ++k) pthread_create(&th[k], NULL, worker, NULL);
        for (int k = 0; k < nt; ++k) pthread_join(th[k], NULL);
        if (lean) {
            const int32_t L = (int32_t)g_inst[i].level;
            for (uint32_t n = 0; n < g_n_nets; ++n)
                if (g_free_after[n] == L) drop_list(n);
        }
        i = j;
    }
    FILE *f = fopen(argv[2], "wb");
    if (!f) die("cannot open result file");
    fwrite("GLSRES01", 1, 8, f);
    fwrite(&g_n_nets, 4, 1, f);
    for (uint32_t n = 0; n < g_n_nets; ++n) {
        const Wave *w = &g_wave[n];
        const int write = w->valid && (!lean || g_keep[n]);
        uint64_t cnt = write ? w->n : UINT64_MAX;
        fwrite(&cnt, 8, 1, f);
        if (!write) continue;
        fwrite(w->t, 8, w->n, f);
        fwrite(w->v, 1, w->n, f);
    }
    for (uint32_t n = 0; n < g_n_nets; ++n) {
        uint64_t r[3] = {UINT64_MAX, UINT64_MAX, UINT64_MAX};
        if (lean && g_saif_done[n]) memcpy(r, g_saif[n], sizeof r);
        else if (g_wave[n].valid) saif_integral(&g_wave[n], g_t_begin, g_t_end, r);
        fwrite(r, 8, 3, f);
    }
    fclose(f);
    return 0;
}
