/*
 * gls.h -- C ABI of the GB300 gate-level simulation library (libgls.so).
 *
 * The reference (YiwiSun/gate-level-simulator) exposes its simulate stage
 * only as a CLI over files; its in-process boundary is the per-level host
 * loop of src/simulate.cu:2027-3254, which stages each level's fan-in
 * waveforms, launches the kernels of src/simulate.cu:486-1555 and writes
 * SAIF through the DumpSaif overloads of src/simulate.cu:113-481.  The entry
 * points below replace that loop; each cites the reference code it stands in
 * for.  The simulation semantics are those of the reference's serial CPU
 * simulator, src/simulate.cpp:872-1506.
 *
 * Conventions
 *   - Every call returns an int status: GLS_OK (0) or a GLS_E* code; the
 *     library never calls exit().  gls_last_error() gives a message.
 *   - The context owns all device memory.  Host pointers passed in are only
 *     read during the call.
 *   - A context is used by one host thread at a time.
 *   - Results do not depend on launch configuration or segment size.
 *
 * Value encoding (src/VCDTypes.h:49-54): 0 = logic 0, 1 = X, 2 = Z, 3 = 1.
 * Times are unsigned 32-bit integers in the VCD time unit, as in the
 * reference GPU tool (src/simulate.cu:2020-2023).
 */
#ifndef GLS_H
#define GLS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GLS_ABI_VERSION 2

/* status codes */
#define GLS_OK 0
#define GLS_EINVAL 1      /* bad argument or malformed netlist / stimulus */
#define GLS_ECUDA 2       /* CUDA runtime error */
#define GLS_ENOMEM 3      /* device or host allocation failed */
#define GLS_ESTATE 4      /* call out of order (e.g. run before load) */
#define GLS_ERANGE 5      /* a time or size does not fit the 32-bit pool */
#define GLS_EOVERFLOW 6   /* event pool exhausted and could not grow */

/* calc modes: which gate-evaluation semantics the cell truth tables use */
#define GLS_CALC_FIXED 0    /* 4-state Verilog primitives (Z reads as X) */
#define GLS_CALC_LITERAL 1  /* the shipped calc of src/simulate.cpp:382-870 */

/* output allocation modes */
#define GLS_ALLOC_BOUND 0   /* slot per gate output reserved up front: its fan-in events + 1 */
#define GLS_ALLOC_EXACT 1   /* count-then-fill: a list is placed once its final length is known */
#define GLS_ALLOC_LEARNED 2 /* slot presized by the presize model (gls_set_presize_model); an
                               output that outgrows its slot is placed exactly instead */

/* primitive ids of the reference function program (src/PreProcess.cpp:1194-1197) */
#define GLS_F_AND 0
#define GLS_F_OR 1
#define GLS_F_XOR 2
#define GLS_F_XNOR 3
#define GLS_F_NOR 4
#define GLS_F_NAND 5
#define GLS_F_BUF 6
#define GLS_F_NOT 7
#define GLS_F_UDP_XBUF 8
#define GLS_F_UDP_MUX2 9
/* pin codes inside a primitive (src/PreProcess.cpp:1199-1263): cell input k
 * is k, cell output k is n_in + k, internal wires follow, and the supply
 * nets are these two constants. */
#define GLS_PIN_SUPPLY0 16
#define GLS_PIN_SUPPLY1 17

typedef struct gls_ctx gls_ctx;

typedef struct {
    int device;            /* CUDA device ordinal */
    int calc_mode;         /* GLS_CALC_* */
    int alloc_mode;        /* GLS_ALLOC_* */
    double delay_factor;   /* SDF delay -> time unit factor; 1.0 for ps
                              (src/simulate.cpp:1165-1175) */
    uint32_t seg_events;   /* fan-in events per time segment (0 = default) */
    uint64_t pool_events;  /* initial event-pool capacity (0 = automatic) */
    void *stream;          /* cudaStream_t to launch on (NULL = own stream) */
    int profile;           /* 1: time every kernel class with CUDA events (the fan-in
                              classes of a level then run one after another) */
} gls_opts;

/* One library cell: its primitive program in the reference encoding
 * (Instance::function_id_vec, src/PreProcess.cpp:1194-1263). */
typedef struct {
    uint8_t n_in, n_out, n_prim, reserved;
    uint32_t prim_start;   /* index of the first primitive in prims[] */
} gls_cell;

typedef struct {
    uint8_t func;          /* GLS_F_* */
    uint8_t n_pins;        /* inputs followed by the one driven pin */
    uint8_t pins[14];
} gls_prim;

/* An SDF IOPATH arc (Delay, src/VCDTypes.h:166-186).  edge: 0 posedge,
 * 1 negedge, 2 both.  Delays are in SDF units before delay_factor. */
typedef struct {
    uint8_t edge, in_pin, out_pin, reserved[5];
    double rise, fall;
} gls_arc;

/* The levelized netlist, as `process` packs it into inter.dat
 * (src/process.cpp:58-79, 252-566).  Instances are stored in level order. */
typedef struct {
    uint32_t n_nets;
    uint32_t n_cells;
    const gls_cell *cells;
    uint32_t n_prims;
    const gls_prim *prims;
    uint32_t n_inst;
    uint32_t n_levels;
    const uint32_t *level_start;   /* n_levels + 1, into the instance arrays */
    const uint32_t *inst_cell;     /* n_inst */
    const uint32_t *inst_pin_start;/* n_inst + 1, into inst_pin_net */
    const uint32_t *inst_pin_net;  /* per instance: n_in input nets, then n_out output nets */
    const uint32_t *inst_arc_start;/* n_inst + 1, into arcs */
    const gls_arc *arcs;
} gls_netlist;

/* Change-only waveforms of the nets the VCD drives (the per-signal time /
 * value vectors of VCDParser, src/VCDParser.h:46-57), plus constant nets
 * (a single event at time 0).  Times strictly increase within a net. */
typedef struct {
    uint32_t n_nets;
    const uint32_t *net;           /* netlist net ids */
    const uint64_t *ev_start;      /* n_nets + 1 */
    const uint32_t *time;
    const uint8_t *value;
} gls_stimulus;

typedef struct {
    uint64_t gate_events;     /* sum over gate outputs of fan-in events */
    uint64_t output_events;   /* events written to gate outputs */
    uint64_t segments;        /* time segments simulated */
    uint64_t pool_events;     /* event-pool capacity in use */
    uint64_t pool_bytes;      /* device bytes held by the pool */
    uint64_t overflow_retries;/* pool regrowths */
    double kernel_ms;         /* device time of the last gls_run */
    uint32_t launches;        /* kernels launched by the last gls_run */
    uint32_t n_windows;
    /* with opts.profile: device time per kernel class in the last gls_run */
    double plan_ms, sim_ms, combine_ms, stim_ms;
    uint64_t fanin_bytes;     /* fan-in event bytes the gate kernels read (5 B per event per net) */
    uint64_t presize_overflows; /* GLS_ALLOC_LEARNED: gate outputs longer than their predicted slot */
    uint64_t pool_used;       /* events allocated in the pool (stimulus + gate-output slots) */
    uint64_t wide_windows;    /* windows run with 64-bit event words (a time past 2^30 - 2) */
} gls_stats;

/* Create a context on opts->device.  Replaces cudaSetDevice(0) and the
 * constant uploads of src/simulate.cu:1897-1957. */
int gls_create(const gls_opts *opts, gls_ctx **out);
int gls_destroy(gls_ctx *ctx);
const char *gls_last_error(const gls_ctx *ctx);

/* Copy the levelized netlist to the device and build per-gate truth tables
 * and arc tables.  Replaces the archive load and the level-invariant uploads
 * of src/simulate.cu:1835-1957 (inter.dat fields listed above). */
int gls_load_netlist(gls_ctx *ctx, const gls_netlist *nl);

/* Add a stimulus window (SAIF integral over [t_begin, t_end)).  Replaces
 * VCDParser::parse/process and the per-level H2D staging of primary inputs
 * (src/simulate.cu:1974-1989, 2166-2219, 2441-2477).  Event times (stimulus
 * and gate outputs) reach 2^32 - 2, the 32-bit times of the reference GPU
 * tool: a window whose times stay within 2^30 - 2 runs in 32-bit event
 * words, a later time switches it to 64-bit words (twice the pool bytes;
 * the window runs alone, never in a wave of gls_run_batched).  A stimulus
 * time of 2^32 - 1 is GLS_ERANGE here, a gate output past 2^32 - 2 is
 * GLS_ERANGE from the run. */
int gls_add_window(gls_ctx *ctx, const gls_stimulus *stim, uint64_t t_begin,
                   uint64_t t_end, uint32_t *window_id);
int gls_clear_windows(gls_ctx *ctx);

/* Simulate every added window through all levels.  Replaces the per-level
 * loop src/simulate.cu:2027-3254 (merge, SimulateCuda, compaction, D2H).
 * Windows run one after the other. */
int gls_run(gls_ctx *ctx);

/* Batched windows (no counterpart in the reference, which takes one VCD
 * window per process): the added windows run in waves, each level of a wave
 * one launch per kernel over all its windows; results equal gls_run's. */
typedef struct {
    uint32_t max_wave;   /* windows per wave (0: all, or as many as device memory holds with saif_only) */
    int use_graph;       /* 1: capture a wave's launches once as a CUDA graph and replay it for every wave */
    int saif_only;       /* 1: free each window's event pool after its wave; SAIF counts and list lengths
                            stay readable, gls_waveform does not */
} gls_batch_opts;
int gls_run_batched(gls_ctx *ctx, const gls_batch_opts *opts);

/* Autotuner: runs the first wave of the added windows (as gls_run_batched
 * would form it; a single window works too) under candidate schedules and
 * keeps the fastest for the context's later runs: first time segments per
 * SM for the thread-per-segment gate kernel (1024, 2048, 4096) times the
 * fan-in classes that run warp-per-segment (none, 1-input, 1- to 3-input),
 * then, on the best of those, each of priority class streams, 256-thread
 * gate-kernel blocks, wider event loads, and both of the last two (13
 * candidates), and with GLS_ALLOC_LEARNED the learned balance of segments
 * (14).  Results never depend on the schedule. */
#define GLS_SCHED_CLASS_PRIORITY 1u   /* wider fan-in classes on higher-priority streams */
#define GLS_SCHED_BLOCK256 2u         /* thread-per-segment gate kernels in blocks of 256 threads (else 128) */
#define GLS_SCHED_WIDE_LOADS 4u       /* thread-per-segment gate kernels load 4 events at a time for 1- and
                                         2-input gates, 2 for wider ones (else 2 and 1) */
#define GLS_SCHED_LEARNED_BALANCE 8u  /* GLS_ALLOC_LEARNED: segments cut to equal predicted work, fan-in
                                         events plus half the presize network's predicted output events
                                         (GLS_BALANCE_WEIGHT sets another factor) */
typedef struct {
    uint32_t n;               /* candidates tried */
    uint32_t best;            /* index of the one kept */
    uint32_t windows;         /* windows in the timed wave */
    uint32_t seg_per_sm[32];
    uint32_t warp_mask[32];
    uint32_t flags[32];       /* GLS_SCHED_* */
    float ms[32];             /* device time of the wave under each (best of two runs) */
} gls_tune_result;
int gls_autotune(gls_ctx *ctx, const gls_batch_opts *opts, gls_tune_result *res);
/* Set the schedule by hand (e.g. one gls_autotune found for another context
 * on the same netlist): time segments per SM for the thread-per-segment gate
 * kernel (64..65536), which fan-in classes run warp-per-segment (bits 0-2
 * for 1-, 2- and 3-input gates), and GLS_SCHED_* flags. */
int gls_set_schedule(gls_ctx *ctx, uint32_t seg_per_sm, uint32_t warp_mask, uint32_t flags);

/* T0 / T1 / TX per net for a window (arrays of n_nets).  Nets the run did
 * not produce read UINT64_MAX.  Replaces the SAIF integrals of
 * src/simulate.cu:174-253, 1592-1677 (serial: src/simulate.cpp:102-163). */
int gls_saif_counts(gls_ctx *ctx, uint32_t window, uint64_t *t0, uint64_t *t1,
                    uint64_t *tx);
/* The same counts as one table of n_nets rows (T0, T1, TX): the device's
 * own layout, read back in one copy.  No counterpart in the reference. */
int gls_saif_table(gls_ctx *ctx, uint32_t window, uint64_t *t3);

/* Number of events of every net (n_nets), UINT32_MAX where not produced. */
int gls_waveform_lengths(gls_ctx *ctx, uint32_t window, uint32_t *len);

/* One net's change list.  *n receives its length; up to cap events are
 * copied.  Replaces the per-level D2H of src/simulate.cu:3207-3222. */
int gls_waveform(gls_ctx *ctx, uint32_t window, uint32_t net, uint32_t *time,
                 uint8_t *value, uint64_t cap, uint64_t *n);

int gls_stats_get(gls_ctx *ctx, gls_stats *st);

/* Host helper: the truth table of output `out` of a cell under calc_mode,
 * 4^n_in entries indexed by sum(value[pin] << 2*pin).  Evaluates the
 * primitive program like RunFunction, src/simulate.cpp:1203-1363. */
int gls_cell_lut(const gls_cell *cell, const gls_prim *prims, int out,
                 int calc_mode, uint8_t *lut, uint32_t lut_cap);

int gls_abi_version(void);

/* The reference's packed per-level arrays (src/process.cpp:423-566),
 * computed on device `device`: the tables `process` archives for its GPU
 * simulator.  Instances are given in level order: level L holds
 * [level_start[L], level_start[L + 1]).  Per instance: its input and output
 * net counts, its delay arcs (arc_start CSR into arcs: the edge, the arc's
 * input and output as positions in the instance's input / output net lists
 * (the list's length when absent) and the rise / fall values) and its
 * function program (row_start CSR into rows; row r holds the entries
 * [entry_start[r], entry_start[r + 1]) of entries).
 *
 * Outputs, as the reference fills them (per level: starts and widths; per
 * instance: counts; padded per level: delay and function tables, -1 where
 * an instance has fewer entries than its level's width).  The padded
 * tables need delay_total and functions_total entries: a call whose caps
 * are smaller writes the two totals and returns GLS_EOVERFLOW, so a caller
 * may size them with a first call. */
typedef struct {
    int16_t edge, in_pos, out_pos, pad;
    float rise, fall;
} gls_pack_arc;
typedef struct {
    uint32_t n_levels, n_inst;
    const uint32_t *level_start;     /* n_levels + 1 */
    const uint16_t *n_in, *n_out;    /* n_inst */
    const uint32_t *arc_start;       /* n_inst + 1 */
    const gls_pack_arc *arcs;
    const uint32_t *row_start;       /* n_inst + 1 */
    const uint32_t *entry_start;     /* rows + 1 */
    const int16_t *entries;
} gls_pack_in;
typedef struct {
    /* n_levels each */
    uint32_t *data_in_num_start, *data_out_num_start, *delay_start, *delay_width, *functions_start,
        *functions_width;
    /* n_inst each */
    int16_t *data_in_num, *data_out_num;
    uint32_t *val_num_start;
    int16_t *delay_val_num, *functions_func_num, *functions_val_num;
    /* delay_cap entries each */
    int16_t *delay_edges, *in_bit, *out_bit;
    float *rise_val, *fall_val;
    int16_t *functions;              /* functions_cap entries */
    uint64_t delay_cap, functions_cap;
    uint64_t delay_total, functions_total;   /* written */
} gls_pack_out;
int gls_pack_levels(int device, const gls_pack_in *in, gls_pack_out *out);

/* Kahn levels of an instance graph, computed on device `device` (replaces
 * GenerateAdjacencyList / SetInDegrees / TopologyOrder, src/process.cpp:
 * 90-176; gls_pack_levels does the packing of 423-566).  pred_start[n_inst + 1]
 * (pred_start[0] = 0, nondecreasing) and pred[] list every instance's
 * predecessors: the instances driving its input nets (repeats are
 * harmless).  Level 0 holds the instances without predecessors; every
 * later level the instances whose predecessors are all placed, in instance
 * order.  order[n_inst] receives the instances level by level,
 * level_start[] (room for n_inst + 1 entries) the first position of every
 * level followed by n_inst, *n_levels the number of levels.  GLS_EINVAL for
 * a malformed table, a predecessor out of range, or a combinational loop
 * (the reference degrades a loop to one instance per level,
 * src/process.cpp:143-155). */
int gls_levelize(int device, uint32_t n_inst, const uint64_t *pred_start,
                 const uint32_t *pred, uint32_t *order, uint32_t *level_start,
                 uint32_t *n_levels);

/* VCD body scan on the GPU (replaces VCDParser::parse_core / combine_core /
 * core, src/VCDParser.cpp:508-644, 458-507, 194-242, for the text after
 * $enddefinitions; the header stays with the caller).  The identifier codes
 * of the header's $var lines, at most 8 bytes each, as little-endian keys
 * (zero-padded), strictly increasing; var_start[n_ids + 1] their
 * declarations; bit_start[n_vars + 1] each declaration's bits (msb first),
 * bits[] the signal of every bit, bus[n_vars] 1 for a bus declaration. */
typedef struct gls_vcd_ids {
    uint32_t n_ids;
    const uint64_t *key;
    const uint32_t *var_start;
    const uint32_t *bit_start;
    const uint32_t *bits;
    const uint8_t *bus;
} gls_vcd_ids;
/* Every bit change in file order: signal, time in force, value (0, 1=X,
 * 2=Z, 3; 255 for a character that is no value, which the reference
 * skips) and whether the bit belongs to a bus declaration (the caller keeps
 * only real changes of those, starting from Z, and lets a later change at
 * the same time replace an earlier one, as the reference does).
 * fallback = 1: the body reads differently token by token (an identifier
 * code equal to $comment or $end); parse it on the host instead. */
typedef struct gls_vcd_changes {
    uint64_t n;
    uint32_t *signal;
    uint64_t *time;
    uint8_t *value;
    uint8_t *bus;
    int fallback;
} gls_vcd_changes;
/* Scan n_bytes (< 2^32 - 2^16) of body text on device `device`; the arrays of
 * *out are allocated by the library, released by gls_vcd_free. */
int gls_vcd_scan(int device, const char *body, uint64_t n_bytes, const gls_vcd_ids *ids,
                 gls_vcd_changes *out);
void gls_vcd_free(gls_vcd_changes *out);

/* ---------------------------------------------------------------------
 * Learned presize.  No counterpart in the reference, which sizes every
 * gate output from its fan-in rows (src/simulate.cu:2300-2306) and then
 * compacts (src/simulate.cu:1104-1357).
 *
 * A multilayer perceptron 32 -> 128 -> 128 -> 1 (ReLU) maps a gate
 * output's features to y ~ log(1 + length of its output list).  Features,
 * in order: 0-12 one-hot cell index (cells 0..12 of the netlist); 13 input
 * pins / 6; 14 distinct input nets / 6; 15-17 log(1 + events) of input nets
 * 0-2 / 12; 18 log(1 + sum of input events) / 12; 19 log(1 + max) / 12;
 * 20 log(1 + min) / 12; 21 log(1 + expected output changes) / 12, where
 * every input change counts with the probability that the other inputs
 * sensitize the output to it (truth table, inputs independent, each at 1
 * for its SAIF share T1 / (T0 + T1)); 22 the probability that the output is
 * 1 under the same assumption; 23 the mean 1-share of the inputs; 24 mean rise, 25 mean fall, 26 min, 27 max arc delay
 * (time units / 100); 28 log(1 + fan-out) / 6; 29 the fraction of single
 * input changes that change the output (from the truth table); 30 1 when
 * every input net has a simple arc set; 31 constant 1.
 * In GLS_ALLOC_LEARNED mode every level first runs the network on the
 * tensor cores (BF16 operands, FP32 accumulation) and reserves
 *   min(fan-in events + 1, ceil((exp(y) - 1) * (1 + margin)) + slack)
 * events per gate output.
 * --------------------------------------------------------------------- */
#define GLS_MLP_IN 32
#define GLS_MLP_HID 128
#define GLS_MLP_PARAMS (GLS_MLP_HID * GLS_MLP_IN + GLS_MLP_HID + GLS_MLP_HID * GLS_MLP_HID + GLS_MLP_HID + GLS_MLP_HID + 1)

typedef struct {
    /* FP32 parameters in this order: w1[128][32], b1[128], w2[128][128],
     * b2[128], w3[128], b3 (row = output unit).  Inference rounds w1 and w2
     * to BF16. */
    float params[GLS_MLP_PARAMS];
    float margin;      /* relative slack on the predicted length */
    uint32_t slack;    /* absolute slack, events */
} gls_presize_model;

/* Install the model used by GLS_ALLOC_LEARNED (copied). */
int gls_set_presize_model(gls_ctx *ctx, const gls_presize_model *model);

/* Training pairs from a finished window: for every gate output (the
 * library's driver order) its 32 features as the learned mode computes them
 * and the length of its output list.  feat holds cap x 32 floats, count cap
 * entries; *n receives the number of gate outputs. */
int gls_presize_samples(gls_ctx *ctx, uint32_t window, float *feat, uint32_t *count, uint64_t cap,
                        uint64_t *n);

/* Run a model on host feature rows: y (n floats).  tensor_cores = 1 uses the
 * kernel of the learned mode (BF16 tcgen05), 0 an FP32 CUDA-core kernel. */
int gls_presize_predict(gls_ctx *ctx, const gls_presize_model *model, const float *feat, uint64_t n,
                        float *y, int tensor_cores);

/* Training on the GPU (FP32, Adam, Huber loss on y - log(1 + count)). */
typedef struct gls_trainer gls_trainer;
typedef struct {
    uint32_t batch;        /* rows per step */
    uint32_t epochs;
    float lr;              /* Adam step size */
    float huber;           /* Huber threshold on the log-length error */
    uint64_t seed;         /* shuffling and initialization */
} gls_train_opts;

int gls_trainer_create(int device, uint64_t seed, gls_trainer **out);
int gls_trainer_destroy(gls_trainer *tr);
const char *gls_trainer_error(const gls_trainer *tr);
/* Copy n training rows (feat n x 32, target n = log(1 + count)) to the device. */
int gls_trainer_set_data(gls_trainer *tr, const float *feat, const float *target, uint64_t n);
/* Train; loss receives the mean loss of every epoch (opts->epochs floats). */
int gls_trainer_fit(gls_trainer *tr, const gls_train_opts *opts, float *loss);
/* Loss and gradient of every parameter (GLS_MLP_PARAMS floats) over rows
 * [first, first + n) of the data, without updating (for gradient checks). */
int gls_trainer_grad(gls_trainer *tr, uint64_t first, uint64_t n, float huber, float *grad, float *loss);
int gls_trainer_get_params(gls_trainer *tr, float *params);
int gls_trainer_set_params(gls_trainer *tr, const float *params);

/* Simulate gate outputs [first, first + count) of one level (in the
 * library's order inside the level; count up to the level's number of gate
 * outputs) without allocating any device memory.  This entry point has no
 * counterpart in the reference.
 *
 * It is for callers that cannot call cudaMalloc while they simulate, e.g.
 * an application that owns all device memory through its own arena, or a
 * latency-bound loop that cannot pay the device synchronization that
 * cudaMalloc / cudaFree can cause.  Such a caller passes its own device
 * buffers for the inputs and outputs:
 *   d_pool     the event pool, one 32-bit word per event, time << 2 | value
 *              (times up to 2^30 - 2); every change list starts on a 4-word
 *              boundary and its allocation is padded to a multiple of 4 words
 *   pool_cap   capacity of d_pool in words
 *   d_top      one 64-bit word: first free pool word; output lists are
 *              appended there (4-word aligned) and it is advanced
 *   d_net_off / d_net_len   per net: pool offset and length; read for the
 *              gate inputs, written for the gate outputs
 *   d_saif     3 x 64-bit per net (T0, T1, TX over [t_begin, t_end)),
 *              written for the gate outputs
 * The segment stacks and segment tables live in one static device array of
 * 20,775,936 bytes (about 20 MiB) that every GPU loading the library holds
 * until exit.  One
 * call handles at most 16384 gate outputs, 65536 time segments and
 * 4194304 segment-stack words; larger requests fail with GLS_ERANGE and a
 * message (pass fewer outputs per call).  A call that fails leaves d_top,
 * d_net_off, d_net_len and d_saif as they were, so it can be retried with
 * fewer outputs.  The call waits for its kernels (on the context's stream)
 * to finish.  The first call on a device looks up the static array's device
 * address, which (with CUDA's default lazy module loading) is also when the
 * array is reserved on that device: make that first call before any stream
 * capture and before an arena takes the remaining device memory; if the
 * array cannot be reserved the call fails with GLS_ENOMEM.  All calls on a
 * device share the array: calls that overlap on the GPU (other threads,
 * other contexts of the same device) race and must be serialized by the
 * caller. */
int gls_run_level_static(gls_ctx *ctx, uint32_t level, uint32_t first, uint32_t count,
                         uint32_t *d_pool, uint64_t pool_cap, unsigned long long *d_top,
                         uint64_t *d_net_off, uint32_t *d_net_len,
                         unsigned long long *d_saif, uint64_t t_begin, uint64_t t_end);

#ifdef __cplusplus
}
#endif

#endif /* GLS_H */
