// Internal device-side data model of libgls (not part of the C ABI).
//
// HBM layout for one stimulus window:
//   pool[u32]        the event pool: every event is one word,
//                    time << 2 | value (value 0, X=1, Z=2, 1=3), so a
//                    16-byte load brings four events; every net's change
//                    list is a contiguous run starting on a 4-event
//                    boundary, its allocation padded to whole chunks.
//   net_off[u64] / net_len[u32]  per net CSR into the pool.
//   saif[u64 x 3]    T0 / T1 / TX per net.
// Netlist (shared by all windows):
//   DrvMeta per gate output ("driver"), ordered by level and, inside a
//   level, by fan-in class; arc and per-net delay tables; the LUT table of
//   cell truth tables, one 2-bit value per byte.
#pragma once
#include <cstdint>

namespace gls {

constexpr int kMaxSlots = 6;        // distinct fan-in nets per gate (MAX_IN_NUM, src/simulate.cu:25)
constexpr int kMaxPins = 6;         // cell inputs covered by a LUT (4^6 entries)
constexpr uint32_t kInf = 0xFFFFFFFFu;
constexpr uint32_t kMaxTime = (1u << 30) - 2;   // largest event time a 32-bit word can carry
constexpr uint32_t kMaxTimeWide = 0xFFFFFFFEu;  // largest event time of a 64-bit word (times stay 32-bit)
constexpr uint8_t kV0 = 0, kVX = 1, kVZ = 2, kV1 = 3;
constexpr int kClasses = 4;         // fan-in classes: 1, 2, 3, 4..6 distinct input nets

// An event is one word, time << 2 | value.  A window whose times fit 30
// bits uses 32-bit words; a window with later times (up to 2^32 - 2, the
// reference GPU tool's 32-bit range) uses 64-bit words.
using WideWord = unsigned long long;
__host__ __device__ inline uint32_t ev_word(uint32_t t, uint32_t v) { return (t << 2) | v; }
__host__ __device__ inline uint32_t ev_time(uint32_t w) { return w >> 2; }
__host__ __device__ inline uint32_t ev_val(uint32_t w) { return w & 3u; }
__host__ __device__ inline uint32_t ev_time(WideWord w) { return (uint32_t)(w >> 2); }
__host__ __device__ inline uint32_t ev_val(WideWord w) { return (uint32_t)w & 3u; }
template <class Wd> struct EvW;
template <> struct EvW<uint32_t> {
    static constexpr uint32_t kMax = kMaxTime;      // largest event time
    static constexpr uint32_t kInfW = 0xFFFFFFFFu;  // above every event word
    __host__ __device__ static uint32_t word(uint32_t t, uint32_t v) { return (t << 2) | v; }
};
template <> struct EvW<WideWord> {
    static constexpr uint32_t kMax = kMaxTimeWide;
    static constexpr WideWord kInfW = ~0ull;
    __host__ __device__ static WideWord word(uint32_t t, uint32_t v) { return ((WideWord)t << 2) | v; }
};

// error bits raised by kernels
constexpr uint32_t kErrPool = 1u;       // event pool exhausted
constexpr uint32_t kErrRegion = 2u;     // segment region overflow (internal invariant)
constexpr uint32_t kErrEmptied = 4u;    // output list emptied (zero delay at t=0)
constexpr uint32_t kErrSegCap = 8u;     // segment table too small
constexpr uint32_t kErrTime = 16u;      // an output time passed the largest time its event word holds
constexpr uint32_t kErrScratch = 32u;   // level scratch exhausted
constexpr uint32_t kErrPresize = 64u;   // the tensor-core presize kernel gave up waiting for its MMA

// output slot allocation (GLS_ALLOC_*): an upper bound reserved before the
// level runs; the exact length once the level's stacks are linked; or a
// predicted length, with the exact placement for gates that outgrow it
constexpr uint32_t kAllocBound = 0, kAllocExact = 1, kAllocLearned = 2;

constexpr uint8_t kFlagIdent = 1;    // slot p feeds pin p for every pin
constexpr uint8_t kFlagRegular = 2;  // every input net has no arc, one both-edge arc, or a posedge/negedge pair
constexpr uint8_t kFlagFirstOut = 4; // first output of its instance (gate-event accounting)

struct DrvMeta {            // one gate output; 48 bytes
    uint32_t out_net;
    uint32_t lut_off;       // byte offset of this output's truth table
    uint32_t arc_off;       // first arc (irregular outputs)
    uint32_t pin_slot;      // 3 bits per pin: distinct-net slot feeding pin p
    uint8_t n_pins, m, n_arcs, flags;
    uint32_t net[kMaxSlots];
    uint32_t dt_off;        // first per-net delay entry (regular outputs)
};
static_assert(sizeof(DrvMeta) == 48, "DrvMeta layout");

struct ArcDev {             // info = edge | slot << 2 ; delays already scaled and truncated
    uint32_t info, rise, fall, pad;
};

// Per input net of a regular gate output: the delay an event on that net
// selects, d[e * 4 + s - 1] for input edge e (0 rising, 1 falling, as
// CheckDelay classes it) and output sense s (1 rise, 2 fall, 3 X->Z, 4 Z->X);
// kInf where no arc applies.
struct NetDelay {
    uint32_t d[8];
};

// CheckDelay (src/simulate.cpp:1178-1201) as a function of (pre, cur)
__host__ __device__ constexpr int sense_of(uint32_t pre, uint32_t cur)
{
    return ((pre == kV0 && cur != kV0) || (cur == kV1 && pre != kV1)) ? 1
         : ((pre == kV1 && cur != kV1) || (cur == kV0 && pre != kV0)) ? 2
         : (pre == kVX && cur == kVZ) ? 3
         : (pre == kVZ && cur == kVX) ? 4 : 0;
}
// 3 bits per (pre * 4 + cur): the sense
__host__ __device__ constexpr uint64_t sense_table()
{
    uint64_t t = 0;
    for (uint32_t k = 0; k < 16; ++k) t |= (uint64_t)sense_of(k >> 2, k & 3u) << (3 * k);
    return t;
}
// 1 bit per (last * 4 + cur): the input counts as a falling edge (sense 2)
__host__ __device__ constexpr uint32_t neg_table()
{
    uint32_t t = 0;
    for (uint32_t k = 0; k < 16; ++k) t |= (sense_of(k >> 2, k & 3u) == 2 ? 1u : 0u) << k;
    return t;
}
constexpr uint64_t kSenseTab = sense_table();
// 2 bits per (pre * 4 + cur), pre != cur: the sense minus one (a change
// always has sense 1..4; entries with pre == cur are 0 and never read)
__host__ __device__ constexpr uint32_t sense1_table()
{
    uint32_t t = 0;
    for (uint32_t k = 0; k < 16; ++k)
        if ((k >> 2) != (k & 3u)) t |= (uint32_t)(sense_of(k >> 2, k & 3u) - 1) << (2 * k);
    return t;
}
constexpr uint32_t kSense1Tab = sense1_table();
static_assert(sense_of(kV0, kVX) == 1 && sense_of(kVX, kV0) == 2 && sense_of(kVX, kVZ) == 3 && sense_of(kVZ, kVX) == 4,
              "sense classes");
// delays are stored capped at kMaxTimeWide: an output time past it is an
// error whichever arc gives it (the kernels add t + d in 64 bits, or check
// the 32-bit sum for wrap-around), and kInf stays free to mean "no arc"
constexpr uint32_t kMaxDelay = kMaxTimeWide;
constexpr uint32_t kNegTab = neg_table();

template <class Wd>
struct SegRecT {            // one time segment of one gate output
    uint32_t region;        // offset of the segment's stack inside the gate's scratch
    uint32_t cnt;           // entries on the segment's local stack
    uint32_t min_o;         // smallest candidate output time in the segment
    Wd last;                // the stack's top entry (when cnt > 0): linking reads no scratch for it
};
using SegRec = SegRecT<uint32_t>;
constexpr size_t kSegRecMax = sizeof(SegRecT<WideWord>);   // table entries are sized for either word

struct CopyRec {            // what k_copy does for one segment
    uint64_t src;           // scratch index of the first kept entry
    uint64_t dst;           // pool index of that entry (bound mode), else its position in the gate output's list
    uint32_t n;             // entries to copy (k_link keeps the cut count here between its passes)
    uint32_t drv;           // gate output (level-relative)
    unsigned long long cprev;  // clamped time of the final event before this segment's first
    uint32_t pclass;        // value class of that event (0: 0, 1: 1, 2: X or Z)
    uint32_t out_net;       // the gate output's net
};

struct WinDev {
    uint64_t *net_off;
    uint32_t *net_len;
    uint32_t *pool;
    unsigned long long *saif;   // 3 per net
    unsigned long long *top;    // pool bump pointer (events)
    unsigned long long *counters;  // [0] gate events, [1] output events, [2] segments, [3] fan-in events
    uint32_t *err;
    uint32_t *seg_base;         // per driver of the level, +1
    uint64_t *slot;             // per driver of the level: final-list slot in the pool
    uint64_t *scr;              // per driver of the level: segment stacks in the scratch
    SegRec *segs;
    CopyRec *copies;            // per segment, written by k_link
    uint32_t *n_segs;
    uint32_t *res;              // per driver of the level: events reserved in its slot (exact / learned modes)
    unsigned long long *n_over; // gate outputs placed exactly because the presize was short (learned mode)
    uint32_t *pred;             // per driver of the level: predicted slot length (learned mode)
    const uint32_t *stim_nets;  // nets the stimulus drives
    uint32_t *scratch;          // level scratch: segment stacks (event words)
    uint64_t cap;               // pool capacity (events)
    uint64_t scr_cap;           // scratch capacity (events)
    uint64_t t_begin, t_end;
    uint32_t seg_cap;           // SegRec capacity
    uint32_t n_stim;
};
static_assert(sizeof(WinDev) <= 192, "WinDev fits the static entry point's descriptor slot");

struct LevelArgs {
    const DrvMeta *meta;
    const uint4 *slut;          // per driver with at most 3 input nets: truth table over its input nets' values,
                                // 2 bits per entry, entry = sum(value(net j) << 2j) (64 entries in 128 bits)
    const ArcDev *arcs;
    const NetDelay *ndel;
    const uint8_t *lut;
    uint32_t lo, hi;            // driver range of the level
    uint32_t seg_events;        // fan-in events per segment (0: sized to fill the GPU)
    uint32_t seg_target;        // segments per class to aim for (thread-per-segment kernels)
    uint32_t seg_target_w;      // segments per class to aim for (warp-per-segment kernels)
    uint32_t warp_mask;         // bit c: fan-in class c runs the warp-per-segment kernel
    uint32_t def_delay;         // delay used when no arc applies
    uint32_t alloc_mode;        // kAllocBound / kAllocExact / kAllocLearned
    uint32_t copy_lanes;        // lanes per segment in the copy kernel (4, 8, 16 or 32)
    unsigned long long *wave_e; // wave of windows: fan-in events of the level per class over all windows (else null)
    uint32_t wide;              // 1: the window holds 64-bit event words (one window per launch)
    uint32_t sim_variant;       // thread-per-segment gate kernel variant: bit 0 256-thread blocks, bit 1 wider loads
    float bal_weight;           // learned mode: segment work = fan-in events + bal_weight * predicted output events
    uint32_t plan_part;         // k_plan: 0 all of it; learned mode split in two: 1 segments and stacks
                                // (slots left open), 2 slot placement from the predictions
};

// Windows simulated together: every level kernel takes a device array of
// WinDev and covers all of them in one launch (at most kMaxWave).
constexpr uint32_t kMaxWave = 1024;

// fan-in class of a gate output by its number of distinct input nets
__host__ __device__ inline int fanin_class(int m) { return m <= 1 ? 0 : (m == 2 ? 1 : (m == 3 ? 2 : 3)); }

// A launch covers nwin windows: `h` is window 0's descriptor on the host
// (used when nwin == 1), `dw` the device array of all nwin descriptors.
void launch_stim_saif(const WinDev *dw, const WinDev &h, uint32_t nwin, uint32_t max_stim, bool wide,
                      cudaStream_t st);
void launch_plan(const WinDev *dw, const WinDev &h, uint32_t nwin, const LevelArgs &a, cudaStream_t st);
// a wave's fan-in events per class into a.wave_e (cleared before), so every
// window of the wave cuts its segments to the same size
void launch_wave_events(const WinDev *dw, uint32_t nwin, const LevelArgs &a, cudaStream_t st);
void launch_sim(const WinDev *dw, const WinDev &h, uint32_t nwin, const LevelArgs &a, int cls, uint32_t d0, uint32_t d1,
                int sm_count, cudaStream_t st);
// link and copy the gate outputs [d0, d1) of the level (level-relative)
void launch_link(const WinDev *dw, const WinDev &h, uint32_t nwin, const LevelArgs &a, uint32_t d0, uint32_t d1,
                 cudaStream_t st);
void launch_copy(const WinDev *dw, const WinDev &h, uint32_t nwin, const LevelArgs &a, uint32_t d0, uint32_t d1,
                 int sm_count, cudaStream_t st);

}  // namespace gls
