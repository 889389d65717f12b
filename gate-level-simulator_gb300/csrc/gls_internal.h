// Internal device-side data model of libgls (not part of the C ABI).
//
// HBM layout for one stimulus window:
//   pool_t[u32] / pool_v[u8]  structure-of-arrays event pool; every net's
//                             change list is a contiguous run starting on a
//                             4-event (16-byte) boundary.
//   net_off[u64] / net_len[u32]  per net CSR into the pool.
//   saif[u64 x 3]             T0 / T1 / TX per net.
// Netlist (shared by all windows):
//   DrvMeta per gate output ("driver"), ordered by level; Arc table; LUT
//   table of 2-bit cell truth tables stored one value per byte.
#pragma once
#include <cstdint>

namespace gls {

constexpr int kMaxSlots = 6;        // distinct fan-in nets per gate (MAX_IN_NUM, src/simulate.cu:25)
constexpr int kMaxPins = 6;         // cell inputs covered by a LUT (4^6 entries)
constexpr uint32_t kInf = 0xFFFFFFFFu;
constexpr uint8_t kV0 = 0, kVX = 1, kVZ = 2, kV1 = 3;

// error bits raised by kernels
constexpr uint32_t kErrPool = 1u;       // event pool exhausted
constexpr uint32_t kErrRegion = 2u;     // segment region overflow (internal invariant)
constexpr uint32_t kErrEmptied = 4u;    // output list emptied (zero delay at t=0)
constexpr uint32_t kErrSegCap = 8u;     // segment table too small
constexpr uint32_t kErrTime = 16u;      // a time reached 2^32-1

struct DrvMeta {            // one gate output; 48 bytes
    uint32_t out_net;
    uint32_t lut_off;       // byte offset of this output's truth table
    uint32_t arc_off;       // first arc
    uint32_t pin_slot;      // 3 bits per pin: distinct-net slot feeding pin p
    uint8_t n_pins, m, n_arcs, ident;   // ident: slot p feeds pin p for every p
    uint32_t net[kMaxSlots];
    uint32_t reserved;
};
static_assert(sizeof(DrvMeta) == 48, "DrvMeta layout");

struct ArcDev {             // info = edge | slot << 2 ; delays already scaled and truncated
    uint32_t info, rise, fall, pad;
};

struct SegRec {             // one time segment of one gate output
    uint32_t region;        // offset of the segment's stack inside the gate's slot
    uint32_t cnt;           // entries on the segment's local stack
    uint32_t min_o;         // smallest candidate output time in the segment
    uint32_t fin;           // entries kept after combine
};

struct WinDev {
    uint64_t *net_off;
    uint32_t *net_len;
    uint32_t *pool_t;
    uint8_t *pool_v;
    unsigned long long *saif;   // 3 per net
    unsigned long long *top;    // pool bump pointer (events)
    unsigned long long *counters;  // [0] gate events, [1] output events, [2] segments, [3] fan-in events
    uint32_t *err;
    uint32_t *seg_base;         // per driver of the level, +1
    uint64_t *slot;             // per driver of the level: slot start in the pool
    SegRec *segs;
    uint32_t *n_segs;
    uint64_t cap;               // pool capacity (events)
    uint32_t seg_cap;           // SegRec capacity
    uint64_t t_begin, t_end;
};

struct LevelArgs {
    const DrvMeta *meta;
    const ArcDev *arcs;
    const uint8_t *lut;
    uint32_t lo, hi;            // driver range of the level
    uint32_t seg_events;        // target fan-in events per segment
    uint32_t def_delay;         // delay used when no arc applies
};

void launch_stim_saif(const WinDev &w, const uint32_t *stim_nets, uint32_t n_stim, cudaStream_t st);
void launch_plan(const WinDev &w, const LevelArgs &a, cudaStream_t st);
void launch_sim(const WinDev &w, const LevelArgs &a, int sm_count, cudaStream_t st);
void launch_combine(const WinDev &w, const LevelArgs &a, cudaStream_t st);

}  // namespace gls
