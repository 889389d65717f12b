// Level kernels of the GB300 gate-level simulator (sm_103a).
//
// One level of gates is simulated by four kinds of launches:
//   k_plan     (1 CTA)   sizes every gate output's slot in the event pool and
//                        its segment stacks in the level scratch, and splits
//                        its fan-in timeline into time segments.
//   k_sim<M>   (1 thread per segment, one instantiation per fan-in class)
//                        merges the segment's fan-in events, evaluates the
//                        cell truth table, picks the SDF delay and runs the
//                        inertial output stack of the reference serial
//                        simulator on the segment.
//   k_link     (1 warp per gate output, a lane per segment) applies the pops
//                        that later segments make into earlier ones, settles
//                        the one undecided duplicate at each segment bottom
//                        and places the segments in the gate's pool slot.
//   k_copy     (8 lanes per segment) moves the kept entries from the level
//                        scratch into the event pool and accumulates T0/T1/TX
//                        (fused SAIF).
//   k_sim_warp<M> (optional per fan-in class: a warp per segment) is the
//                        same contract as k_sim, merged by tiles.
//
// Semantics follow src/simulate.cpp:872-1506 of the reference.  Why the
// segment split is exact: a candidate output event k (time o_k) is removed
// from the output list iff some later candidate j has o_j <= o_k
// (src/simulate.cpp:991-1001); the push test (1002-1008) of a candidate that
// survives compares against the last surviving entry before it.  So a
// segment can run the stack locally, the entries of segment s are cut to
// those with o < min(o over all later segments), and a segment's first
// entry is dropped iff it repeats the value of the last kept entry before it.
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>
#include "gls_internal.h"

namespace gls {

__device__ __forceinline__ int check_delay(uint32_t pre, uint32_t cur)
{
    // CheckDelay, src/simulate.cpp:1178-1201
    if ((pre == kV0 && cur != kV0) || (cur == kV1 && pre != kV1)) return 1;
    if ((pre == kV1 && cur != kV1) || (cur == kV0 && pre != kV0)) return 2;
    if (pre == kVX && cur == kVZ) return 3;
    if (pre == kVZ && cur == kVX) return 4;
    return 0;
}

__device__ __forceinline__ uint32_t pick(uint32_t rise, uint32_t fall, int s)
{
    return s == 1 ? rise : s == 2 ? fall : s == 3 ? max(rise, fall) : min(rise, fall);
}

__device__ __forceinline__ uint32_t slot_val(uint32_t pack, int j) { return (pack >> (2 * j)) & 3u; }

// AddDelay, src/simulate.cpp:1012-1176, on delays pre-scaled by the time
// factor and truncated (truncation commutes with min/max on non-negative
// values, so selecting after truncation gives the same integer).
__device__ uint32_t select_delay(const ArcDev *__restrict__ arcs, int n_arcs, uint32_t chg, int so,
                                 uint32_t curp, uint32_t lastp, uint32_t defd)
{
    const int num_in = __popc(chg);
    if (num_in == 1) {
        int nrel = 0;
        ArcDev r0 = {0, 0, 0, 0};
        for (int a = 0; a < n_arcs; ++a) {
            ArcDev A = arcs[a];
            if (!((chg >> (A.info >> 2)) & 1u)) continue;
            if (nrel == 0) r0 = A;
            ++nrel;
        }
        if (nrel == 0) return defd;
        if (nrel == 1) return pick(r0.rise, r0.fall, so);
        const int j = r0.info >> 2;
        const int e = (check_delay(slot_val(lastp, j), slot_val(curp, j)) == 2) ? 1 : 0;
        for (int a = 0; a < n_arcs; ++a) {
            ArcDev A = arcs[a];
            if (!((chg >> (A.info >> 2)) & 1u)) continue;
            if ((int)(A.info & 3u) == e) return pick(A.rise, A.fall, so);
        }
        return defd;
    }
    uint32_t mn = kInf;
    bool any = false;
    for (int a = 0; a < n_arcs; ++a) {
        ArcDev A = arcs[a];
        const int j = A.info >> 2;
        if (!((chg >> j) & 1u)) continue;
        const int edge = A.info & 3u;
        if (edge != 2) {
            const int e = (check_delay(slot_val(lastp, j), slot_val(curp, j)) == 2) ? 1 : 0;
            if (e != edge) continue;
        }
        mn = min(mn, pick(A.rise, A.fall, so));
        any = true;
    }
    return any ? mn : defd;
}

// Delay of an active step of a regular gate output: the smallest delay the
// changed nets select for their own input edge and the output sense, or the
// default when none applies.  Equals AddDelay (src/simulate.cpp:1012-1176)
// whenever every input net has no arc, one both-edge arc, or one posedge and
// one negedge arc: then a single changed net selects exactly one arc (or
// none), and several changed nets take the minimum over their arcs.
template <int M>
__device__ __forceinline__ uint32_t regular_delay(const NetDelay *__restrict__ nd, uint32_t chg, uint32_t so1,
                                                  uint32_t curp, uint32_t lastp, uint32_t defd)
{
    uint32_t d = kInf;   // so1: the output sense minus one
    if (M > 1 && chg != 0u && (chg & (chg - 1u)) == 0u) {
        // one input net changed (most steps): one table entry, no loop
        const int j = __ffs(chg) - 1;
        const uint32_t neg = (kNegTab >> (slot_val(lastp, j) * 4 + slot_val(curp, j))) & 1u;
        d = __ldg(&nd[j].d[neg * 4 + so1]);
        return d == kInf ? defd : d;
    }
#pragma unroll
    for (int j = 0; j < M; ++j) {
        if ((chg >> j) & 1u) {
            const uint32_t neg = (kNegTab >> (slot_val(lastp, j) * 4 + slot_val(curp, j))) & 1u;
            d = min(d, __ldg(&nd[j].d[neg * 4 + so1]));
        }
    }
    return d == kInf ? defd : d;
}

__device__ __forceinline__ uint32_t lut_index(uint32_t curp, const DrvMeta &md)
{
    if (md.flags & kFlagIdent) return curp & ((1u << (2 * md.n_pins)) - 1u);
    uint32_t idx = 0;
    for (int p = 0; p < md.n_pins; ++p)
        idx |= slot_val(curp, (md.pin_slot >> (3 * p)) & 7u) << (2 * p);
    return idx;
}

// ------------------------------------------------------------------ plan
template <typename T>
__device__ T block_excl_scan(T x, T *total, T *sm)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) sm[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        T v = lane < nw ? sm[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        sm[lane] = v;
    }
    __syncthreads();
    T pre = wid ? sm[wid - 1] : T(0);
    *total = sm[31];
    __syncthreads();
    return pre + inc - x;
}

// One block per window of a wave: the level's fan-in events per fan-in class,
// summed over the wave into a.wave_e.
__global__ void __launch_bounds__(1024) k_wave_events(const WinDev *__restrict__ wv, LevelArgs a)
{
    __shared__ unsigned long long sm64[32];
    const WinDev &w = wv[blockIdx.x];
    const uint32_t n = a.hi - a.lo;
    unsigned long long e_cls[kClasses] = {0, 0, 0, 0};
    if (!*w.err) {
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            const DrvMeta &md = a.meta[a.lo + i];
            unsigned long long E = 0;
            for (int j = 0; j < md.m; ++j) E += w.net_len[md.net[j]];
            const int c = fanin_class(md.m);
#pragma unroll
            for (int k = 0; k < kClasses; ++k) if (k == c) e_cls[k] += E;
        }
    }
#pragma unroll
    for (int k = 0; k < kClasses; ++k) {
        unsigned long long tot;
        block_excl_scan<unsigned long long>(e_cls[k], &tot, sm64);
        if (threadIdx.x == 0 && tot) atomicAdd(&a.wave_e[k], tot);
    }
}

// The windows a launch covers: one window passed by value (kernel
// parameter space, no indirection in the hot loops), or a device array.
template <bool kBatch> struct WinSet;
template <> struct WinSet<false> {
    static constexpr bool kIsBatch = false;
    WinDev w;
    __device__ __forceinline__ const WinDev &get(uint32_t) const { return w; }
    __device__ __forceinline__ uint32_t size() const { return 1; }
};
template <> struct WinSet<true> {
    static constexpr bool kIsBatch = true;
    const WinDev *wv;
    uint32_t n;
    __device__ __forceinline__ const WinDev &get(uint32_t k) const { return wv[k]; }
    __device__ __forceinline__ uint32_t size() const { return n; }
};

// Exclusive block-wide scan of three quantities at once (two barriers for
// the three); *t* receive the block totals.
__device__ void block_excl_scan3(uint32_t &x, unsigned long long &y, unsigned long long &z, uint32_t &tx,
                                 unsigned long long &ty, unsigned long long &tz, uint32_t *sx,
                                 unsigned long long *sy, unsigned long long *sz)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t ix = x;
    unsigned long long iy = y, iz = z;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ux = __shfl_up_sync(FULL, ix, o);
        const unsigned long long uy = __shfl_up_sync(FULL, iy, o), uz = __shfl_up_sync(FULL, iz, o);
        if (lane >= o) { ix += ux; iy += uy; iz += uz; }
    }
    if (lane == 31) { sx[wid] = ix; sy[wid] = iy; sz[wid] = iz; }
    __syncthreads();
    if (wid == 0) {
        uint32_t vx = lane < nw ? sx[lane] : 0u;
        unsigned long long vy = lane < nw ? sy[lane] : 0ull, vz = lane < nw ? sz[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t ux = __shfl_up_sync(FULL, vx, o);
            const unsigned long long uy = __shfl_up_sync(FULL, vy, o), uz = __shfl_up_sync(FULL, vz, o);
            if (lane >= o) { vx += ux; vy += uy; vz += uz; }
        }
        sx[lane] = vx; sy[lane] = vy; sz[lane] = vz;
    }
    __syncthreads();
    const uint32_t px = wid ? sx[wid - 1] : 0u;
    const unsigned long long py = wid ? sy[wid - 1] : 0ull, pz = wid ? sz[wid - 1] : 0ull;
    tx = sx[31]; ty = sy[31]; tz = sz[31];
    __syncthreads();   // the arrays are reused by the next call
    x = px + ix - x; y = py + iy - y; z = pz + iz - z;
}

// gate outputs per thread in one round of k_plan's first pass (their loads overlap)
constexpr int kPlanPer = 4;

// one block per window
// Part 2 of a split plan (learned mode): every gate output's slot, sized
// from its prediction once the presize has run, placed by a block scan;
// the pool pointer moves only when the slots fit.  Part 1 left the gate
// output's fan-in events in the slot table as E << 2 | class.  The segment
// tables are already in use by the gate kernels: a failure only raises the
// window's flag, and its link and copy skip it.
__device__ void plan_slots(const WinDev &w, const LevelArgs &a, uint32_t n, uint32_t *sm32,
                           unsigned long long *sm64, unsigned long long *sm64b)
{
    __shared__ unsigned long long s_top;
    __shared__ bool s_skip;
    if (threadIdx.x == 0) {
        s_skip = *(volatile uint32_t *)w.err != 0;
        s_top = *w.top;
    }
    __syncthreads();
    if (s_skip) return;
    const unsigned long long base = s_top;
    unsigned long long run_slot = 0;
    for (uint32_t r = 0; r < n; r += blockDim.x) {
        const uint32_t i = r + threadIdx.x;
        unsigned long long slot = 0;
        if (i < n) {
            const unsigned long long E = w.slot[i] >> 2;
            slot = min((E + 1 + 3) & ~3ull, ((unsigned long long)w.pred[i] + 3) & ~3ull);
            w.res[i] = (uint32_t)slot;
        }
        uint32_t xs = 0, tS;
        unsigned long long xo = slot, xc = 0, tSlot, tScr;
        block_excl_scan3(xs, xo, xc, tS, tSlot, tScr, sm32, sm64, sm64b);
        if (i < n) w.slot[i] = base + run_slot + xo;
        run_slot += tSlot;
    }
    if (threadIdx.x == 0) {
        if (base + run_slot > w.cap) atomicOr(w.err, kErrPool);
        else *w.top = base + run_slot;
    }
}

template <bool kBatch>
__global__ void __launch_bounds__(1024) k_plan(const WinSet<kBatch> ws, LevelArgs a)
{
    __shared__ unsigned long long sm64[32], sm64b[32], s_sum[kClasses + 1];
    __shared__ uint32_t sm32[32];
    __shared__ uint32_t s_seg[kClasses];
    __shared__ float s_wseg[kClasses];   // learned balance: work units per segment
    __shared__ unsigned long long s_pred[kClasses];
    __shared__ unsigned long long s_base;
    const WinDev &w = ws.get(blockIdx.x);
    const uint32_t n = a.hi - a.lo;
    if (a.plan_part == 2) {
        plan_slots(w, a, n, sm32, sm64, sm64b);
        return;
    }
    if (*w.err) {   // a failed window: an empty segment table keeps the later kernels off it
        for (uint32_t i = threadIdx.x; i <= n; i += blockDim.x) w.seg_base[i] = 0;
        if (threadIdx.x == 0) *w.n_segs = 0;
        return;
    }
    if (threadIdx.x <= kClasses) s_sum[threadIdx.x] = 0;
    if (threadIdx.x < kClasses) s_pred[threadIdx.x] = 0;
    // Learned balance (learned allocation): a segment's work is its fan-in
    // events plus bal_weight times the gate output's predicted events, and
    // segments are cut to equal work, so gates that change their output
    // often get more, shorter segments and the lanes of a warp finish
    // together.
    const bool bal = a.alloc_mode == kAllocLearned && a.bal_weight > 0.f && a.plan_part == 0;
    // Pass 1: every gate output's fan-in events E and fan-in class, parked
    // in its slot entry as E << 2 | class until pass 2 overwrites it; the
    // level's fan-in events per
    // class (every class runs as its own launch, so every class is split
    // into about seg_target segments) and its gate events.
    const uint32_t step = blockDim.x * kPlanPer;
    unsigned long long e_cls[kClasses] = {0, 0, 0, 0}, p_cls[kClasses] = {0, 0, 0, 0}, g_tot = 0;
    for (uint32_t r = 0; r < n; r += step) {
#pragma unroll
        for (int k = 0; k < kPlanPer; ++k) {
            const uint32_t i = r + k * blockDim.x + threadIdx.x;
            if (i >= n) break;
            const DrvMeta &md = a.meta[a.lo + i];
            const int m = md.m;
            unsigned long long E = 0;
#pragma unroll
            for (int j = 0; j < kMaxSlots; ++j)
                if (j < m) E += w.net_len[md.net[j]];
            const int c = fanin_class(m);
            const unsigned long long pr = bal ? w.pred[i] : 0u;
#pragma unroll
            for (int q = 0; q < kClasses; ++q) if (q == c) { e_cls[q] += E; p_cls[q] += pr; }
            if (md.flags & kFlagFirstOut) {  // first output of its instance: count fan-in per pin
                for (int p = 0; p < md.n_pins; ++p) g_tot += w.net_len[md.net[(md.pin_slot >> (3 * p)) & 7u]];
            }
            w.slot[i] = (E << 2) | (unsigned long long)c;
        }
    }
    __syncthreads();   // s_sum cleared
    {
        const unsigned FULL = 0xffffffffu;
#pragma unroll
        for (int q = 0; q <= kClasses; ++q) {
            unsigned long long v = q < kClasses ? e_cls[q] : g_tot;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
            if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s_sum[q], v);
        }
        if (bal) {
#pragma unroll
            for (int q = 0; q < kClasses; ++q) {
                unsigned long long v = p_cls[q];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
                if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s_pred[q], v);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long e_tot = 0;
        for (int q = 0; q < kClasses; ++q) e_tot += s_sum[q];
        unsigned long long floor_seg = 8;
        if (w.seg_cap <= n) {
            atomicOr(w.err, kErrSegCap);
        } else {
            const unsigned long long room = w.seg_cap - n;
            floor_seg = max(floor_seg, (e_tot + room - 1) / room + 1);
        }
        for (int k = 0; k < kClasses; ++k) {
            unsigned long long seg = a.seg_events;
            const bool warp = (a.warp_mask >> k) & 1u;
            const unsigned long long target = warp ? a.seg_target_w : a.seg_target;
            const unsigned long long ev = a.wave_e ? a.wave_e[k] : s_sum[k];   // the wave shares the GPU
            if (!seg) seg = max(warp ? 128ull : 32ull, (ev + target - 1) / max(1ull, target));
            s_seg[k] = (uint32_t)min(max(seg, floor_seg), 0x7FFFFFFFull);
            // as many segments in the class as without the balance
            s_wseg[k] = (float)s_seg[k] * (1.f + a.bal_weight * (float)s_pred[k] / (float)max(1ull, s_sum[k]));
        }
        s_base = *w.top;
        atomicAdd(&w.counters[0], s_sum[kClasses]);
        atomicAdd(&w.counters[3], e_tot);
    }
    __syncthreads();
    if (*w.err) {
        for (uint32_t i = threadIdx.x; i <= n; i += blockDim.x) w.seg_base[i] = 0;
        if (threadIdx.x == 0) *w.n_segs = 0;
        return;
    }
    // Pass 2: segments, slot and scratch sizes, placed by a block scan in
    // gate-output order (part 1: no slots; the parked E << 2 | class stays
    // in the slot table for part 2)
    const bool slots = a.plan_part != 1;
    const unsigned long long base = s_base;
    uint32_t run_seg = 0;
    unsigned long long run_slot = 0, run_scr = 0;
    for (uint32_t r = 0; r < n; r += blockDim.x) {
        const uint32_t i = r + threadIdx.x;
        uint32_t S = 0;
        unsigned long long slot = 0, scr = 0;
        if (i < n) {
            const unsigned long long ec = w.slot[i];
            const unsigned long long E = ec >> 2;
            const uint32_t seg = s_seg[ec & 3u];
            S = (uint32_t)max(1ull, (E + seg - 1) / seg);
            if (bal && E > 0) {
                const float work = (float)E + a.bal_weight * (float)w.pred[i];
                const float sf = ceilf(work / s_wseg[ec & 3u]);
                // at most one segment per fan-in event, and within the segment floor's count
                S = (uint32_t)min((float)E, max(1.f, min(sf, (float)((E + seg - 1) / seg) * 4.f)));
            }
            slot = (E + 1 + 3) & ~3ull;     // final list: at most one event per step plus (0, X)
            if (a.alloc_mode == kAllocExact || !slots) slot = 0;
            else if (a.alloc_mode == kAllocLearned) slot = min(slot, ((unsigned long long)w.pred[i] + 3) & ~3ull);
            if (a.alloc_mode != kAllocBound && slots) w.res[i] = (uint32_t)slot;
            scr = (E + S + 3) & ~3ull;      // segment stacks: events of the segment (+1 for the first)
        }
        uint32_t xs = S, tS;
        unsigned long long xo = slot, xc = scr, tSlot, tScr;
        block_excl_scan3(xs, xo, xc, tS, tSlot, tScr, sm32, sm64, sm64b);
        if (i < n) {
            w.seg_base[i] = run_seg + xs;
            if (slots) w.slot[i] = base + run_slot + xo;
            w.scr[i] = run_scr + xc;
        }
        run_seg += tS;
        run_slot += tSlot;
        run_scr += tScr;
    }
    __shared__ bool s_fail;
    if (threadIdx.x == 0) {
        w.seg_base[n] = run_seg;
        *w.n_segs = run_seg;
        uint32_t e = 0;
        if (run_seg > w.seg_cap) e |= kErrSegCap;
        if (run_scr > w.scr_cap) e |= kErrScratch;
        if (base + run_slot > w.cap) e |= kErrPool;
        // the pool pointer moves only for a plan that holds: a caller that
        // owns the pool may retry a failed level with fewer outputs
        if (e) atomicOr(w.err, e);
        else *w.top = base + run_slot;
        s_fail = e != 0;
        atomicAdd(&w.counters[2], (unsigned long long)run_seg);
    }
    __syncthreads();
    if (s_fail) {
        for (uint32_t i = threadIdx.x; i <= n; i += blockDim.x) w.seg_base[i] = 0;
        if (threadIdx.x == 0) *w.n_segs = 0;
    }
}

// ------------------------------------------------------------------- sim
// First index of the change list x[0..n) with time >= key, searched from a
// guess: gallop away from the guess, then bisect.  Event lists of one gate
// share the clock, so a position scaled from another list is usually a few
// events off.  Compares whole words: time >= key <=> word >= key << 2.
template <class Wd>
__device__ __forceinline__ uint32_t search_from(const Wd *__restrict__ x, uint32_t n, uint32_t key, uint32_t g)
{
    if (n == 0) return 0;
    const Wd kw = (Wd)key << 2;
    if (g >= n) g = n - 1;
    int64_t lo, hi;
    if (x[g] < kw) {
        int64_t a = g, b;
        uint32_t step = 1;
        for (;;) {
            b = a + step;
            if (b >= (int64_t)n) { b = n; break; }
            if (x[b] >= kw) break;
            a = b;
            step <<= 1;
        }
        lo = a + 1; hi = b;
    } else {
        int64_t b = g, a;
        uint32_t step = 1;
        for (;;) {
            a = b - step;
            if (a < 0) { a = -1; break; }
            if (x[a] < kw) break;
            b = a;
            step <<= 1;
        }
        lo = a + 1; hi = b;
    }
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (x[mid] < kw) lo = mid + 1; else hi = mid;
    }
    return (uint32_t)lo;
}

__device__ __forceinline__ uint32_t sel4(const uint4 &q, uint32_t k)
{
    return k == 0 ? q.x : (k == 1 ? q.y : (k == 2 ? q.z : q.w));
}

#ifndef GLS_READER_W2
#define GLS_READER_W2 2   // events per reader chunk in the 1- and 2-input gate kernels
#endif
#ifndef GLS_SIM_WARP_BATCH
#define GLS_SIM_WARP_BATCH 1   // thread-per-segment kernels: a warp takes 32 segments at a time
#endif
// Threads per block of the thread-per-segment kernels: 128, or 256 in the
// kernel variants with bit kSimV256 (as many threads resident per SM: half
// the blocks, each balancing its segments over twice the warps).  Variants
// with bit kSimVWide read twice the events per load (4 for 1- and 2-input
// gates, 2 for wider ones: fewer loads, more registers).  The autotuner picks
// the variant; 64-bit windows always run variant 0.
constexpr uint32_t kSimBlock = 128;
constexpr int kSimV256 = 1, kSimVWide = 2;
template <int kV> constexpr uint32_t sim_block() { return (kV & kSimV256) ? 256u : kSimBlock; }
#ifndef GLS_READER_W3
#define GLS_READER_W3 1   // events per reader chunk in the wider gate kernels
#endif

// Buffered reader of one change list: the chunk of W events holding the
// head and the next chunk are kept in registers (W = 4: one 16-byte load per
// four events; 2: one 8-byte load per two; 1: one word per event).  Lists
// start on a 4-event boundary and their allocations are padded to whole
// 4-event chunks.  The gate kernels are bound by registers: narrower chunks
// cost more loads but free registers, which removed spills and let more
// warps stay resident (measured on the 200,000-cell workload: 1-word chunks
// for the 3-input and wider gates at 8 blocks per SM, 2-word chunks for the
// 1- and 2-input gates, gate kernels 27.3 → 19.5 ms per step).
template <int W> struct ChunkOf;
template <> struct ChunkOf<4> { using T = uint4; };
template <> struct ChunkOf<2> { using T = uint2; };
template <> struct ChunkOf<1> { using T = uint32_t; };
__device__ __forceinline__ uint32_t sel_chunk(const uint4 &q, uint32_t k) { return sel4(q, k); }
__device__ __forceinline__ uint32_t sel_chunk(const uint2 &q, uint32_t k) { return k == 0 ? q.x : q.y; }
__device__ __forceinline__ uint32_t sel_chunk(uint32_t q, uint32_t) { return q; }

template <int W>
struct Reader {
    using C = typename ChunkOf<W>::T;
    uint64_t cb;        // chunk index of the list start (the list offset / W; pools pass 2^34 events)
    uint32_t p, e;      // head and end index within the list
    C ct, nt;           // chunk holding the head, next chunk

    __device__ __forceinline__ void start(const C *__restrict__ P, uint64_t off, uint32_t p0, uint32_t e0)
    {
        cb = off / W;
        p = p0;
        e = e0;
        if (p < e) {
            const uint64_t c = cb + p / W;
            ct = __ldg(P + c);
            if ((p / W + 1) * W < e) nt = __ldg(P + c + 1);
        }
    }
    // head event word, kInf once exhausted (kInf exceeds every event word)
    __device__ __forceinline__ uint32_t head() const { return p < e ? sel_chunk(ct, p % W) : kInf; }
    __device__ __forceinline__ void advance(const C *__restrict__ P)
    {
        ++p;
        if (p % W == 0 && p < e) {
            ct = nt;
            if ((p / W + 1) * W < e) nt = __ldg(P + cb + p / W + 1);
        }
    }
    // the head after `start`, and after each move
    __device__ __forceinline__ uint32_t first(const C *__restrict__ P, uint64_t off, uint32_t p0, uint32_t e0)
    {
        start(P, off, p0, e0);
        return head();
    }
    __device__ __forceinline__ uint32_t next(const C *__restrict__ P)
    {
        advance(P);
        return head();
    }
};

// One-event chunks: the caller keeps the head, the reader only the
// prefetched event after it, the place of the one after that and the count
// left (four registers per list).
template <>
struct Reader<1> {
    using C = uint32_t;
    const uint32_t *q;  // the event after the prefetched one
    uint32_t left;      // events after the head
    uint32_t nt;        // the event after the head (when left > 0)

    __device__ __forceinline__ uint32_t first(const C *__restrict__ P, uint64_t off, uint32_t p0, uint32_t e0)
    {
        left = 0;
        if (p0 >= e0) return kInf;
        const uint32_t *x = P + off + p0;
        const uint32_t h = __ldg(x);
        left = e0 - p0 - 1;
        if (left) nt = __ldg(x + 1);
        q = x + 2;
        return h;
    }
    __device__ __forceinline__ uint32_t next(const C *__restrict__)
    {
        if (!left) return kInf;
        const uint32_t h = nt;
        if (--left) nt = __ldg(q++);
        return h;
    }
};

// The same one-event reader for 64-bit words (windows with times past
// 2^30 - 2); EvW<WideWord>::kInfW once exhausted.
struct ReaderWide {
    using C = WideWord;
    const WideWord *q;
    uint32_t left;
    WideWord nt;

    __device__ __forceinline__ WideWord first(const C *__restrict__ P, uint64_t off, uint32_t p0, uint32_t e0)
    {
        left = 0;
        if (p0 >= e0) return EvW<WideWord>::kInfW;
        const WideWord *x = P + off + p0;
        const WideWord h = __ldg(x);
        left = e0 - p0 - 1;
        if (left) nt = __ldg(x + 1);
        q = x + 2;
        return h;
    }
    __device__ __forceinline__ WideWord next(const C *__restrict__)
    {
        if (!left) return EvW<WideWord>::kInfW;
        const WideWord h = nt;
        if (--left) nt = __ldg(q++);
        return h;
    }
};

// x * y / z for 32-bit operands, in 32-bit arithmetic when the product fits
__device__ __forceinline__ uint32_t mul_div(uint32_t x, uint32_t y, uint32_t z)
{
    if (__umulhi(x, y) == 0) return (x * y) / z;
    return (uint32_t)((uint64_t)x * y / z);
}

// output value for the input-net values `curp` (2 bits per net) from the
// slot truth table held in registers
template <int M>
__device__ __forceinline__ uint32_t slut_get(const uint4 &t, uint32_t curp)
{
    const uint32_t x = curp & ((1u << (2 * M)) - 1u);
    uint32_t wd = t.x;
    if (M == 3) wd = (x >> 4) == 0 ? t.x : ((x >> 4) == 1 ? t.y : ((x >> 4) == 2 ? t.z : t.w));
    return (wd >> (2 * (x & 15u))) & 3u;
}

// Time of the merged event of rank r (0-based) of two event lists X and Y
// (r < nx + ny), found by a merge-path search galloping from the guess g for
// the number of X events among the first r; on return ix / iy are the
// first events of X / Y at or after that time.  Equal times may sit in both
// lists (not within one), so a cut at the returned time keeps every time's
// events on one side.
template <class Wd>
__device__ __forceinline__ uint32_t rank_time2(const Wd *__restrict__ X, uint32_t nx, const Wd *__restrict__ Y,
                                               uint32_t ny, uint32_t r, uint32_t g, uint32_t &ix, uint32_t &iy)
{
    // short(i): the first r merged events hold more than i events of X
    // (true for small i, false from the answer on)
    auto short_x = [&](uint32_t i) { return i < nx && r - i > 0 && ev_time(Y[r - i - 1]) > ev_time(X[i]); };
    const uint32_t lo0 = r > ny ? r - ny : 0u, hi0 = min(r, nx);
    g = min(max(g, lo0), hi0);
    uint32_t lo, hi;   // the answer lies in [lo, hi]
    if (short_x(g)) {
        uint32_t a = g, step = 1;
        for (;;) {
            const uint32_t b = a + step;
            if (b >= hi0) { lo = a + 1; hi = hi0; break; }
            if (!short_x(b)) { lo = a + 1; hi = b; break; }
            a = b;
            step <<= 1;
        }
    } else {
        uint32_t b = g, step = 1;
        for (;;) {
            if (b - lo0 < step) { lo = lo0; hi = b; break; }
            const uint32_t a = b - step;
            if (short_x(a)) { lo = a + 1; hi = b; break; }
            b = a;
            step <<= 1;
        }
    }
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (short_x(mid)) lo = mid + 1; else hi = mid;
    }
    const uint32_t i = lo, j = r - lo;
    const uint32_t tx = i < nx ? ev_time(X[i]) : kInf, ty = j < ny ? ev_time(Y[j]) : kInf;
    const uint32_t T = min(tx, ty);
    ix = i - ((i > 0 && ev_time(X[i - 1]) == T) ? 1u : 0u);
    iy = j - ((j > 0 && ev_time(Y[j - 1]) == T) ? 1u : 0u);
    return T;
}

// Cut sk of S (0 < sk < S) of a gate output's fan-in timeline: the time of
// the event of rank sk * (plen + slen) / S in the merge of its two longest
// input lists (piv, sec), so that those two (all of them for gates with two
// input nets) split into segments of equal size; with one input net the
// event of rank sk * plen / S of that list.  cut[j] receives list j's first
// event at or after that time.  The cut time does not decrease with sk.
template <int M, class Wd>
__device__ __forceinline__ void cut_at(const Wd *__restrict__ pool, const uint64_t (&off)[M],
                                       const uint32_t (&len)[M], int m, int piv, int sec, uint64_t poff, uint64_t soff,
                                       uint32_t plen, uint32_t slen, uint32_t sk, uint32_t S, uint32_t (&cut)[M])
{
    uint32_t ip, is = 0, T;
    if (sec >= 0) {
        const uint32_t r = mul_div(sk, plen + slen, S);
        T = rank_time2(pool + poff, plen, pool + soff, slen, r, mul_div(r, plen, plen + slen), ip, is);
    } else {
        ip = mul_div(sk, plen, S);
        T = ev_time(pool[poff + ip]);
    }
#pragma unroll
    for (int j = 0; j < M; ++j) {
        if (j < m)
            cut[j] = j == piv ? ip : (j == sec ? is : search_from(pool + off[j], len[j], T, mul_div(ip, len[j], plen)));
    }
}

template <int M, class Wd, bool kWideChunk>
__device__ void sim_segment(const WinDev &w, const LevelArgs &a, const DrvMeta &md, uint32_t s,
                            uint32_t S, uint32_t seg_id, uint64_t scr, const uint4 sl)
{
    constexpr bool kSlut = M <= 3;   // truth table in registers
    constexpr int kRW = (M >= 3 ? GLS_READER_W3 : GLS_READER_W2) * (kWideChunk ? 2 : 1);   // events per reader chunk
    // 64-bit words (a window with times past 2^30 - 2) are read one at a time
    using RD = typename std::conditional<std::is_same<Wd, uint32_t>::value, Reader<kRW>, ReaderWide>::type;
    using RC = typename RD::C;
    const RC *P = reinterpret_cast<const RC *>(w.pool);
    const Wd *pw = reinterpret_cast<const Wd *>(w.pool);
    uint64_t off[M];
    uint32_t len[M];
    int piv = 0, sec = -1;   // the longest input list and the longest of the others
    uint32_t plen = 0, slen = 0;
#pragma unroll
    for (int j = 0; j < M; ++j) {
        len[j] = 0; off[j] = 0;
        if (j < md.m) {
            const uint32_t net = md.net[j];
            off[j] = w.net_off[net];
            len[j] = w.net_len[net];
            if (len[j] > plen) { sec = piv; slen = plen; plen = len[j]; piv = j; }
            else if (sec < 0 || len[j] > slen) { sec = j; slen = len[j]; }
        }
    }
    if (md.m < 2) sec = -1;
    uint64_t poff = 0, soff = 0;
#pragma unroll
    for (int j = 0; j < M; ++j) {
        if (j == piv) poff = off[j];
        if (j == sec) soff = off[j];
    }
    // the segment's first events (cut s) and end events (cut s + 1)
    uint32_t cb[M], ce[M];
    if (s > 0) cut_at<M>(pw, off, len, md.m, piv, sec, poff, soff, plen, slen, s, S, cb);
    if (s + 1 < S) cut_at<M>(pw, off, len, md.m, piv, sec, poff, soff, plen, slen, s + 1, S, ce);
    uint32_t curp = 0x555u;   // every slot X
    uint32_t region = s, capn = 1;
    bool before = false;
    RD rd[M];
    Wd hk[M];         // head word of every list with the value bits set: equal times compare equal
#pragma unroll
    for (int j = 0; j < M; ++j) {
        uint32_t b = 0, e = 0;
        if (j < md.m) {
            b = s > 0 ? cb[j] : 0u;
            e = s + 1 < S ? ce[j] : len[j];
            region += b;
            capn += e - b;
            if (b > 0) {
                curp = (curp & ~(3u << (2 * j))) | (ev_val(pw[off[j] + b - 1]) << (2 * j));
                before = true;
            }
        }
        hk[j] = rd[j].first(P, off[j], b, e);
    }
    const uint8_t *lut = a.lut + md.lut_off;
    const NetDelay *nd = a.ndel + md.dt_off;
    const bool regular = md.flags & kFlagRegular;
    Wd *ot = reinterpret_cast<Wd *>(w.scratch) + scr + region;
    uint32_t cnt = 0;                 // stack size
    Wd top = 0;                       // its top word
    int popped_v = -1;
    if (s == 0) { top = EvW<Wd>::word(0, kVX); ot[0] = top; cnt = 1; }
    uint32_t fprev = before ? (kSlut ? slut_get<M>(sl, curp) : lut[lut_index(curp, md)]) : kVX;
    uint32_t min_o = kInf;
    for (;;) {
        Wd mk = hk[0] | 3u;
#pragma unroll
        for (int j = 1; j < M; ++j) mk = min(mk, (Wd)(hk[j] | 3u));
        if (mk == EvW<Wd>::kInfW) break;
        const uint32_t lastp = curp;
        uint32_t chg = 0;
#pragma unroll
        for (int j = 0; j < M; ++j) {
            if ((hk[j] | 3u) == mk) {
                chg |= 1u << j;
                curp = (curp & ~(3u << (2 * j))) | (ev_val(hk[j]) << (2 * j));
                hk[j] = rd[j].next(P);
            }
        }
        const uint32_t F = kSlut ? slut_get<M>(sl, curp) : lut[lut_index(curp, md)];
        if (F == fprev) continue;
        const uint32_t so1 = (kSense1Tab >> (2 * (fprev * 4 + F))) & 3u;   // F != fprev: sense 1..4, minus one
        fprev = F;
        const uint32_t t = ev_time(mk);
        const uint32_t d = regular ? regular_delay<M>(nd, chg, so1, curp, lastp, a.def_delay)
                                   : select_delay(a.arcs + md.arc_off, md.n_arcs, chg, (int)so1 + 1, curp, lastp,
                                                  a.def_delay);
        const uint64_t o64 = (uint64_t)t + d;   // 64 bits: delays reach 2^32 - 2
        if (o64 > EvW<Wd>::kMax) { atomicOr(w.err, kErrTime); break; }
        const uint32_t o = (uint32_t)o64;
        min_o = min(min_o, o);
        // inertial update, src/simulate.cpp:991-1009
        while (cnt > 0 && ev_time(top) >= o) {
            if (s == 0 && cnt == 1) { popped_v = (int)ev_val(top); cnt = 0; break; }
            --cnt;
            if (cnt > 0) top = ot[cnt - 1];
        }
        const int prevv = cnt > 0 ? (int)ev_val(top) : (s == 0 ? popped_v : -1);
        if (prevv != (int)F) {
            if (cnt >= capn) { atomicOr(w.err, kErrRegion); break; }
            top = EvW<Wd>::word(o, F);
            ot[cnt++] = top;
        } else if (cnt == 0) {
            atomicOr(w.err, kErrEmptied);
            break;
        }
    }
    SegRecT<Wd> r;
    r.region = region; r.cnt = cnt; r.min_o = min_o; r.last = top;
    reinterpret_cast<SegRecT<Wd> *>(w.segs)[seg_id] = r;
}

// Segments of all windows of a launch form one index space: s_pre[k] is
// the first index of window k.
// skip_err leaves out windows whose error flag is set; only kernels during
// which no flag can change may use it (all blocks must see the same counts).
template <bool kSkipErr, bool kBatch, class Count>
__device__ uint32_t window_prefix(const WinSet<kBatch> &ws, Count count, uint32_t *s_pre, uint32_t *sm32)
{
    const uint32_t nwin = ws.size();
    if (!kBatch) {   // one window: no scan
        const WinDev &w = ws.get(0);
        const uint32_t v = (kSkipErr && *w.err) ? 0u : count(w);
        if (threadIdx.x == 0) { s_pre[0] = 0; s_pre[1] = v; }
        __syncthreads();
        return v;
    }
    uint32_t run = 0;
    for (uint32_t c = 0; c < nwin; c += blockDim.x) {
        const uint32_t k = c + threadIdx.x;
        uint32_t v = 0;
        if (k < nwin && !(kSkipErr && *ws.get(k).err)) v = count(ws.get(k));
        uint32_t tot;
        const uint32_t x = block_excl_scan<uint32_t>(v, &tot, sm32);
        if (k < nwin) s_pre[k] = run + x;
        run += tot;
    }
    if (threadIdx.x == 0) s_pre[nwin] = run;
    __syncthreads();
    return run;
}

// the window holding index q: the last k with s_pre[k] <= q
__device__ __forceinline__ uint32_t window_of(const uint32_t *s_pre, uint32_t nwin, uint32_t q)
{
    if (nwin == 1) return 0;
    uint32_t lo = 0, hi = nwin;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_pre[mid] <= q) lo = mid; else hi = mid;
    }
    return lo;
}

// Gates of a level are sorted by fan-in class; one instantiation per class
// keeps the register budget of the common narrow gates small.  Each block
// owns a contiguous share of the class's segments and its threads take the
// next one from a shared counter as they finish, so long and short segments
// balance inside the block.
template <int M, bool kBatch, class Wd, int kV>
#ifndef GLS_SIM2_BLOCKS
#define GLS_SIM2_BLOCKS 8   // resident blocks per SM the 1- and 2-input gate kernels are compiled for
#endif
#ifndef GLS_SIM3_BLOCKS
#define GLS_SIM3_BLOCKS 8   // resident blocks per SM the 3-input gate kernel is compiled for
#endif
#ifndef GLS_SIM1_BLOCKS
#define GLS_SIM1_BLOCKS GLS_SIM2_BLOCKS   // resident blocks per SM the 1-input gate kernel is compiled for
#endif
__global__ void __launch_bounds__(sim_block<kV>(), (M == 1 ? GLS_SIM1_BLOCKS : (M == 2 ? GLS_SIM2_BLOCKS : (M == 3 ? GLS_SIM3_BLOCKS : 4))) /
                                                    ((kV & kSimV256) ? 2 : 1))
    k_sim(const WinSet<kBatch> ws, LevelArgs a, uint32_t d0, uint32_t d1)
{
    __shared__ uint32_t s_next;
    __shared__ uint32_t s_pre[kBatch ? kMaxWave + 1 : 2];
    __shared__ uint32_t sm32[32];
    const uint32_t nwin = ws.size();
    // segment indices: the window's own for one window, else one space over
    // all windows (a window whose plan failed has an all-zero segment table)
    uint32_t g0 = 0, total;
    if (kBatch) {
        total = window_prefix<false>(
            ws, [&](const WinDev &x) { return x.seg_base[d1] - x.seg_base[d0]; }, s_pre, sm32);
    } else {
        g0 = ws.get(0).seg_base[d0];
        total = ws.get(0).seg_base[d1] - g0;
    }
    const uint32_t per = (total + gridDim.x - 1) / gridDim.x;
    const uint32_t b0 = g0 + min(total, blockIdx.x * per), b1 = g0 + min(total, (blockIdx.x + 1) * per);
    __shared__ uint32_t s_hint;   // a driver near the block's latest segment
    if (threadIdx.x == 0) { s_next = b0; s_hint = d0; }
    __syncthreads();
#if GLS_SIM_WARP_BATCH
    // A warp takes 32 consecutive segments at a time, one per lane, so that
    // its lanes start (cut searches), walk and finish their segments
    // together: the segments of one gate output hold equal shares of its
    // two longest input lists.  Lanes that took segments one by one drift
    // apart, and then a segment's setup runs on one lane while the others
    // walk events, each path issued for the few lanes on it.
    const uint32_t lane_id = threadIdx.x & 31u;
    for (;;) {
        uint32_t qb = 0;
        if (lane_id == 0) qb = atomicAdd(&s_next, 32u);
        qb = __shfl_sync(0xffffffffu, qb, 0);
        if (qb >= b1) break;
        const uint32_t q = qb + lane_id;
        if (q >= b1) continue;
#else
    for (;;) {
        const uint32_t q = atomicAdd(&s_next, 1u);
        if (q >= b1) break;
#endif
        const uint32_t win = kBatch ? window_of(s_pre, nwin, q) : 0u;
        const WinDev &w = ws.get(win);
        const uint32_t g = kBatch ? q - s_pre[win] + w.seg_base[d0] : q;
        // driver owning segment g: last i in [d0, d1) with seg_base[i] <= g.
        // Segments go out in increasing order, so with one window the block's
        // latest driver is a close guess: gallop from it, then bisect.
        uint32_t lo = d0, hi = d1;
        if (!kBatch) {
            const uint32_t h = min(max(*(volatile uint32_t *)&s_hint, d0), d1 - 1);
            if (w.seg_base[h] <= g) {
                lo = h;
                uint32_t step = 1;
                while (lo + step < d1 && w.seg_base[lo + step] <= g) { lo += step; step <<= 1; }
                hi = min(d1, lo + step);
            } else {
                hi = h;
                uint32_t step = 1;
                while (hi - d0 > step && w.seg_base[hi - step] > g) { hi -= step; step <<= 1; }
                lo = hi - d0 > step ? hi - step : d0;
            }
        }
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (w.seg_base[mid] <= g) lo = mid; else hi = mid;
        }
        const uint32_t i = lo;
        if (!kBatch) s_hint = i;
        const uint32_t sb = w.seg_base[i];
        const uint32_t S = w.seg_base[i + 1] - sb;
        const DrvMeta md = a.meta[a.lo + i];
        const uint4 sl = M <= 3 ? __ldg(a.slut + a.lo + i) : make_uint4(0, 0, 0, 0);
        sim_segment<M, Wd, (kV & kSimVWide) != 0>(w, a, md, g - sb, S, g, w.scr[i], sl);
    }
}

// ------------------------------------------------------------- warp sim
// Warp-per-segment kernels for gates with 1, 2 or 3 distinct input nets.
// A tile is the next kTile fan-in events of the segment in time order,
// kItems consecutive events per lane; inside a lane the events are walked
// in order with plain registers, and lanes meet only in a few warp scans
// per tile (input values before the lane, the candidate suffix minimum,
// the previous surviving candidate, the push offsets).
constexpr int kItems = 4;                 // events per lane per tile (more than 3: a step spans at most 2 lanes)
constexpr int kTile = 32 * kItems;        // events per tile; ring size of every input list

template <int M>
struct WarpSmem {
    uint32_t ring[M][kTile];              // the next kTile events of every input list (kInf past its end)
    uint32_t ab[M == 3 ? kTile : 1];      // 3-input gates: lists 0 and 1 merged
    uint8_t abj[M == 3 ? kTile : 1];      // and the list each came from
    uint32_t nd[8 * M];                   // NetDelay of the gate output's input nets
    uint8_t lut[1 << (2 * M)];            // output value for the input nets' values (2 bits per net)
};

__device__ __forceinline__ uint32_t tkey(uint32_t word) { return word | 3u; }   // orders by time, kInf stays kInf

// Merge path: positions [d, d + kItems) of the stable merge of two sorted
// arrays of L entries each (A first on equal times).  Bit k of src tells
// whether output k came from B, pos[k] its index in the array it came from.
template <class FA, class FB>
__device__ __forceinline__ void merge_items(FA A, FB B, uint32_t L, uint32_t d, uint32_t out[kItems], uint32_t &src,
                                            uint32_t pos[kItems])
{
    uint32_t lo = d > L ? d - L : 0u, hi = min(d, L);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (tkey(A(mid)) <= tkey(B(d - 1 - mid))) lo = mid + 1; else hi = mid;
    }
    uint32_t i = lo, j = d - lo;
    uint32_t a = i < L ? A(i) : kInf, b = j < L ? B(j) : kInf;
    src = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const bool takeb = j < L && (i >= L || tkey(b) < tkey(a));
        out[k] = takeb ? b : a;
        pos[k] = takeb ? j : i;
        if (takeb) {
            src |= 1u << k;
            ++j;
            b = j < L ? B(j) : kInf;
        } else {
            ++i;
            a = i < L ? A(i) : kInf;
        }
    }
}

// regular_delay with the gate's NetDelay entries in shared memory
template <int M>
__device__ __forceinline__ uint32_t regular_delay_s(const uint32_t *nd, uint32_t chg, int so, uint32_t curp,
                                                    uint32_t lastp, uint32_t defd)
{
    uint32_t d = kInf;
#pragma unroll
    for (int j = 0; j < M; ++j) {
        if ((chg >> j) & 1u) {
            const uint32_t neg = (kNegTab >> (slot_val(lastp, j) * 4 + slot_val(curp, j))) & 1u;
            d = min(d, nd[j * 8 + neg * 4 + so - 1]);
        }
    }
    return d == kInf ? defd : d;
}

// One time segment of one gate output, run by a whole warp: the same
// segment contract as sim_segment (stack region, local stack, min_o).
//
// A tile merges the next kTile events of the input lists and keeps those
// strictly before the time of the last merged one, so that every step (the
// events of one time, which the reference evaluates once) is whole.  Lane l
// holds merged events [4l, 4l + 4).  The lanes rebuild the input values
// after every event, evaluate the cell at the last event of every step,
// pick the delay, and run the inertial stack in closed form: a candidate
// survives the tile iff its output time is below every later candidate's,
// the old stack loses its entries at or after the tile's smallest candidate
// time, and a survivor is pushed iff its value differs from the previous
// survivor's (or, for the first, from the stack top).
template <int M>
__device__ void sim_segment_warp(const WinDev &w, const LevelArgs &a, const DrvMeta &md, uint32_t drv, uint32_t s,
                                 uint32_t S, uint32_t seg_id, uint64_t scr, WarpSmem<M> &sm)
{
    const unsigned FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned lower = (1u << lane) - 1u;
    const uint32_t *__restrict__ pool = w.pool;
    // list geometry: lane j < m holds list j, then every lane gets a copy
    uint64_t myoff = 0;
    uint32_t mylen = 0;
    if (lane < md.m) {
        const uint32_t net = __ldg(&a.meta[drv].net[lane]);
        myoff = w.net_off[net];
        mylen = w.net_len[net];
    }
    uint64_t off[M];
    uint32_t len[M];
    int piv = 0;
    uint32_t plen = 0;
#pragma unroll
    for (int j = 0; j < M; ++j) {
        off[j] = __shfl_sync(FULL, myoff, j);
        len[j] = __shfl_sync(FULL, mylen, j);
        if (len[j] > plen) { plen = len[j]; piv = j; }
    }
    uint64_t poff = 0;
#pragma unroll
    for (int j = 0; j < M; ++j) if (j == piv) poff = off[j];
    const uint32_t plo = (uint32_t)((uint64_t)s * plen / S), phi = (uint32_t)((uint64_t)(s + 1) * plen / S);
    const uint32_t tlo = s > 0 ? ev_time(__ldg(pool + poff + plo)) : 0u;
    const uint32_t thi = s + 1 < S ? ev_time(__ldg(pool + poff + phi)) : kInf;
    uint32_t b = 0, e = 0, vb = kVX;
    if (lane < md.m) {
        const uint32_t gl = plen ? (uint32_t)((uint64_t)plo * mylen / plen) : 0u;
        const uint32_t gh = plen ? (uint32_t)((uint64_t)phi * mylen / plen) : 0u;
        b = s > 0 ? ((int)lane == piv ? plo : search_from(pool + myoff, mylen, tlo, gl)) : 0u;
        e = s + 1 < S ? ((int)lane == piv ? phi : search_from(pool + myoff, mylen, thi, gh)) : mylen;
        if (b > 0) vb = ev_val(__ldg(pool + myoff + b - 1));
    }
    uint32_t p[M], E[M];
    uint32_t region = s, capn = 1, curp_c = 0;
    bool before = false;
#pragma unroll
    for (int j = 0; j < M; ++j) {
        p[j] = __shfl_sync(FULL, b, j);
        E[j] = __shfl_sync(FULL, e, j);
        curp_c |= __shfl_sync(FULL, vb, j) << (2 * j);
        region += p[j];
        capn += E[j] - p[j];
        before |= p[j] > 0;
    }
    uint32_t *ot = w.scratch + scr + region;
    uint32_t cnt = 0, top = 0, popped_v = kVX;   // stack size, its top word, value of a popped bottom
    __syncwarp();   // the warp's previous segment is done with the shared tables
    for (uint32_t k = lane; k < (1u << (2 * M)); k += 32) sm.lut[k] = __ldg(a.lut + md.lut_off + lut_index(k, md));
    const bool regular = md.flags & kFlagRegular;
    if (regular && lane < 8u * md.m) sm.nd[lane] = __ldg(&a.ndel[md.dt_off + lane / 8].d[lane % 8]);
#pragma unroll
    for (int j = 0; j < M; ++j) {
#pragma unroll
        for (int r = 0; r < kItems; ++r) {
            const uint32_t x = p[j] + r * 32 + lane;
            sm.ring[j][x & (kTile - 1)] = x < E[j] ? __ldg(pool + off[j] + x) : kInf;
        }
    }
    if (s == 0) {
        top = ev_word(0, kVX);
        if (lane == 0) ot[0] = top;
        cnt = 1;
    }
    __syncwarp();
    uint32_t fprev = before ? sm.lut[curp_c] : kVX;
    uint32_t min_o = kInf;
    const uint32_t d0 = lane * kItems;
    for (;;) {
        // ---- merge: lane holds merged events d0 .. d0+3 and their lists (2 bits each)
        uint32_t wd[kItems], jsrc = 0;
        if (M == 1) {
#pragma unroll
            for (int k = 0; k < kItems; ++k) wd[k] = sm.ring[0][(p[0] + d0 + k) & (kTile - 1)];
        } else {
            const uint32_t *r0 = sm.ring[0], *r1 = sm.ring[1];
            const uint32_t q0 = p[0], q1 = p[1];
            auto A0 = [&](uint32_t i) { return r0[(q0 + i) & (kTile - 1)]; };
            auto A1 = [&](uint32_t i) { return r1[(q1 + i) & (kTile - 1)]; };
            uint32_t srcb, pos[kItems];
            if (M == 2) {
                merge_items(A0, A1, kTile, d0, wd, srcb, pos);
#pragma unroll
                for (int k = 0; k < kItems; ++k) jsrc |= ((srcb >> k) & 1u) << (2 * k);
            } else {
                uint32_t t01[kItems];
                merge_items(A0, A1, kTile, d0, t01, srcb, pos);
#pragma unroll
                for (int k = 0; k < kItems; ++k) {
                    sm.ab[d0 + k] = t01[k];
                    sm.abj[d0 + k] = (uint8_t)((srcb >> k) & 1u);
                }
                __syncwarp();
                const uint32_t *r2 = sm.ring[M - 1];
                const uint32_t q2 = p[M - 1];
                auto AB = [&](uint32_t i) { return sm.ab[i]; };
                auto A2 = [&](uint32_t i) { return r2[(q2 + i) & (kTile - 1)]; };
                merge_items(AB, A2, kTile, d0, wd, srcb, pos);
#pragma unroll
                for (int k = 0; k < kItems; ++k)
                    jsrc |= (((srcb >> k) & 1u) ? 2u : (uint32_t)sm.abj[pos[k]]) << (2 * k);
            }
        }
        // ---- this tile: the events before the time of the last merged one
        const uint32_t tc = M == 1 ? kInf : __shfl_sync(FULL, tkey(wd[kItems - 1]), 31);
        uint32_t vm = 0, cl[M];
#pragma unroll
        for (int j = 0; j < M; ++j) cl[j] = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            if (tkey(wd[k]) < tc) {
                vm |= 1u << k;
#pragma unroll
                for (int j = 0; j < M; ++j) cl[j] += ((jsrc >> (2 * k)) & 3u) == (uint32_t)j ? 1u : 0u;
            }
        }
        uint32_t c[M], n = 0;
#pragma unroll
        for (int j = 0; j < M; ++j) {
            c[j] = __reduce_add_sync(FULL, cl[j]);
            n += c[j];
        }
        if (n == 0) break;
        // next events of the lists, stored into the ring after this tile
        uint32_t nv[M][kItems];
#pragma unroll
        for (int j = 0; j < M; ++j) {
#pragma unroll
            for (int r = 0; r < kItems; ++r) {
                const uint32_t x = r * 32 + lane, src = p[j] + kTile + x;
                nv[j][r] = (x < c[j] && src < E[j]) ? __ldg(pool + off[j] + src) : kInf;
            }
        }
        // ---- input values before the lane's first event: the last event of
        // every list in the lanes before, else the values before the tile
        uint32_t lv = 0, has = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            if ((vm >> k) & 1u) {
                const uint32_t J = (jsrc >> (2 * k)) & 3u;
                lv = (lv & ~(3u << (2 * J))) | (ev_val(wd[k]) << (2 * J));
                has |= 1u << J;
            }
        }
        uint32_t curp0 = 0;
#pragma unroll
        for (int j = 0; j < M; ++j) {
            const unsigned pre = __ballot_sync(FULL, (has >> j) & 1u) & lower;
            const uint32_t v = __shfl_sync(FULL, lv, pre ? 31 - __clz(pre) : lane);
            curp0 |= (pre ? slot_val(v, j) : slot_val(curp_c, j)) << (2 * j);
        }
        // ---- steps: values after every event; the last event of a step
        // evaluates the cell with the values before the step and the nets
        // that changed in it (a step may start in the lane before)
        uint32_t tt[kItems];
#pragma unroll
        for (int k = 0; k < kItems; ++k) tt[k] = ((vm >> k) & 1u) ? ev_time(wd[k]) : kInf;
        uint32_t t_next = __shfl_down_sync(FULL, tt[0], 1);
        if (lane == 31u) t_next = kInf;
        uint32_t t_prev = __shfl_up_sync(FULL, tt[kItems - 1], 1);
        if (lane == 0) t_prev = kInf;
        uint32_t st = curp0, gs = curp0, gc = 0, em = 0, chp = 0, fv = 0;
        uint32_t cp[kItems], lp[kItems];
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            cp[k] = 0;
            lp[k] = 0;
            if ((vm >> k) & 1u) {
                const bool newg = tt[k] != (k == 0 ? t_prev : tt[k > 0 ? k - 1 : 0]);
                if (newg) { gs = st; gc = 0; }
                const uint32_t J = (jsrc >> (2 * k)) & 3u;
                st = (st & ~(3u << (2 * J))) | (ev_val(wd[k]) << (2 * J));
                gc |= 1u << J;
                cp[k] = st;
                lp[k] = gs;
                chp |= gc << (4 * k);
                if ((k + 1 < kItems ? tt[k + 1 < kItems ? k + 1 : 0] : t_next) != tt[k]) {
                    em |= 1u << k;
                    fv |= (uint32_t)sm.lut[st] << (2 * k);
                }
            }
        }
        {   // a step continued from the lane before: its start values and changed nets come from there
            const uint32_t in_gs = __shfl_up_sync(FULL, gs, 1);
            const uint32_t in_gc = __shfl_up_sync(FULL, gc, 1);
            if ((vm & 1u) && tt[0] == t_prev && em) {
                const int k1 = __ffs(em) - 1;
#pragma unroll
                for (int k = 0; k < kItems; ++k) {
                    if (k == k1) {
                        lp[k] = in_gs;
                        chp |= in_gc << (4 * k);
                    }
                }
            }
        }
        const uint32_t lastF = em ? (fv >> (2 * (31 - __clz(em)))) & 3u : 0u;
        uint32_t fp = __shfl_up_sync(FULL, lastF, 1);
        if (lane == 0) fp = fprev;
        // ---- candidates: steps whose output value changes
        uint32_t o[kItems], am = 0, sov = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            o[k] = kInf;
            if ((em >> k) & 1u) {
                const uint32_t F = (fv >> (2 * k)) & 3u;
                if (F != fp) {
                    sov |= (uint32_t)((kSenseTab >> (3 * (fp * 4 + F))) & 7u) << (4 * k);
                    am |= 1u << k;
                }
                fp = F;
            }
        }
        bool bad = false;
        if (regular) {
#pragma unroll
            for (int k = 0; k < kItems; ++k) {
                if ((am >> k) & 1u) {
                    const uint32_t d = regular_delay_s<M>(sm.nd, (chp >> (4 * k)) & 15u, (int)((sov >> (4 * k)) & 15u),
                                                          cp[k], lp[k], a.def_delay);
                    o[k] = tt[k] + d;
                    bad |= o[k] > kMaxTime || o[k] < tt[k];
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < kItems; ++k) {
                if ((am >> k) & 1u) {
                    const uint32_t d = select_delay(a.arcs + md.arc_off, md.n_arcs, (chp >> (4 * k)) & 15u,
                                                    (int)((sov >> (4 * k)) & 15u), cp[k], lp[k], a.def_delay);
                    o[k] = tt[k] + d;
                    bad |= o[k] > kMaxTime || o[k] < tt[k];
                }
            }
        }
        if (__ballot_sync(FULL, bad)) {
            if (lane == 0) atomicOr(w.err, kErrTime);
            break;
        }
        // ---- inertial stack, src/simulate.cpp:991-1009 in closed form
        uint32_t later[kItems], sfx = kInf;
#pragma unroll
        for (int k = kItems - 1; k >= 0; --k) {
            later[k] = sfx;
            sfx = min(sfx, o[k]);
        }
        uint32_t x = sfx;   // suffix minimum over the lanes
#pragma unroll
        for (int q = 1; q < 32; q <<= 1) {
            const uint32_t y = __shfl_down_sync(FULL, x, q);
            if (lane + q < 32u) x = min(x, y);
        }
        uint32_t lx = __shfl_down_sync(FULL, x, 1);
        if (lane == 31u) lx = kInf;
        const uint32_t tmin = __shfl_sync(FULL, x, 0);
        if (tmin != kInf) {
            min_o = min(min_o, tmin);
            if (cnt > 0 && ev_time(top) >= tmin) {
                for (;;) {   // drop the stack entries at or after tmin
                    const uint32_t base = cnt > 32u ? cnt - 32u : 0u;
                    const uint32_t idx = base + lane;
                    const uint32_t ent = idx < cnt ? ot[idx] : 0u;
                    const uint32_t nk = __popc(__ballot_sync(FULL, idx < cnt && ev_time(ent) < tmin));
                    if (nk > 0) {
                        cnt = base + nk;
                        top = __shfl_sync(FULL, ent, nk - 1);
                        break;
                    }
                    if (base == 0) {
                        popped_v = ev_val(__shfl_sync(FULL, ent, 0));
                        cnt = 0;
                        break;
                    }
                    cnt = base;
                }
            }
            uint32_t sv = 0;   // survivors
#pragma unroll
            for (int k = 0; k < kItems; ++k)
                if (((am >> k) & 1u) && o[k] < min(later[k], lx)) sv |= 1u << k;
            const uint32_t lastSF = sv ? (fv >> (2 * (31 - __clz(sv)))) & 3u : 0u;
            const unsigned pre = __ballot_sync(FULL, sv != 0) & lower;
            const uint32_t pv = __shfl_sync(FULL, lastSF, pre ? 31 - __clz(pre) : lane);
            int prevv = pre ? (int)pv : (cnt > 0 ? (int)ev_val(top) : (s == 0 ? (int)popped_v : -1));
            bool first = pre == 0, emptied = false;
            uint32_t pm = 0;
#pragma unroll
            for (int k = 0; k < kItems; ++k) {
                if ((sv >> k) & 1u) {
                    const int F = (int)((fv >> (2 * k)) & 3u);
                    if (F != prevv) pm |= 1u << k;
                    else if (first && cnt == 0) emptied = true;
                    first = false;
                    prevv = F;
                }
            }
            if (__ballot_sync(FULL, emptied)) {
                if (lane == 0) atomicOr(w.err, kErrEmptied);
                break;
            }
            const uint32_t np = __popc(pm);
            uint32_t inc = np;
#pragma unroll
            for (int q = 1; q < 32; q <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, inc, q);
                if (lane >= (uint32_t)q) inc += y;
            }
            const uint32_t total = __shfl_sync(FULL, inc, 31);
            if (cnt + total > capn) {
                if (lane == 0) atomicOr(w.err, kErrRegion);
                break;
            }
            uint32_t wpos = cnt + inc - np, lastw = 0;
#pragma unroll
            for (int k = 0; k < kItems; ++k) {
                if ((pm >> k) & 1u) {
                    lastw = ev_word(o[k], (fv >> (2 * k)) & 3u);
                    ot[wpos++] = lastw;
                }
            }
            if (total) {
                top = __shfl_sync(FULL, lastw, 31 - __clz(__ballot_sync(FULL, np > 0)));
                cnt += total;
            }
        }
        // ---- carry to the next tile, then refill the rings
        const uint32_t ll = (n - 1) / kItems;
        curp_c = __shfl_sync(FULL, st, ll);
        fprev = __shfl_sync(FULL, lastF, ll);
        __syncwarp();
#pragma unroll
        for (int j = 0; j < M; ++j) {
#pragma unroll
            for (int r = 0; r < kItems; ++r) {
                const uint32_t xr = r * 32 + lane;
                if (xr < c[j]) sm.ring[j][(p[j] + xr) & (kTile - 1)] = nv[j][r];
            }
            p[j] += c[j];
        }
        __syncwarp();
    }
    if (lane == 0) {
        SegRec r;
        r.region = region; r.cnt = cnt; r.min_o = min_o; r.last = top;
        w.segs[seg_id] = r;
    }
}

// Warp-per-segment launch for the 1-, 2- and 3-input classes: each block
// owns a contiguous share of the class's segments and its warps take the
// next one from a shared counter as they finish.
template <int M, bool kBatch>
__global__ void __launch_bounds__(128, M == 1 ? 8 : (M == 2 ? 7 : 6))
    k_sim_warp(const WinSet<kBatch> ws, LevelArgs a, uint32_t d0, uint32_t d1)
{
    constexpr int kWarps = 4;
    __shared__ uint32_t s_next;
    __shared__ WarpSmem<M> sm[kWarps];
    __shared__ uint32_t s_pre[kBatch ? kMaxWave + 1 : 2];
    __shared__ uint32_t sm32[32];
    const uint32_t nwin = ws.size();
    uint32_t g0 = 0, total;
    if (kBatch) {
        total = window_prefix<false>(
            ws, [&](const WinDev &x) { return x.seg_base[d1] - x.seg_base[d0]; }, s_pre, sm32);
    } else {
        g0 = ws.get(0).seg_base[d0];
        total = ws.get(0).seg_base[d1] - g0;
    }
    const uint32_t per = (total + gridDim.x - 1) / gridDim.x;
    const uint32_t b0 = g0 + min(total, blockIdx.x * per), b1 = g0 + min(total, (blockIdx.x + 1) * per);
    if (threadIdx.x == 0) s_next = b0;
    __syncthreads();
    const uint32_t wid = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t q = 0;
        if (lane == 0) q = atomicAdd(&s_next, 1u);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= b1) break;
        const uint32_t win = kBatch ? window_of(s_pre, nwin, q) : 0u;
        const WinDev &w = ws.get(win);
        const uint32_t g = kBatch ? q - s_pre[win] + w.seg_base[d0] : q;
        uint32_t lo = d0, hi = d1;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (w.seg_base[mid] <= g) lo = mid; else hi = mid;
        }
        const uint32_t i = lo;
        const uint32_t sb = w.seg_base[i];
        const uint32_t S = w.seg_base[i + 1] - sb;
        const DrvMeta md = a.meta[a.lo + i];
        sim_segment_warp<M>(w, a, md, a.lo + i, g - sb, S, g, w.scr[i], sm[wid]);
    }
}

// --------------------------------------------------------------- combine
__device__ __forceinline__ unsigned long long clampt(uint32_t t, unsigned long long lo, unsigned long long hi)
{
    unsigned long long x = t;
    return x < lo ? lo : (x > hi ? hi : x);
}
__device__ __forceinline__ int vclass(uint32_t v) { return v == kV0 ? 0 : (v == kV1 ? 1 : 2); }

__device__ __forceinline__ void saif_add(unsigned long long acc[3], int cls, unsigned long long d)
{
    if (cls == 0) acc[0] += d; else if (cls == 1) acc[1] += d; else acc[2] += d;
}

// k_link: one warp per gate output, a lane per segment.  Pass A cuts each
// segment's stack at the smallest candidate time of the later segments;
// pass B drops a segment's first entry when it repeats the last kept value
// before it, places the segments back to back in the gate's pool slot and
// hands each segment's copy to k_copy with the final event that precedes it.
template <bool kBatch, class Wd>
#ifndef GLS_LINK_BLOCKS
#define GLS_LINK_BLOCKS 1   // resident blocks per SM the link kernel is compiled for (1: no bound)
#endif
__global__ void __launch_bounds__(256, GLS_LINK_BLOCKS) k_link(const WinSet<kBatch> ws, LevelArgs a, uint32_t d0, uint32_t d1)
{
    // gate outputs [d0, d1) of the level (one fan-in class, or all)
    const uint32_t n = d1 - d0;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= (uint64_t)n * ws.size()) return;
    const uint32_t i = d0 + (uint32_t)(gw % n);
    const WinDev &w = ws.get((uint32_t)(gw / n));
    if (*w.err) return;
    const unsigned FULL = 0xffffffffu;
    const uint32_t sb = w.seg_base[i], se = w.seg_base[i + 1];
    const uint64_t slot = w.slot[i];
    const uint64_t scr = w.scr[i];
    const Wd *sx = reinterpret_cast<const Wd *>(w.scratch) + scr;
    const SegRecT<Wd> *segs = reinterpret_cast<const SegRecT<Wd> *>(w.segs);
    const uint32_t out_net = a.meta[a.lo + i].out_net;
    // pass A (right to left)
    uint32_t carry_min = kInf;
    for (int64_t base = se; base > (int64_t)sb; base -= 32) {
        const int64_t s = base - 32 + lane;
        const bool valid = s >= (int64_t)sb;
        SegRecT<Wd> r = {0, 0, kInf, 0};
        if (valid) r = segs[s];
        uint32_t x = r.min_o;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_down_sync(FULL, x, o);
            if (lane + o < 32) x = min(x, y);
        }
        uint32_t ex = __shfl_down_sync(FULL, x, 1);
        if (lane == 31) ex = kInf;
        const uint32_t M = min(ex, carry_min);
        if (valid) {
            uint32_t keep = r.cnt;   // stack times increase: cut from the top
            if (keep > 0 && ev_time(r.last) >= M) {
                --keep;
                while (keep > 0 && ev_time(sx[r.region + keep - 1]) >= M) --keep;
            }
            w.copies[s].n = keep;    // until pass B
        }
        carry_min = min(carry_min, __shfl_sync(FULL, x, 0));
    }
    __syncwarp();
    // pass B (left to right)
    uint32_t carry_pos = 0, carry_v = kVX;
    unsigned long long cprev = w.t_begin;    // clamped time of the previous final event
    int pclass = 2;                          // its value class
    for (uint32_t base = sb; base < se; base += 32) {
        const uint32_t s = base + lane;
        const bool valid = s < se;
        uint32_t keep = 0, region = 0, firstv = 0, lastv = 0, lastt = 0;
        if (valid) {
            const SegRecT<Wd> r = segs[s];
            keep = w.copies[s].n;
            region = r.region;
            if (keep) {
                firstv = ev_val(sx[region]);
                const Wd lw = keep == r.cnt ? r.last : sx[region + keep - 1];
                lastv = ev_val(lw);
                lastt = ev_time(lw);
            }
        }
        const unsigned bal = __ballot_sync(FULL, keep > 0);
        const unsigned prior = bal & ((1u << lane) - 1u);
        const uint32_t vsh = __shfl_sync(FULL, lastv, prior ? 31 - __clz(prior) : 0);
        const uint32_t vprev = prior ? vsh : carry_v;
        const uint32_t drop = (s > sb && keep > 0 && firstv == vprev) ? 1u : 0u;
        const uint32_t fin = keep - drop;
        uint32_t inc = fin;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += y;
        }
        const uint32_t pos = carry_pos + inc - fin;
        const unsigned fb = __ballot_sync(FULL, fin > 0);
        const unsigned fprior = fb & ((1u << lane) - 1u);
        const int fsrc = fprior ? 31 - __clz(fprior) : 0;
        const unsigned long long clast = clampt(lastt, w.t_begin, w.t_end);
        const unsigned long long csh = __shfl_sync(FULL, clast, fsrc);
        const int ksh = __shfl_sync(FULL, vclass(lastv), fsrc);
        if (valid) {
            CopyRec c;
            c.src = scr + region + drop;
            c.dst = a.alloc_mode == kAllocBound ? slot + pos : pos;
            c.n = fin;
            c.drv = i;
            c.cprev = fprior ? csh : cprev;
            c.pclass = (uint32_t)(fprior ? ksh : pclass);
            c.out_net = out_net;
            w.copies[s] = c;
        }
        if (bal) carry_v = __shfl_sync(FULL, lastv, 31 - __clz(bal));
        if (fb) {
            const int top = 31 - __clz(fb);
            cprev = __shfl_sync(FULL, clast, top);
            pclass = __shfl_sync(FULL, vclass(lastv), top);
        }
        carry_pos += __shfl_sync(FULL, inc, 31);
    }
    if (lane == 0) {
        if (a.alloc_mode != kAllocBound) {
            // exact placement now that the length is known (every gate in
            // exact mode, gates that outgrew their predicted slot in learned mode)
            uint64_t st = slot;
            if (a.alloc_mode == kAllocExact || carry_pos > w.res[i]) {
                const unsigned long long need = (carry_pos + 3ull) & ~3ull;
                st = atomicAdd(w.top, need);
                if (st + need > w.cap) atomicOr(w.err, kErrPool);
                if (a.alloc_mode == kAllocLearned) atomicAdd(w.n_over, 1ull);
                w.slot[i] = st;
            }
            w.net_off[out_net] = st;
        } else {
            w.net_off[out_net] = slot;   // written here, not by the plan: a failed level leaves the table as it was
        }
        // the last event holds until t_end; k_copy adds the rest
        unsigned long long acc[3] = {0, 0, 0};
        saif_add(acc, pclass, w.t_end - cprev);
        w.net_len[out_net] = carry_pos;
        w.saif[3ull * out_net + 0] = acc[0];
        w.saif[3ull * out_net + 1] = acc[1];
        w.saif[3ull * out_net + 2] = acc[2];
        atomicAdd(&w.counters[1], (unsigned long long)carry_pos);
    }
}

// Window-relative clamped times in 32 bits.  Event times are at most
// kMaxTime, so max(t, t_begin) - t_begin never exceeds kMaxTime (or is 0
// when the window starts past every event): with the bounds capped at 2^31
// the clamp gives the same values as in 64 bits, and a relative time
// shifted left by 2 still fits 32 bits next to a 2-bit value class.
// With 64-bit words (times up to 2^32 - 2) the same runs in 64 bits: the
// bounds are capped at 2^32 and a relative time needs 33 bits.
template <class P> struct RelClampT;
template <> struct RelClampT<uint32_t> {
    uint32_t lo, hi;
    __device__ __forceinline__ RelClampT(unsigned long long b, unsigned long long e)
        : lo((uint32_t)min(b, 1ull << 31)), hi((uint32_t)min(e, 1ull << 31)) {}
    __device__ __forceinline__ uint32_t operator()(uint32_t t) const { return min(max(t, lo), hi) - lo; }
};
template <> struct RelClampT<unsigned long long> {
    unsigned long long lo, hi;
    __device__ __forceinline__ RelClampT(unsigned long long b, unsigned long long e)
        : lo(min(b, 1ull << 32)), hi(min(e, 1ull << 32)) {}
    __device__ __forceinline__ unsigned long long operator()(uint32_t t) const
    {
        const unsigned long long x = t;
        return min(max(x, lo), hi) - lo;
    }
};
using RelClamp = RelClampT<uint32_t>;
// the packed (relative time << 2 | value class) and the sums of a window's word type
template <class Wd> using SaifP = typename std::conditional<std::is_same<Wd, uint32_t>::value, uint32_t,
                                                            unsigned long long>::type;

template <class P>
__device__ __forceinline__ void saif_add32(P acc[3], P cls, P d)
{
    acc[0] += cls == 0 ? d : P(0);
    acc[1] += cls == 1 ? d : P(0);
    acc[2] += cls == 2 ? d : P(0);
}

// SAIF contributions of W consecutive events of a list held one per lane of
// a W-lane group: an event holds the net from its time to the next event's,
// clipped to [t_begin, t_end) (src/simulate.cpp:102-163).  `prev` is the
// event before the group's first as (relative clamped time << 2 | value
// class) and is advanced past its last.  The sums of one segment or one
// list are at most one window long, so they fit 32 bits.
template <int W, class Wd, class P>
__device__ __forceinline__ void integrate_group(const RelClampT<P> &rc, Wd word, bool v, uint32_t n_here, bool any,
                                                P &prev, P acc[3])
{
    const unsigned FULL = 0xffffffffu;
    const int sub = threadIdx.x & (W - 1);
    const P me = (rc(ev_time(word)) << 2) | (P)vclass(ev_val(word));
    P pv = __shfl_up_sync(FULL, me, 1, W);
    if (sub == 0) pv = prev;
    if (v) saif_add32<P>(acc, pv & 3u, (me >> 2) - (pv >> 2));
    const int last = (int)min((uint32_t)(W - 1), n_here - 1);
    const P nx = __shfl_sync(FULL, me, last, W);
    if (any) prev = nx;
}

#ifndef GLS_COPY_UNROLL
#define GLS_COPY_UNROLL 8
#endif
constexpr int kCopyUnroll = GLS_COPY_UNROLL;   // entries per lane loaded ahead in k_copy

// k_copy: one W-lane group per segment: copy the kept entries from the
// level scratch into the pool and add their SAIF contributions to the gate
// output's counters.  The next segment's record is loaded while the current
// one is copied.
template <bool kBatch, int W, class Wd>
#ifndef GLS_COPY_BLOCKS
#define GLS_COPY_BLOCKS 5   // resident blocks per SM the copy kernel is compiled for (48 registers)
#endif
__global__ void __launch_bounds__(256, GLS_COPY_BLOCKS) k_copy(const WinSet<kBatch> ws, LevelArgs a, uint32_t d0, uint32_t d1)
{
    const unsigned FULL = 0xffffffffu;
    __shared__ uint32_t s_pre[kBatch ? kMaxWave + 1 : 2];
    __shared__ uint32_t sm32[32];
    __shared__ uint32_t s_skip, s_base;
    const uint32_t nwin = ws.size();
    // The segments of gate outputs [d0, d1), counted from the segment tables
    // (fixed once planned; a failed plan leaves them zero).  A gate kernel of
    // another fan-in class may raise a window's flag while this runs: a
    // window whose flag was up before its link ran is skipped (its copy
    // records are stale), one raised later is copied harmlessly.
    uint32_t nseg;
    if (!kBatch) {
        if (threadIdx.x == 0) {
            const WinDev &w = ws.get(0);
            s_skip = *(volatile uint32_t *)w.err != 0;
            s_base = w.seg_base[d0];
            s_pre[0] = 0;
            s_pre[1] = w.seg_base[d1] - s_base;
        }
        __syncthreads();
        if (s_skip) return;
        nseg = s_pre[1];
    } else {
        nseg = window_prefix<false>(
            ws, [&](const WinDev &x) { return x.seg_base[d1] - x.seg_base[d0]; }, s_pre, sm32);
    }
    const int sub = threadIdx.x & (W - 1);
    const uint32_t gpb = blockDim.x / W;
    const uint32_t stride = gridDim.x * gpb;
    uint32_t s = blockIdx.x * gpb + threadIdx.x / W;
    // every group of a warp runs the same number of rounds (shuffles need the full warp)
    const uint32_t warp_first = blockIdx.x * gpb + (threadIdx.x & ~31u) / W;
    const uint32_t rounds = warp_first < nseg ? (nseg - warp_first + stride - 1) / stride : 0;
    auto fetch = [&](uint32_t q, uint32_t &win) {
        CopyRec c = {0, 0, 0, 0, 0, 0, 0};
        win = 0;
        if (q < nseg) {
            win = window_of(s_pre, nwin, q);
            const WinDev &x = ws.get(win);
            if (!kBatch) c = x.copies[q + s_base];
            else if (!*(volatile uint32_t *)x.err) c = x.copies[q - s_pre[win] + x.seg_base[d0]];
        }
        return c;
    };
    uint32_t cw;
    CopyRec c = fetch(s, cw);
    for (uint32_t r = 0; r < rounds; ++r, s += stride) {
        uint32_t nw;
        const CopyRec nx = fetch(s + stride, nw);
        const WinDev &w = ws.get(cw);
        const bool live = s < nseg && c.n > 0;
        using P = SaifP<Wd>;
        const RelClampT<P> rc(w.t_begin, w.t_end);
        P acc[3] = {0, 0, 0};
        // c.cprev is a clamped absolute time: at most the largest event time
        // unless the window starts past every event (then it is t_begin,
        // relative 0)
        P prev = (rc((uint32_t)min(c.cprev, (unsigned long long)EvW<Wd>::kMax)) << 2) | c.pclass;
        const uint32_t n = live ? c.n : 0;
        // groups of one warp may have different lengths: loop to the warp's longest
        uint32_t nmax = n;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nmax = max(nmax, __shfl_xor_sync(FULL, nmax, o));
        const uint64_t dst = !live ? 0 : (a.alloc_mode == kAllocBound ? c.dst : w.slot[c.drv] + c.dst);
        // kCopyUnroll loads per lane go out before the stores that follow
        // them: scratch and pool never overlap, and a segment's copy costs
        // one memory round trip per W * kCopyUnroll entries, not per W
        const Wd *__restrict__ sp = reinterpret_cast<const Wd *>(w.scratch) + c.src;
        Wd *__restrict__ dp = reinterpret_cast<Wd *>(w.pool) + dst;
        for (uint32_t i0 = 0; i0 < nmax; i0 += W * kCopyUnroll) {
            Wd wd[kCopyUnroll];
#pragma unroll
            for (int u = 0; u < kCopyUnroll; ++u) {
                const uint32_t i = i0 + u * W + sub;
                wd[u] = i < n ? __ldcs(sp + i) : Wd(0);   // read once: stream it past L1
            }
#pragma unroll
            for (int u = 0; u < kCopyUnroll; ++u) {
                const uint32_t ib = i0 + u * W;
                if (ib >= nmax) break;   // the same for the whole warp
                const uint32_t i = ib + sub;
                const bool v = i < n;
                if (v) dp[i] = wd[u];
                integrate_group<W, Wd, P>(rc, wd[u], v, ib < n ? n - ib : 1u, ib < n, prev, acc);
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int o = W / 2; o > 0; o >>= 1) acc[k] += __shfl_down_sync(FULL, acc[k], o, W);
        if (sub == 0 && live) {
            const uint32_t out_net = c.out_net;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if (acc[k]) atomicAdd(&w.saif[3ull * out_net + k], (unsigned long long)acc[k]);
        }
        c = nx;
        cw = nw;
    }
}

// ------------------------------------------------------- stimulus SAIF
// one warp per stimulus net; blockIdx.y is the window
template <bool kBatch, class Wd>
__global__ void __launch_bounds__(256) k_stim_saif(const WinSet<kBatch> ws)
{
    const WinDev &w = ws.get(blockIdx.y);
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= w.n_stim) return;
    const uint32_t net = w.stim_nets[i];
    const uint64_t off = w.net_off[net];
    const uint32_t len = w.net_len[net];
    using P = SaifP<Wd>;
    const RelClampT<P> rc(w.t_begin, w.t_end);
    P prev = 2u;   // before the first event: X from t_begin
    P acc[3] = {0, 0, 0};
    const Wd *pw = reinterpret_cast<const Wd *>(w.pool);
    for (uint32_t i0 = 0; i0 < len; i0 += 32) {
        const bool v = i0 + lane < len;
        const Wd word = v ? pw[off + i0 + lane] : Wd(0);
        integrate_group<32, Wd, P>(rc, word, v, len - i0, true, prev, acc);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    if (lane == 0) {
        // the last event holds until t_end
        unsigned long long tot[3] = {acc[0], acc[1], acc[2]};
        saif_add(tot, (int)(prev & 3u), w.t_end - (w.t_begin + (prev >> 2)));
        w.saif[3ull * net + 0] = tot[0];
        w.saif[3ull * net + 1] = tot[1];
        w.saif[3ull * net + 2] = tot[2];
    }
}

// One window goes by value, several through the device array dw.
#define GLS_DISPATCH(h, dw, nwin, LAUNCH)                       \
    do {                                                         \
        if ((nwin) == 1) {                                       \
            const WinSet<false> ws{h};                           \
            LAUNCH;                                              \
        } else {                                                 \
            const WinSet<true> ws{dw, nwin};                     \
            LAUNCH;                                              \
        }                                                        \
    } while (0)

// Windows of 64-bit event words (times past 2^30 - 2) run one at a time
// through the thread-per-segment kernels: the host never batches them.
void launch_stim_saif(const WinDev *dw, const WinDev &h, uint32_t nwin, uint32_t max_stim, bool wide, cudaStream_t st)
{
    if (!max_stim || !nwin) return;
    const dim3 grid((uint32_t)(((uint64_t)max_stim * 32 + 255) / 256), nwin);
    if (wide) {
        k_stim_saif<false, WideWord><<<grid, 256, 0, st>>>(WinSet<false>{h});
        return;
    }
    GLS_DISPATCH(h, dw, nwin, (k_stim_saif<decltype(ws)::kIsBatch, uint32_t><<<grid, 256, 0, st>>>(ws)));
}

void launch_wave_events(const WinDev *dw, uint32_t nwin, const LevelArgs &a, cudaStream_t st)
{
    k_wave_events<<<nwin, 1024, 0, st>>>(dw, a);
}

void launch_plan(const WinDev *dw, const WinDev &h, uint32_t nwin, const LevelArgs &a, cudaStream_t st)
{
    GLS_DISPATCH(h, dw, nwin, (k_plan<<<nwin, 1024, 0, st>>>(ws, a)));
}

// one block per resident slot of every SM
template <class Wd, int kV, class WS>
static void sim_thread(const WS &ws, const LevelArgs &a, int cls, uint32_t d0, uint32_t d1, int sm_count,
                       cudaStream_t st)
{
    constexpr bool B = std::is_same<WS, WinSet<true>>::value;
    constexpr uint32_t bs = sim_block<kV>();
    const int per_sm = (cls == 0 ? GLS_SIM1_BLOCKS : (cls == 1 ? GLS_SIM2_BLOCKS : (cls == 2 ? GLS_SIM3_BLOCKS : 4))) /
                       ((kV & kSimV256) ? 2 : 1);
    const int grid = sm_count * per_sm;
    switch (cls) {
    case 0: k_sim<1, B, Wd, kV><<<grid, bs, 0, st>>>(ws, a, d0, d1); break;
    case 1: k_sim<2, B, Wd, kV><<<grid, bs, 0, st>>>(ws, a, d0, d1); break;
    case 2: k_sim<3, B, Wd, kV><<<grid, bs, 0, st>>>(ws, a, d0, d1); break;
    default: k_sim<kMaxSlots, B, Wd, kV><<<grid, bs, 0, st>>>(ws, a, d0, d1); break;
    }
}

template <class Wd, class WS>
static void sim_kernels(const WS &ws, const LevelArgs &a, int cls, uint32_t d0, uint32_t d1, int sm_count,
                        cudaStream_t st)
{
    constexpr bool B = std::is_same<WS, WinSet<true>>::value;
    if (std::is_same<Wd, uint32_t>::value && ((a.warp_mask >> cls) & 1u)) {
        const int wgrid = sm_count * 8;
        switch (cls) {
        case 0: k_sim_warp<1, B><<<wgrid, 128, 0, st>>>(ws, a, d0, d1); return;
        case 1: k_sim_warp<2, B><<<wgrid, 128, 0, st>>>(ws, a, d0, d1); return;
        case 2: k_sim_warp<3, B><<<wgrid, 128, 0, st>>>(ws, a, d0, d1); return;
        default: break;
        }
    }
    if constexpr (std::is_same<Wd, uint32_t>::value) {
        switch (a.sim_variant) {
        case 1: sim_thread<Wd, 1>(ws, a, cls, d0, d1, sm_count, st); return;
        case 2: sim_thread<Wd, 2>(ws, a, cls, d0, d1, sm_count, st); return;
        case 3: sim_thread<Wd, 3>(ws, a, cls, d0, d1, sm_count, st); return;
        default: break;
        }
    }
    sim_thread<Wd, 0>(ws, a, cls, d0, d1, sm_count, st);
}

void launch_sim(const WinDev *dw, const WinDev &h, uint32_t nwin, const LevelArgs &a, int cls, uint32_t d0, uint32_t d1,
                int sm_count, cudaStream_t st)
{
    if (a.wide) {
        sim_kernels<WideWord>(WinSet<false>{h}, a, cls, d0, d1, sm_count, st);
        return;
    }
    GLS_DISPATCH(h, dw, nwin, sim_kernels<uint32_t>(ws, a, cls, d0, d1, sm_count, st));
}

void launch_link(const WinDev *dw, const WinDev &h, uint32_t nwin, const LevelArgs &a, uint32_t d0, uint32_t d1,
                 cudaStream_t st)
{
    const uint64_t warps = (uint64_t)(d1 - d0) * nwin;
    if (!warps) return;
    const uint32_t blocks = (uint32_t)((warps * 32 + 255) / 256);
    if (a.wide) {
        k_link<false, WideWord><<<blocks, 256, 0, st>>>(WinSet<false>{h}, a, d0, d1);
        return;
    }
    GLS_DISPATCH(h, dw, nwin, (k_link<decltype(ws)::kIsBatch, uint32_t><<<blocks, 256, 0, st>>>(ws, a, d0, d1)));
}

void launch_copy(const WinDev *dw, const WinDev &h, uint32_t nwin, const LevelArgs &a, uint32_t d0, uint32_t d1,
                 int sm_count, cudaStream_t st)
{
    const int grid = sm_count * 8;
    if (a.wide) {   // 8 lanes move 64 bytes a step, as 16 lanes of 32-bit words do
        k_copy<false, 8, WideWord><<<grid, 256, 0, st>>>(WinSet<false>{h}, a, d0, d1);
        return;
    }
    if (a.copy_lanes == 4) GLS_DISPATCH(h, dw, nwin, (k_copy<decltype(ws)::kIsBatch, 4, uint32_t><<<grid, 256, 0, st>>>(ws, a, d0, d1)));
    else if (a.copy_lanes == 8) GLS_DISPATCH(h, dw, nwin, (k_copy<decltype(ws)::kIsBatch, 8, uint32_t><<<grid, 256, 0, st>>>(ws, a, d0, d1)));
    else if (a.copy_lanes == 32) GLS_DISPATCH(h, dw, nwin, (k_copy<decltype(ws)::kIsBatch, 32, uint32_t><<<grid, 256, 0, st>>>(ws, a, d0, d1)));
    else GLS_DISPATCH(h, dw, nwin, (k_copy<decltype(ws)::kIsBatch, 16, uint32_t><<<grid, 256, 0, st>>>(ws, a, d0, d1)));
}

}  // namespace gls
