// Level kernels of the GB300 gate-level simulator (sm_103a).
//
// One level of gates is simulated by three launches:
//   k_plan     (1 CTA)   sizes every gate output's slot in the event pool and
//                        splits its fan-in timeline into time segments.
//   k_sim      (1 thread per segment) merges the segment's fan-in events,
//                        evaluates the cell truth table, picks the SDF delay
//                        and runs the inertial output stack of the reference
//                        serial simulator on the segment.
//   k_combine  (1 warp per gate output) applies the pops that later segments
//                        make into earlier ones, settles the one undecided
//                        duplicate at each segment bottom, compacts the list
//                        and accumulates T0/T1/TX (fused SAIF).
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

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *__restrict__ t, uint32_t n, uint32_t key)
{
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (t[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t lut_index(uint32_t curp, const DrvMeta &md)
{
    if (md.ident) return curp & ((1u << (2 * md.n_pins)) - 1u);
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

__global__ void __launch_bounds__(1024) k_plan(WinDev w, LevelArgs a)
{
    __shared__ unsigned long long sm64[32];
    __shared__ uint32_t sm32[32];
    __shared__ uint32_t s_seg;
    __shared__ unsigned long long s_base;
    if (*w.err) return;
    const uint32_t n = a.hi - a.lo;
    // total fan-in events of the level, to fit the segment table
    unsigned long long e_tot = 0, g_tot = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const DrvMeta &md = a.meta[a.lo + i];
        for (int j = 0; j < md.m; ++j) e_tot += w.net_len[md.net[j]];
        if (md.reserved) {  // first output of its instance: count fan-in per pin
            for (int p = 0; p < md.n_pins; ++p) g_tot += w.net_len[md.net[(md.pin_slot >> (3 * p)) & 7u]];
        }
    }
    unsigned long long tot;
    block_excl_scan<unsigned long long>(e_tot, &tot, sm64);
    e_tot = tot;
    block_excl_scan<unsigned long long>(g_tot, &tot, sm64);
    g_tot = tot;
    if (threadIdx.x == 0) {
        uint32_t seg = max(a.seg_events, 8u);
        if (w.seg_cap <= n) {
            atomicOr(w.err, kErrSegCap);
        } else {
            unsigned long long room = w.seg_cap - n;
            unsigned long long need = (e_tot + room - 1) / room;
            if (need > seg) seg = (uint32_t)min(need + 1, 0xFFFFFFFull);
        }
        s_seg = seg;
        s_base = *w.top;
        atomicAdd(&w.counters[0], g_tot);
        atomicAdd(&w.counters[3], e_tot);
    }
    __syncthreads();
    if (*w.err) return;
    const uint32_t seg = s_seg;
    const unsigned long long base = s_base;
    uint32_t run_seg = 0;
    unsigned long long run_slot = 0;
    for (uint32_t c = 0; c < n; c += blockDim.x) {
        const uint32_t i = c + threadIdx.x;
        uint32_t S = 0;
        unsigned long long slot = 0;
        if (i < n) {
            const DrvMeta &md = a.meta[a.lo + i];
            unsigned long long E = 0;
            for (int j = 0; j < md.m; ++j) E += w.net_len[md.net[j]];
            S = (uint32_t)max(1ull, (E + seg - 1) / seg);
            slot = (E + S + 3) & ~3ull;
        }
        uint32_t tS;
        unsigned long long tSlot;
        uint32_t xs = block_excl_scan<uint32_t>(S, &tS, sm32);
        unsigned long long xo = block_excl_scan<unsigned long long>(slot, &tSlot, sm64);
        if (i < n) {
            w.seg_base[i] = run_seg + xs;
            const unsigned long long st = base + run_slot + xo;
            w.slot[i] = st;
            w.net_off[a.meta[a.lo + i].out_net] = st;
        }
        run_seg += tS;
        run_slot += tSlot;
    }
    if (threadIdx.x == 0) {
        w.seg_base[n] = run_seg;
        *w.n_segs = run_seg;
        if (run_seg > w.seg_cap) atomicOr(w.err, kErrSegCap);
        if (base + run_slot > w.cap) atomicOr(w.err, kErrPool);
        else *w.top = base + run_slot;
        atomicAdd(&w.counters[2], (unsigned long long)run_seg);
    }
}

// ------------------------------------------------------------------- sim
template <int M>
__device__ void sim_segment(const WinDev &w, const LevelArgs &a, const DrvMeta &md, uint32_t s,
                            uint32_t S, uint32_t seg_id, uint64_t slot)
{
    const uint32_t *bt[M];
    const uint8_t *bv[M];
    uint32_t len[M], pos[M], end[M], ht[M];
    const int m = md.m;
    int piv = 0;
    uint32_t plen = 0;
#pragma unroll
    for (int j = 0; j < M; ++j) {
        len[j] = 0; bt[j] = w.pool_t; bv[j] = w.pool_v;
        if (j < m) {
            const uint32_t net = md.net[j];
            const uint64_t off = w.net_off[net];
            len[j] = w.net_len[net];
            bt[j] = w.pool_t + off;
            bv[j] = w.pool_v + off;
            if (len[j] > plen) { plen = len[j]; piv = j; }
        }
    }
    const uint32_t *pt = w.pool_t;
#pragma unroll
    for (int j = 0; j < M; ++j) if (j == piv) pt = bt[j];
    const uint32_t tlo = s > 0 ? pt[(uint64_t)s * plen / S] : 0u;
    const uint32_t thi = s + 1 < S ? pt[(uint64_t)(s + 1) * plen / S] : kInf;
    uint32_t curp = 0x555u;   // every slot X
    uint32_t region = s, capn = 1;
    bool before = false;
#pragma unroll
    for (int j = 0; j < M; ++j) {
        pos[j] = end[j] = 0;
        ht[j] = kInf;
        if (j < m) {
            const uint32_t b = s > 0 ? lower_bound_u32(bt[j], len[j], tlo) : 0u;
            const uint32_t e = s + 1 < S ? lower_bound_u32(bt[j], len[j], thi) : len[j];
            region += b;
            capn += e - b;
            pos[j] = b; end[j] = e;
            if (b > 0) {
                curp = (curp & ~(3u << (2 * j))) | ((uint32_t)bv[j][b - 1] << (2 * j));
                before = true;
            }
            if (b < e) ht[j] = bt[j][b];
        }
    }
    const uint8_t *lut = a.lut + md.lut_off;
    const ArcDev *arcs = a.arcs + md.arc_off;
    uint32_t *ot = w.pool_t + slot + region;
    uint8_t *ov = w.pool_v + slot + region;
    uint32_t cnt = 0, top_t = 0, top_v = kVX;
    int popped_v = -1;
    if (s == 0) { ot[0] = 0; ov[0] = kVX; cnt = 1; }
    uint32_t fprev = before ? lut[lut_index(curp, md)] : kVX;
    uint32_t min_o = kInf;
    for (;;) {
        uint32_t t = ht[0];
#pragma unroll
        for (int j = 1; j < M; ++j) t = min(t, ht[j]);
        if (t == kInf) break;
        const uint32_t lastp = curp;
        uint32_t chg = 0;
#pragma unroll
        for (int j = 0; j < M; ++j) {
            if (ht[j] == t) {
                chg |= 1u << j;
                const uint32_t v = bv[j][pos[j]];
                curp = (curp & ~(3u << (2 * j))) | (v << (2 * j));
                ++pos[j];
                ht[j] = pos[j] < end[j] ? bt[j][pos[j]] : kInf;
            }
        }
        const uint32_t F = lut[lut_index(curp, md)];
        if (F == fprev) continue;
        const int so = check_delay(fprev, F);
        fprev = F;
        const uint32_t d = select_delay(arcs, md.n_arcs, chg, so, curp, lastp, a.def_delay);
        const uint32_t o = t + d;
        if (o < t || o == kInf) { atomicOr(w.err, kErrTime); break; }
        min_o = min(min_o, o);
        // inertial update, src/simulate.cpp:991-1009
        while (cnt > 0 && top_t >= o) {
            if (s == 0 && cnt == 1) { popped_v = (int)top_v; cnt = 0; break; }
            --cnt;
            if (cnt > 0) { top_t = ot[cnt - 1]; top_v = ov[cnt - 1]; }
        }
        const int prevv = cnt > 0 ? (int)top_v : (s == 0 ? popped_v : -1);
        if (prevv != (int)F) {
            if (cnt >= capn) { atomicOr(w.err, kErrRegion); break; }
            ot[cnt] = o; ov[cnt] = (uint8_t)F;
            ++cnt; top_t = o; top_v = F;
        } else if (cnt == 0) {
            atomicOr(w.err, kErrEmptied);
            break;
        }
    }
    SegRec r;
    r.region = region; r.cnt = cnt; r.min_o = min_o; r.fin = 0;
    w.segs[seg_id] = r;
}

__global__ void __launch_bounds__(128) k_sim(WinDev w, LevelArgs a)
{
    if (*w.err) return;
    const uint32_t n = a.hi - a.lo;
    const uint32_t nseg = *w.n_segs;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < nseg; g += gridDim.x * blockDim.x) {
        // driver owning segment g: last i with seg_base[i] <= g
        uint32_t lo = 0, hi = n;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (w.seg_base[mid] <= g) lo = mid; else hi = mid;
        }
        const uint32_t i = lo;
        const uint32_t sb = w.seg_base[i];
        const uint32_t S = w.seg_base[i + 1] - sb;
        const DrvMeta md = a.meta[a.lo + i];
        const uint64_t slot = w.slot[i];
        if (md.m <= 2) sim_segment<2>(w, a, md, g - sb, S, g, slot);
        else if (md.m == 3) sim_segment<3>(w, a, md, g - sb, S, g, slot);
        else sim_segment<kMaxSlots>(w, a, md, g - sb, S, g, slot);
    }
}

// --------------------------------------------------------------- combine
__device__ __forceinline__ unsigned long long clampt(uint32_t t, unsigned long long lo, unsigned long long hi)
{
    unsigned long long x = t;
    return x < lo ? lo : (x > hi ? hi : x);
}
__device__ __forceinline__ int vclass(uint32_t v) { return v == kV0 ? 0 : (v == kV1 ? 1 : 2); }

// Copy `n` events from pool[src..] to pool[dst..] (dst <= src) and add their
// SAIF contributions: event i holds the net from its time until the next
// event, clipped to [t_begin, t_end) (src/simulate.cpp:102-163).
__device__ void copy_and_integrate(const WinDev &w, uint64_t src, uint64_t dst, uint32_t n,
                                   unsigned long long &cprev, int &pclass, unsigned long long acc[3])
{
    const int lane = threadIdx.x & 31;
    for (uint32_t i0 = 0; i0 < n; i0 += 32) {
        const uint32_t i = i0 + lane;
        const bool v = i < n;
        uint32_t t = 0, val = 0;
        if (v) { t = w.pool_t[src + i]; val = w.pool_v[src + i]; }
        __syncwarp();
        if (v && src != dst) { w.pool_t[dst + i] = t; w.pool_v[dst + i] = (uint8_t)val; }
        const unsigned long long c = clampt(t, w.t_begin, w.t_end);
        unsigned long long cp = __shfl_up_sync(0xffffffffu, c, 1);
        int pc = __shfl_up_sync(0xffffffffu, vclass(val), 1);
        if (lane == 0) { cp = cprev; pc = pclass; }
        if (v) {
            const unsigned long long dlt = c - cp;
            if (pc == 0) acc[0] += dlt; else if (pc == 1) acc[1] += dlt; else acc[2] += dlt;
        }
        const int last = (int)min(31u, n - 1 - i0);
        cprev = __shfl_sync(0xffffffffu, c, last);
        pclass = __shfl_sync(0xffffffffu, vclass(val), last);
    }
}

__global__ void __launch_bounds__(256) k_combine(WinDev w, LevelArgs a)
{
    if (*w.err) return;
    const uint32_t n = a.hi - a.lo;
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const uint32_t sb = w.seg_base[i], se = w.seg_base[i + 1];
    const uint64_t slot = w.slot[i];
    const uint32_t out_net = a.meta[a.lo + i].out_net;
    // pass A (right to left): cut each segment's stack at the smallest
    // candidate time of all later segments.
    uint32_t carry_min = kInf;
    for (int64_t base = se; base > (int64_t)sb; base -= 32) {
        const int64_t s = base - 32 + lane;
        const bool valid = s >= (int64_t)sb;
        SegRec r = {0, 0, kInf, 0};
        if (valid) r = w.segs[s];
        uint32_t x = r.min_o;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_down_sync(0xffffffffu, x, o);
            if (lane + o < 32) x = min(x, y);
        }
        uint32_t ex = __shfl_down_sync(0xffffffffu, x, 1);
        if (lane == 31) ex = kInf;
        const uint32_t M = min(ex, carry_min);
        if (valid) {
            const uint32_t keep = lower_bound_u32(w.pool_t + slot + r.region, r.cnt, M);
            w.segs[s].fin = keep;
        }
        carry_min = min(carry_min, __shfl_sync(0xffffffffu, x, 0));
    }
    __syncwarp();
    // pass B (left to right): settle the bottom entry of every segment after
    // the first, place the segments back to back, integrate SAIF.
    uint32_t carry_pos = 0;
    uint32_t carry_v = kVX;
    unsigned long long cprev = w.t_begin;
    int pclass = 2;
    unsigned long long acc[3] = {0, 0, 0};
    for (uint32_t base = sb; base < se; base += 32) {
        const uint32_t s = base + lane;
        const bool valid = s < se;
        uint32_t keep = 0, region = 0, firstv = 0, lastv = 0;
        if (valid) {
            const SegRec r = w.segs[s];
            keep = r.fin;
            region = r.region;
            if (keep) {
                firstv = w.pool_v[slot + region];
                lastv = w.pool_v[slot + region + keep - 1];
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep > 0);
        const unsigned prior = bal & ((1u << lane) - 1u);
        const int srcl = prior ? 31 - __clz(prior) : 0;
        const uint32_t vsh = __shfl_sync(0xffffffffu, lastv, srcl);
        const uint32_t vprev = prior ? vsh : carry_v;
        const uint32_t drop = (s > sb && keep > 0 && firstv == vprev) ? 1u : 0u;
        const uint32_t fin = keep - drop;
        uint32_t inc = fin;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        const uint32_t pos = carry_pos + inc - fin;
        if (bal) carry_v = __shfl_sync(0xffffffffu, lastv, 31 - __clz(bal));
        carry_pos += __shfl_sync(0xffffffffu, inc, 31);
        const uint32_t cnt_here = min(32u, se - base);
        for (uint32_t k = 0; k < cnt_here; ++k) {
            const uint32_t kf = __shfl_sync(0xffffffffu, fin, k);
            const uint32_t kr = __shfl_sync(0xffffffffu, region + drop, k);
            const uint32_t kp = __shfl_sync(0xffffffffu, pos, k);
            if (kf) copy_and_integrate(w, slot + kr, slot + kp, kf, cprev, pclass, acc);
        }
    }
    // the last event holds until t_end
    if (lane == 0) {
        const unsigned long long dlt = w.t_end - cprev;
        if (pclass == 0) acc[0] += dlt; else if (pclass == 1) acc[1] += dlt; else acc[2] += dlt;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    if (lane == 0) {
        w.net_len[out_net] = carry_pos;
        w.saif[3ull * out_net + 0] = acc[0];
        w.saif[3ull * out_net + 1] = acc[1];
        w.saif[3ull * out_net + 2] = acc[2];
        atomicAdd(&w.counters[1], (unsigned long long)carry_pos);
    }
}

// ------------------------------------------------------- stimulus SAIF
__global__ void __launch_bounds__(256) k_stim_saif(WinDev w, const uint32_t *__restrict__ nets, uint32_t n)
{
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const uint32_t net = nets[i];
    const uint64_t off = w.net_off[net];
    const uint32_t len = w.net_len[net];
    unsigned long long cprev = w.t_begin;
    int pclass = 2;
    unsigned long long acc[3] = {0, 0, 0};
    copy_and_integrate(w, off, off, len, cprev, pclass, acc);
    if (lane == 0) {
        const unsigned long long dlt = w.t_end - cprev;
        if (pclass == 0) acc[0] += dlt; else if (pclass == 1) acc[1] += dlt; else acc[2] += dlt;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    if (lane == 0) {
        w.saif[3ull * net + 0] = acc[0];
        w.saif[3ull * net + 1] = acc[1];
        w.saif[3ull * net + 2] = acc[2];
    }
}

void launch_stim_saif(const WinDev &w, const uint32_t *stim_nets, uint32_t n_stim, cudaStream_t st)
{
    if (!n_stim) return;
    const uint32_t blocks = (uint32_t)(((uint64_t)n_stim * 32 + 255) / 256);
    k_stim_saif<<<blocks, 256, 0, st>>>(w, stim_nets, n_stim);
}

void launch_plan(const WinDev &w, const LevelArgs &a, cudaStream_t st)
{
    k_plan<<<1, 1024, 0, st>>>(w, a);
}

void launch_sim(const WinDev &w, const LevelArgs &a, int sm_count, cudaStream_t st)
{
    k_sim<<<sm_count * 16, 128, 0, st>>>(w, a);
}

void launch_combine(const WinDev &w, const LevelArgs &a, cudaStream_t st)
{
    const uint32_t n = a.hi - a.lo;
    const uint32_t blocks = (uint32_t)(((uint64_t)n * 32 + 255) / 256);
    k_combine<<<blocks, 256, 0, st>>>(w, a);
}

}  // namespace gls
