// gls_pack_levels: the packed per-level tables of `process` on the GPU.
//
// The reference's `process` lays its levelized design out for its GPU
// simulator (src/process.cpp:423-566): per level the first instance, the
// widest delay list and the widest function program; per instance its net
// counts, the start of its inputs within the level and its delay and
// program sizes; and two tables padded to each level's width, holding every
// instance's delay arcs and its function program rows (each row padded to
// the level width divided by the instance's row count), -1 where an
// instance has fewer entries.  Here a thread per instance counts and
// raises its level's widths, a scan gives the positions of the inputs, one
// block places the levels, and a thread per instance fills its padded rows.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <vector>
#include "gls.h"

namespace {

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;
constexpr uint32_t kScanTile = kScanBlock * kScanItems;

struct PackDev {
    uint32_t n_levels, n_inst;
    const uint32_t *level_start;
    const uint16_t *n_in, *n_out;
    const uint32_t *arc_start;
    const gls_pack_arc *arcs;
    const uint32_t *row_start, *entry_start;
    const int16_t *entries;
    uint32_t *data_in_num_start, *data_out_num_start, *delay_start, *delay_width, *functions_start, *functions_width;
    int16_t *data_in_num, *data_out_num;
    uint32_t *val_num_start;
    int16_t *delay_val_num, *functions_func_num, *functions_val_num;
    int16_t *delay_edges, *in_bit, *out_bit;
    float *rise_val, *fall_val;
    int16_t *functions;
    unsigned long long *in_prefix;   // exclusive prefix of n_in over all instances
    unsigned long long *tile_sum;    // per scan tile
    unsigned long long *totals;      // [0] delay entries, [1] function entries
};

__device__ __forceinline__ uint32_t level_of(const uint32_t *__restrict__ ls, uint32_t nl, uint32_t i)
{
    uint32_t lo = 0, hi = nl;   // last L with ls[L] <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (ls[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// every instance's counts; its level's widths raised to its own
__global__ void k_pack_counts(PackDev p)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n_inst) return;
    const uint32_t L = level_of(p.level_start, p.n_levels, i);
    p.data_in_num[i] = (int16_t)p.n_in[i];
    p.data_out_num[i] = (int16_t)p.n_out[i];
    const uint32_t nd = p.arc_start[i + 1] - p.arc_start[i];
    p.delay_val_num[i] = (int16_t)nd;
    const uint32_t r0 = p.row_start[i], r1 = p.row_start[i + 1];
    uint32_t w = 0;
    for (uint32_t r = r0; r < r1; ++r) w = max(w, p.entry_start[r + 1] - p.entry_start[r]);
    p.functions_func_num[i] = (int16_t)(r1 - r0);
    p.functions_val_num[i] = (int16_t)w;
    atomicMax(&p.delay_width[L], nd);
    atomicMax(&p.functions_width[L], w * (r1 - r0));
}

// block-wide exclusive scan of one value per thread; *total gets the sum
__device__ unsigned long long block_excl(unsigned long long v, unsigned long long *total)
{
    __shared__ unsigned long long warp_sum[kScanBlock / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        unsigned long long s = lane < (int)(blockDim.x >> 5) ? warp_sum[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sum[lane] = s;   // inclusive over warps
    }
    __syncthreads();
    const unsigned long long before = (wid ? warp_sum[wid - 1] : 0ull) + x - v;
    *total = warp_sum[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

// exclusive prefix of n_in within each tile of kScanTile instances, and the tile's sum
__global__ void __launch_bounds__(kScanBlock) k_scan_tiles(PackDev p)
{
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    unsigned long long v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < p.n_inst ? p.n_in[base + k] : 0u;
        s += v[k];
    }
    unsigned long long tot;
    unsigned long long run = block_excl(s, &tot);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < p.n_inst) p.in_prefix[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) p.tile_sum[blockIdx.x] = tot;
}

// One block: the tiles' offsets, then every level's starts and the padded
// tables' sizes, both by chunked scans (each thread a run of entries).
__global__ void __launch_bounds__(kScanBlock) k_scan_levels(PackDev p, uint32_t n_tiles)
{
    const uint32_t per_t = (n_tiles + kScanBlock - 1) / kScanBlock;
    const uint32_t t0 = min(n_tiles, threadIdx.x * per_t), t1 = min(n_tiles, t0 + per_t);
    unsigned long long s = 0, tot;
    for (uint32_t t = t0; t < t1; ++t) s += p.tile_sum[t];
    unsigned long long run = block_excl(s, &tot);
    for (uint32_t t = t0; t < t1; ++t) {
        const unsigned long long x = p.tile_sum[t];
        p.tile_sum[t] = run;
        run += x;
    }
    const uint32_t per = (p.n_levels + kScanBlock - 1) / kScanBlock;
    const uint32_t l0 = min(p.n_levels, threadIdx.x * per), l1 = min(p.n_levels, l0 + per);
    unsigned long long sd = 0, sf = 0, td, tf;
    for (uint32_t L = l0; L < l1; ++L) {
        const unsigned long long cnt = p.level_start[L + 1] - p.level_start[L];
        sd += cnt * p.delay_width[L];
        sf += cnt * p.functions_width[L];
    }
    unsigned long long rd = block_excl(sd, &td), rf = block_excl(sf, &tf);
    for (uint32_t L = l0; L < l1; ++L) {
        const unsigned long long cnt = p.level_start[L + 1] - p.level_start[L];
        p.data_in_num_start[L] = p.level_start[L];
        p.data_out_num_start[L] = p.level_start[L];
        p.delay_start[L] = (uint32_t)rd;
        p.functions_start[L] = (uint32_t)rf;
        rd += cnt * p.delay_width[L];
        rf += cnt * p.functions_width[L];
    }
    if (threadIdx.x == 0) {
        p.totals[0] = td;
        p.totals[1] = tf;
    }
}

// the start of each instance's inputs within its level
__global__ void k_val_num(PackDev p)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n_inst) return;
    const uint32_t L = level_of(p.level_start, p.n_levels, i);
    const uint32_t f = p.level_start[L];
    const unsigned long long at = p.in_prefix[i] + p.tile_sum[i / kScanTile];
    const unsigned long long first = p.in_prefix[f] + p.tile_sum[f / kScanTile];
    p.val_num_start[i] = (uint32_t)(at - first);
}

// every instance's rows of the padded delay and function tables
__global__ void k_pack_fill(PackDev p)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n_inst) return;
    const uint32_t L = level_of(p.level_start, p.n_levels, i);
    const uint64_t j = i - p.level_start[L];
    const uint32_t dw = p.delay_width[L], a0 = p.arc_start[i], na = p.arc_start[i + 1] - a0;
    const uint64_t d0 = p.delay_start[L] + j * dw;
    for (uint32_t k = 0; k < dw; ++k) {
        if (k < na) {
            const gls_pack_arc a = p.arcs[a0 + k];
            p.delay_edges[d0 + k] = a.edge;
            p.in_bit[d0 + k] = a.in_pos;
            p.out_bit[d0 + k] = a.out_pos;
            p.rise_val[d0 + k] = a.rise;
            p.fall_val[d0 + k] = a.fall;
        } else {
            p.delay_edges[d0 + k] = p.in_bit[d0 + k] = p.out_bit[d0 + k] = -1;
            p.rise_val[d0 + k] = p.fall_val[d0 + k] = -1.0f;
        }
    }
    const uint32_t fw = p.functions_width[L], r0 = p.row_start[i], h = p.row_start[i + 1] - r0;
    const uint32_t w = h ? fw / h : 0;   // the row stride: the level width over this instance's rows
    const uint64_t f0 = p.functions_start[L] + j * fw;
    for (uint32_t r = 0; r < h; ++r) {
        const uint32_t e0 = p.entry_start[r0 + r], n = p.entry_start[r0 + r + 1] - e0;
        for (uint32_t k = 0; k < w; ++k) p.functions[f0 + r * w + k] = k < n ? p.entries[e0 + k] : (int16_t)-1;
    }
    for (uint32_t k = w * h; k < fw; ++k) p.functions[f0 + k] = -1;
}

struct Bufs {
    std::vector<void *> all;
    cudaError_t err = cudaSuccess;
    template <class T> T *get(size_t n)
    {
        void *q = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
        if (err == cudaSuccess) all.push_back(q);
        return static_cast<T *>(q);
    }
    template <class T> T *up(const T *h, size_t n)
    {
        T *d = get<T>(n);
        if (err == cudaSuccess && n) err = cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice);
        return d;
    }
    ~Bufs()
    {
        for (void *q : all) cudaFree(q);
    }
};

template <class T> cudaError_t down(T *h, const T *d, size_t n)
{
    return n ? cudaMemcpy(h, d, n * sizeof(T), cudaMemcpyDeviceToHost) : cudaSuccess;
}

}  // namespace

extern "C" int gls_pack_levels(int device, const gls_pack_in *in, gls_pack_out *out)
{
    if (!in || !out) return GLS_EINVAL;
    const uint32_t nl = in->n_levels, n = in->n_inst;
    if (!in->level_start || in->level_start[0] != 0 || in->level_start[nl] != n) return GLS_EINVAL;
    for (uint32_t L = 0; L < nl; ++L)
        if (in->level_start[L + 1] < in->level_start[L]) return GLS_EINVAL;
    if (n && (!in->n_in || !in->n_out || !in->arc_start || !in->row_start)) return GLS_EINVAL;
    const uint32_t n_arcs = n ? in->arc_start[n] : 0, n_rows = n ? in->row_start[n] : 0;
    for (uint32_t i = 0; i < n; ++i)
        if (in->arc_start[i + 1] < in->arc_start[i] || in->row_start[i + 1] < in->row_start[i]) return GLS_EINVAL;
    if ((n_arcs && !in->arcs) || (n_rows && !in->entry_start)) return GLS_EINVAL;
    const uint32_t n_ent = n_rows ? in->entry_start[n_rows] : 0;
    for (uint32_t r = 0; r < n_rows; ++r)
        if (in->entry_start[r + 1] < in->entry_start[r]) return GLS_EINVAL;
    if (n_ent && !in->entries) return GLS_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return GLS_ECUDA;
    const uint32_t n_tiles = (n + kScanTile - 1) / kScanTile;
    Bufs b;
    PackDev p{};
    p.n_levels = nl;
    p.n_inst = n;
    p.level_start = b.up(in->level_start, (size_t)nl + 1);
    p.n_in = b.up(in->n_in, n);
    p.n_out = b.up(in->n_out, n);
    p.arc_start = b.up(in->arc_start, (size_t)n + 1);
    p.arcs = b.up(in->arcs, n_arcs);
    p.row_start = b.up(in->row_start, (size_t)n + 1);
    std::vector<uint32_t> one_zero(1, 0);
    p.entry_start = n_rows ? b.up(in->entry_start, (size_t)n_rows + 1) : b.up(one_zero.data(), 1);
    p.entries = b.up(in->entries, n_ent);
    p.data_in_num_start = b.get<uint32_t>(nl);
    p.data_out_num_start = b.get<uint32_t>(nl);
    p.delay_start = b.get<uint32_t>(nl);
    p.delay_width = b.get<uint32_t>(nl);
    p.functions_start = b.get<uint32_t>(nl);
    p.functions_width = b.get<uint32_t>(nl);
    p.data_in_num = b.get<int16_t>(n);
    p.data_out_num = b.get<int16_t>(n);
    p.val_num_start = b.get<uint32_t>(n);
    p.delay_val_num = b.get<int16_t>(n);
    p.functions_func_num = b.get<int16_t>(n);
    p.functions_val_num = b.get<int16_t>(n);
    p.in_prefix = b.get<unsigned long long>(n);
    p.tile_sum = b.get<unsigned long long>(n_tiles);
    p.totals = b.get<unsigned long long>(2);
    if (b.err != cudaSuccess) return b.err == cudaErrorMemoryAllocation ? GLS_ENOMEM : GLS_ECUDA;
    if (nl) {
        cudaMemset(p.delay_width, 0, nl * 4);
        cudaMemset(p.functions_width, 0, nl * 4);
    }
    const uint32_t grid = (n + 255) / 256;
    if (n) {
        k_pack_counts<<<grid, 256>>>(p);
        k_scan_tiles<<<n_tiles, kScanBlock>>>(p);
    }
    k_scan_levels<<<1, kScanBlock>>>(p, n_tiles);
    if (n) k_val_num<<<grid, 256>>>(p);
    unsigned long long tot[2] = {0, 0};
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = down(tot, p.totals, 2);
    if (e != cudaSuccess) return GLS_ECUDA;
    out->delay_total = tot[0];
    out->functions_total = tot[1];
    // the reference keeps these starts in 32 bits
    if (tot[0] > 0xFFFFFFFFull || tot[1] > 0xFFFFFFFFull) return GLS_ERANGE;
    if (tot[0] > out->delay_cap || tot[1] > out->functions_cap) return GLS_EOVERFLOW;
    p.delay_edges = b.get<int16_t>(tot[0]);
    p.in_bit = b.get<int16_t>(tot[0]);
    p.out_bit = b.get<int16_t>(tot[0]);
    p.rise_val = b.get<float>(tot[0]);
    p.fall_val = b.get<float>(tot[0]);
    p.functions = b.get<int16_t>(tot[1]);
    if (b.err != cudaSuccess) return b.err == cudaErrorMemoryAllocation ? GLS_ENOMEM : GLS_ECUDA;
    if (n) k_pack_fill<<<grid, 256>>>(p);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = down(out->data_in_num_start, p.data_in_num_start, nl);
    if (e == cudaSuccess) e = down(out->data_out_num_start, p.data_out_num_start, nl);
    if (e == cudaSuccess) e = down(out->delay_start, p.delay_start, nl);
    if (e == cudaSuccess) e = down(out->delay_width, p.delay_width, nl);
    if (e == cudaSuccess) e = down(out->functions_start, p.functions_start, nl);
    if (e == cudaSuccess) e = down(out->functions_width, p.functions_width, nl);
    if (e == cudaSuccess) e = down(out->data_in_num, p.data_in_num, n);
    if (e == cudaSuccess) e = down(out->data_out_num, p.data_out_num, n);
    if (e == cudaSuccess) e = down(out->val_num_start, p.val_num_start, n);
    if (e == cudaSuccess) e = down(out->delay_val_num, p.delay_val_num, n);
    if (e == cudaSuccess) e = down(out->functions_func_num, p.functions_func_num, n);
    if (e == cudaSuccess) e = down(out->functions_val_num, p.functions_val_num, n);
    if (e == cudaSuccess) e = down(out->delay_edges, p.delay_edges, tot[0]);
    if (e == cudaSuccess) e = down(out->in_bit, p.in_bit, tot[0]);
    if (e == cudaSuccess) e = down(out->out_bit, p.out_bit, tot[0]);
    if (e == cudaSuccess) e = down(out->rise_val, p.rise_val, tot[0]);
    if (e == cudaSuccess) e = down(out->fall_val, p.fall_val, tot[0]);
    if (e == cudaSuccess) e = down(out->functions, p.functions, tot[1]);
    return e == cudaSuccess ? GLS_OK : GLS_ECUDA;
}
