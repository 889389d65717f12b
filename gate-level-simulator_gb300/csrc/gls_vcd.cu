// gls_vcd_scan: the body of a VCD file (after $enddefinitions) turned into
// bit changes on the GPU.
//
// The reference reads VCD text with one thread (VCDParser::parse_core,
// src/VCDParser.cpp:508-644) and then bit-blasts buses (combine_core,
// 458-507, and core, 194-242).  Here every step is data-parallel over bytes
// or tokens:
//   1. token starts: a tile of bytes per block, a block scan inside the
//      tile and a device scan of the tiles' counts for their places;
//   2. token classes: times (#), value changes (scalar 0/1/x/z<code>,
//      vector b<bits> <code>, real r<value> <code>), keywords,
//      $comment ... $end;
//   3. one scan of four running maxima: the last $comment opener, the last
//      $end, the start of the current run of b/r tokens (a b/r token takes
//      the next token as its identifier code, so in a run of them every
//      second one is a code) and the last time;
//   4. per change token its bit count (the code looked up in the sorted
//      code table), a scan for places, and the bits written with the time
//      in force.
// The host then appends the changes per signal in file order (the
// same-time replacement and the bus-bit filtering of the host reader).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include "gls.h"

namespace {

constexpr uint32_t kTileBytes = 8192;        // bytes per block in the token-start pass
constexpr uint32_t kBytesPerThread = 32;     // 256 threads per tile
constexpr uint32_t kScanItems = 16;          // items per thread in the device scans (tiles of 4096)
constexpr uint32_t kScanTile = 256 * kScanItems;

enum : uint8_t { kOther = 0, kTime, kOpen, kEnd, kKey, kVec, kReal, kScalar };

__device__ __forceinline__ bool is_space(uint8_t c) { return c == ' ' || (c >= 9 && c <= 13); }

__device__ __forceinline__ uint8_t value_code(uint8_t c)
{
    return c == '0' ? 0 : c == '1' ? 3 : (c == 'x' || c == 'X') ? 1 : (c == 'z' || c == 'Z') ? 2 : 255;
}

__device__ __forceinline__ uint32_t shfl_up(uint32_t v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
__device__ __forceinline__ unsigned long long shfl_up(unsigned long long v, int o)
{
    return __shfl_up_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ uint4 shfl_up(uint4 v, int o)
{
    return make_uint4(shfl_up(v.x, o), shfl_up(v.y, o), shfl_up(v.z, o), shfl_up(v.w, o));
}

struct Sum {
    __device__ uint32_t operator()(uint32_t a, uint32_t b) const { return a + b; }
    __device__ uint32_t ident() const { return 0u; }
};
struct Sum64 {
    __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a + b; }
    __device__ unsigned long long ident() const { return 0ull; }
};
struct Max4 {   // four running maxima at once
    __device__ uint4 operator()(uint4 a, uint4 b) const
    {
        return make_uint4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w));
    }
    __device__ uint4 ident() const { return make_uint4(0, 0, 0, 0); }
};

// inclusive scan over the block; every thread gets its own prefix
template <typename T, typename Op>
__device__ T block_incl_scan(T x, T *sm32, Op op)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = shfl_up(x, o);
        if (lane >= o) x = op(x, y);
    }
    if (lane == 31) sm32[wid] = x;
    __syncthreads();
    if (wid == 0) {
        T v = lane < nw ? sm32[lane] : op.ident();
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = shfl_up(v, o);
            if (lane >= o) v = op(v, y);
        }
        sm32[lane] = v;
    }
    __syncthreads();
    const T r = wid ? op(sm32[wid - 1], x) : x;
    __syncthreads();
    return r;
}

// ------------------------------------------------------------ device scans
// Inclusive scan of n items: tile aggregates, one block scanning those, then
// every tile again from its carry-in.
template <typename T, typename Op>
__global__ void __launch_bounds__(256) k_tile_reduce(const T *__restrict__ in, uint64_t n, T *agg, Op op)
{
    __shared__ T sm[32];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    T x = op.ident();
    for (uint32_t j = 0; j < kScanItems; ++j)
        if (base + j < n) x = op(x, in[base + j]);
    const T r = block_incl_scan<T>(x, sm, op);
    if (threadIdx.x == blockDim.x - 1) agg[blockIdx.x] = r;
}

template <typename T, typename Op>
__global__ void __launch_bounds__(1024) k_agg_scan(T *agg, uint32_t m, Op op)
{
    __shared__ T sm[32];
    __shared__ T s_carry;
    if (threadIdx.x == 0) s_carry = op.ident();
    __syncthreads();
    for (uint32_t b = 0; b < m; b += blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const T inc = block_incl_scan<T>(i < m ? agg[i] : op.ident(), sm, op);
        const T v = op(s_carry, inc);
        if (i < m) agg[i] = v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry = v;
        __syncthreads();
    }
}

template <typename T, typename Op>
__global__ void __launch_bounds__(256) k_tile_scan(const T *in, T *out, uint64_t n,   // in may be out
                                                   const T *__restrict__ agg_incl, Op op)
{
    __shared__ T sm[32];
    __shared__ T s_inc[256];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    T v[kScanItems];
    T x = op.ident();
    for (uint32_t j = 0; j < kScanItems; ++j) {
        v[j] = base + j < n ? in[base + j] : op.ident();
        x = op(x, v[j]);
    }
    const T inc = block_incl_scan<T>(x, sm, op);
    s_inc[threadIdx.x] = inc;
    __syncthreads();
    T run = blockIdx.x ? agg_incl[blockIdx.x - 1] : op.ident();
    if (threadIdx.x) run = op(run, s_inc[threadIdx.x - 1]);
    for (uint32_t j = 0; j < kScanItems; ++j) {
        run = op(run, v[j]);
        if (base + j < n) out[base + j] = run;
    }
}

template <typename T, typename Op>
cudaError_t device_incl_scan(const T *in, T *out, uint64_t n, T *agg, Op op, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    const uint32_t tiles = (uint32_t)((n + kScanTile - 1) / kScanTile);
    k_tile_reduce<T, Op><<<tiles, 256, 0, st>>>(in, n, agg, op);
    k_agg_scan<T, Op><<<1, 1024, 0, st>>>(agg, tiles, op);
    k_tile_scan<T, Op><<<tiles, 256, 0, st>>>(in, out, n, agg, op);
    return cudaGetLastError();
}

// ------------------------------------------------------------ token starts
__device__ __forceinline__ bool token_start(const uint8_t *__restrict__ B, uint32_t i)
{
    return !is_space(B[i]) && (i == 0 || is_space(B[i - 1]));
}

__global__ void __launch_bounds__(256) k_count_starts(const uint8_t *__restrict__ B, uint32_t n, uint32_t *cnt)
{
    __shared__ uint32_t sm[32];
    const uint32_t a = blockIdx.x * kTileBytes + threadIdx.x * kBytesPerThread;
    uint32_t c = 0;
    for (uint32_t i = a; i < min(n, a + kBytesPerThread); ++i) c += token_start(B, i);
    const uint32_t r = block_incl_scan<uint32_t>(c, sm, Sum());
    if (threadIdx.x == blockDim.x - 1) cnt[blockIdx.x] = r;
}

__global__ void __launch_bounds__(256) k_write_starts(const uint8_t *__restrict__ B, uint32_t n,
                                                      const uint32_t *__restrict__ tile_incl, uint32_t *tok)
{
    __shared__ uint32_t sm[32];
    const uint32_t a = blockIdx.x * kTileBytes + threadIdx.x * kBytesPerThread;
    uint32_t c = 0;
    for (uint32_t i = a; i < min(n, a + kBytesPerThread); ++i) c += token_start(B, i);
    const uint32_t inc = block_incl_scan<uint32_t>(c, sm, Sum());
    uint32_t at = (blockIdx.x ? tile_incl[blockIdx.x - 1] : 0u) + inc - c;
    for (uint32_t i = a; i < min(n, a + kBytesPerThread); ++i)
        if (token_start(B, i)) tok[at++] = i;
}

// ------------------------------------------------------------ classes
__device__ __forceinline__ uint32_t token_len(const uint8_t *__restrict__ B, uint32_t n, uint32_t p)
{
    uint32_t q = p;
    while (q < n && !is_space(B[q])) ++q;
    return q - p;
}

__device__ __forceinline__ bool same(const uint8_t *__restrict__ B, uint32_t p, uint32_t len, const char *lit,
                                     uint32_t ll)
{
    if (len != ll) return false;
    for (uint32_t j = 0; j < ll; ++j)
        if (B[p + j] != (uint8_t)lit[j]) return false;
    return true;
}

// per token: class and length; the scan inputs (x: $comment + 1, y: $end
// + 1, z: first b/r of a run + 1, w: time + 1; 0 where none) come later
__global__ void __launch_bounds__(256) k_classify(const uint8_t *__restrict__ B, uint32_t n,
                                                  const uint32_t *__restrict__ tok, uint32_t T, uint8_t *cls,
                                                  uint32_t *len)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
        const uint32_t p = tok[k];
        const uint32_t l = token_len(B, n, p);
        const uint8_t c = B[p];
        uint8_t t = kOther;
        if (c == '#') t = kTime;
        else if (c == '$') t = same(B, p, l, "$comment", 8) ? kOpen : (same(B, p, l, "$end", 4) ? kEnd : kKey);
        else if (c == 'b' || c == 'B') t = kVec;
        else if (c == 'r' || c == 'R') t = kReal;
        else if (value_code(c) != 255) t = kScalar;
        cls[k] = t;
        len[k] = l;
    }
}

// the first pass of the running maxima: comment openers and closers
__global__ void __launch_bounds__(256) k_marks1(const uint8_t *__restrict__ cls, uint32_t T, uint4 *mk)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x)
        mk[k] = make_uint4(cls[k] == kOpen ? k + 1 : 0u, cls[k] == kEnd ? k + 1 : 0u, 0u, 0u);
}

// inside a comment: the latest opener at or before k after the latest
// closer before k
__device__ __forceinline__ bool inside(const uint4 *__restrict__ m1, uint32_t k)
{
    const uint32_t open = m1[k].x, end_before = k ? m1[k - 1].y : 0u;
    return open > end_before;
}

// the second pass: runs of b/r tokens outside comments, and times
__global__ void __launch_bounds__(256) k_marks2(const uint8_t *__restrict__ cls, uint32_t T,
                                                const uint4 *__restrict__ m1, uint4 *mk)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
        const bool cand = !inside(m1, k) && (cls[k] == kVec || cls[k] == kReal);
        const bool prev = k > 0 && !inside(m1, k - 1) && (cls[k - 1] == kVec || cls[k - 1] == kReal);
        mk[k] = make_uint4(0u, 0u, cand && !prev ? k + 1 : 0u, 0u);
    }
}

__device__ __forceinline__ bool candidate(const uint8_t *__restrict__ cls, const uint4 *__restrict__ m1, uint32_t k)
{
    return !inside(m1, k) && (cls[k] == kVec || cls[k] == kReal);
}

// token k is the identifier code of the b/r token before it
__device__ __forceinline__ bool consumed(const uint8_t *__restrict__ cls, const uint4 *__restrict__ m1,
                                         const uint4 *__restrict__ m2, uint32_t k)
{
    if (k == 0 || !candidate(cls, m1, k - 1)) return false;
    const uint32_t s = m2[k - 1].z - 1;   // the run's first b/r token
    return ((k - 1 - s) & 1u) == 0;
}

__device__ __forceinline__ bool acting(const uint8_t *__restrict__ cls, const uint4 *__restrict__ m1,
                                       const uint4 *__restrict__ m2, uint32_t k)
{
    return !inside(m1, k) && !consumed(cls, m1, m2, k);
}

// the third pass: times in force; and the tokens the host reader would
// read differently (a keyword taken as an identifier code)
__global__ void __launch_bounds__(256) k_marks3(const uint8_t *__restrict__ cls, uint32_t T,
                                                const uint4 *__restrict__ m1, const uint4 *__restrict__ m2,
                                                uint4 *mk, uint32_t *fallback)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
        const bool t = cls[k] == kTime && acting(cls, m1, m2, k);
        mk[k] = make_uint4(0u, 0u, 0u, t ? k + 1 : 0u);
        if ((cls[k] == kOpen || cls[k] == kEnd) && consumed(cls, m1, m2, k)) *fallback = 1;
    }
}

// identifier code of up to 8 bytes as a little-endian key (0: longer or empty)
__device__ __forceinline__ uint64_t code_key(const uint8_t *__restrict__ B, uint32_t p, uint32_t l)
{
    if (l == 0 || l > 8) return 0;
    uint64_t k = 0;
    for (uint32_t j = 0; j < l; ++j) k |= (uint64_t)B[p + j] << (8 * j);
    return k;
}

__device__ __forceinline__ int64_t find_code(const uint64_t *__restrict__ keys, uint32_t n_ids, uint64_t key)
{
    if (!key) return -1;
    uint32_t lo = 0, hi = n_ids;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (keys[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo < n_ids && keys[lo] == key ? (int64_t)lo : -1;
}

struct Ids {
    const uint64_t *key;
    const uint32_t *var_start, *bit_start, *bits;
    const uint8_t *bus;
    uint32_t n_ids;
};

// the code a change token names: scalar: its own text after the value;
// vector: the next token
__device__ __forceinline__ int64_t token_code(const uint8_t *__restrict__ B, const uint32_t *__restrict__ tok,
                                              const uint32_t *__restrict__ len, uint32_t T, uint8_t c, uint32_t k,
                                              const Ids &ids)
{
    if (c == kScalar) return find_code(ids.key, ids.n_ids, code_key(B, tok[k] + 1, len[k] - 1));
    if (c == kVec && k + 1 < T) return find_code(ids.key, ids.n_ids, code_key(B, tok[k + 1], len[k + 1]));
    return -1;
}

__global__ void __launch_bounds__(256) k_count_bits(const uint8_t *__restrict__ B, const uint32_t *__restrict__ tok,
                                                    const uint32_t *__restrict__ len, const uint8_t *__restrict__ cls,
                                                    uint32_t T, const uint4 *__restrict__ m1,
                                                    const uint4 *__restrict__ m2, Ids ids, unsigned long long *cnt)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
        unsigned long long c = 0;
        const uint8_t t = cls[k];
        if ((t == kScalar || t == kVec) && acting(cls, m1, m2, k)) {
            const int64_t id = token_code(B, tok, len, T, t, k, ids);
            if (id >= 0) c = ids.bit_start[ids.var_start[id + 1]] - ids.bit_start[ids.var_start[id]];
        }
        cnt[k] = c;
    }
}

__device__ __forceinline__ uint64_t parse_time(const uint8_t *__restrict__ B, uint32_t p, uint32_t l)
{
    uint64_t t = 0;
    for (uint32_t j = 1; j < l; ++j) {
        const uint8_t d = B[p + j];
        if (d < '0' || d > '9') break;
        t = t * 10 + (d - '0');
    }
    return t;
}

__global__ void __launch_bounds__(256) k_emit(const uint8_t *__restrict__ B, const uint32_t *__restrict__ tok,
                                              const uint32_t *__restrict__ len, const uint8_t *__restrict__ cls,
                                              uint32_t T, const uint4 *__restrict__ m3, Ids ids,
                                              const unsigned long long *__restrict__ cnt,
                                              const unsigned long long *__restrict__ at_incl,
                                              uint32_t *o_sig, unsigned long long *o_time, uint8_t *o_val,
                                              uint8_t *o_bus)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
        if (!cnt[k]) continue;
        const uint8_t t = cls[k];
        const int64_t id = token_code(B, tok, len, T, t, k, ids);
        if (id < 0) continue;   // cnt > 0 implies a code
        const uint32_t tt = m3[k].w;
        const uint64_t now = tt ? parse_time(B, tok[tt - 1], len[tt - 1]) : 0ull;
        unsigned long long at = at_incl[k] - cnt[k];
        const uint32_t p = tok[k], L = len[k] - 1;   // vector digits after the b
        const uint8_t c0 = B[p];
        for (uint32_t v = ids.var_start[id]; v < ids.var_start[id + 1]; ++v) {
            const uint32_t b0 = ids.bit_start[v], w = ids.bit_start[v + 1] - b0;
            const uint8_t bus = ids.bus[v];
            for (uint32_t b = 0; b < w; ++b) {
                uint8_t ch = c0;
                if (t == kVec) {
                    if (L < w) {
                        // short values extend on the left: x and z with themselves, else 0
                        const uint8_t f = L ? B[p + 1] : (uint8_t)'0';
                        const uint8_t pad = (f == 'x' || f == 'X') ? 'x' : (f == 'z' || f == 'Z') ? 'z' : '0';
                        ch = b < w - L ? pad : B[p + 1 + (b - (w - L))];
                    } else {
                        ch = B[p + 1 + (L - w) + b];
                    }
                }
                o_sig[at] = ids.bits[b0 + b];
                o_time[at] = now;
                o_val[at] = value_code(ch);
                o_bus[at] = bus;
                ++at;
            }
        }
    }
}

struct Dev {
    void *p = nullptr;
    ~Dev() { if (p) cudaFree(p); }
    bool alloc(size_t n) { return cudaMalloc(&p, n ? n : 16) == cudaSuccess; }
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

}  // namespace

extern "C" int gls_vcd_scan(int device, const char *body, uint64_t n_bytes, const gls_vcd_ids *ids,
                            gls_vcd_changes *out)
{
    if (!out || !ids || (n_bytes && !body)) return GLS_EINVAL;
    std::memset(out, 0, sizeof *out);
    if (n_bytes >= 0xFFFF0000ull) return GLS_ERANGE;   // positions (and a tile's end) stay 32-bit
    if (n_bytes == 0) return GLS_OK;
    const uint32_t n = (uint32_t)n_bytes;
    const uint32_t n_vars = ids->var_start[ids->n_ids];
    const uint32_t n_bits = ids->bit_start[n_vars];
    if (ids->var_start[0] != 0 || ids->bit_start[0] != 0) return GLS_EINVAL;
    for (uint32_t i = 0; i < ids->n_ids; ++i)
        if (ids->var_start[i + 1] < ids->var_start[i] || (i && ids->key[i] <= ids->key[i - 1]) || !ids->key[i])
            return GLS_EINVAL;
    for (uint32_t v = 0; v < n_vars; ++v)
        if (ids->bit_start[v + 1] < ids->bit_start[v]) return GLS_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return GLS_ECUDA;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return GLS_ECUDA;
    int rc = GLS_OK;
    Dev dB, dTileCnt, dTileAgg, dTok, dLen, dCls, dM1, dM2, dM3, dAgg4, dCnt, dAt, dAgg1, dKey, dVs, dBs, dBits, dBus,
        dFlag, dSig, dTime, dVal, dBusOut;
    do {
        const uint32_t tiles = (n + kTileBytes - 1) / kTileBytes;
        if (!dB.alloc(n) || !dTileCnt.alloc((size_t)tiles * 4) || !dTileAgg.alloc((size_t)tiles * 4) ||
            !dFlag.alloc(16) || !dKey.alloc((size_t)ids->n_ids * 8) || !dVs.alloc((size_t)(ids->n_ids + 1) * 4) ||
            !dBs.alloc((size_t)(n_vars + 1) * 4) || !dBits.alloc((size_t)n_bits * 4) || !dBus.alloc(n_vars)) {
            rc = GLS_ENOMEM;
            break;
        }
        if (cudaMemcpyAsync(dB.p, body, n, cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(dKey.p, ids->key, (size_t)ids->n_ids * 8, cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(dVs.p, ids->var_start, (size_t)(ids->n_ids + 1) * 4, cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(dBs.p, ids->bit_start, (size_t)(n_vars + 1) * 4, cudaMemcpyHostToDevice, st) ||
            (n_bits && cudaMemcpyAsync(dBits.p, ids->bits, (size_t)n_bits * 4, cudaMemcpyHostToDevice, st)) ||
            (n_vars && cudaMemcpyAsync(dBus.p, ids->bus, n_vars, cudaMemcpyHostToDevice, st)) ||
            cudaMemsetAsync(dFlag.p, 0, 16, st)) {
            rc = GLS_ECUDA;
            break;
        }
        const uint8_t *B = dB.as<uint8_t>();
        k_count_starts<<<tiles, 256, 0, st>>>(B, n, dTileCnt.as<uint32_t>());
        if (device_incl_scan<uint32_t>(dTileCnt.as<uint32_t>(), dTileCnt.as<uint32_t>(), tiles,
                                       dTileAgg.as<uint32_t>(), Sum(), st)) {
            rc = GLS_ECUDA;
            break;
        }
        uint32_t T = 0;
        if (cudaMemcpyAsync(&T, dTileCnt.as<uint32_t>() + tiles - 1, 4, cudaMemcpyDeviceToHost, st) ||
            cudaStreamSynchronize(st)) {
            rc = GLS_ECUDA;
            break;
        }
        if (T == 0) break;
        const uint32_t T_tiles = (T + kScanTile - 1) / kScanTile;
        if (!dTok.alloc((size_t)T * 4) || !dLen.alloc((size_t)T * 4) || !dCls.alloc(T) ||
            !dM1.alloc((size_t)T * 16) || !dM2.alloc((size_t)T * 16) || !dM3.alloc((size_t)T * 16) ||
            !dAgg4.alloc((size_t)T_tiles * 16) || !dCnt.alloc((size_t)T * 8) || !dAt.alloc((size_t)T * 8) ||
            !dAgg1.alloc((size_t)T_tiles * 8)) {
            rc = GLS_ENOMEM;
            break;
        }
        k_write_starts<<<tiles, 256, 0, st>>>(B, n, dTileCnt.as<uint32_t>(), dTok.as<uint32_t>());
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        const uint32_t grid = (uint32_t)std::max(1, sms) * 8;
        k_classify<<<grid, 256, 0, st>>>(B, n, dTok.as<uint32_t>(), T, dCls.as<uint8_t>(), dLen.as<uint32_t>());
        k_marks1<<<grid, 256, 0, st>>>(dCls.as<uint8_t>(), T, dM1.as<uint4>());
        if (device_incl_scan<uint4>(dM1.as<uint4>(), dM1.as<uint4>(), T, dAgg4.as<uint4>(), Max4(), st)) {
            rc = GLS_ECUDA;
            break;
        }
        k_marks2<<<grid, 256, 0, st>>>(dCls.as<uint8_t>(), T, dM1.as<uint4>(), dM2.as<uint4>());
        if (device_incl_scan<uint4>(dM2.as<uint4>(), dM2.as<uint4>(), T, dAgg4.as<uint4>(), Max4(), st)) {
            rc = GLS_ECUDA;
            break;
        }
        k_marks3<<<grid, 256, 0, st>>>(dCls.as<uint8_t>(), T, dM1.as<uint4>(), dM2.as<uint4>(), dM3.as<uint4>(),
                                       dFlag.as<uint32_t>());
        if (device_incl_scan<uint4>(dM3.as<uint4>(), dM3.as<uint4>(), T, dAgg4.as<uint4>(), Max4(), st)) {
            rc = GLS_ECUDA;
            break;
        }
        Ids di{dKey.as<uint64_t>(), dVs.as<uint32_t>(), dBs.as<uint32_t>(), dBits.as<uint32_t>(), dBus.as<uint8_t>(),
               ids->n_ids};
        k_count_bits<<<grid, 256, 0, st>>>(B, dTok.as<uint32_t>(), dLen.as<uint32_t>(), dCls.as<uint8_t>(), T,
                                           dM1.as<uint4>(), dM2.as<uint4>(), di, dCnt.as<unsigned long long>());
        if (device_incl_scan<unsigned long long>(dCnt.as<unsigned long long>(), dAt.as<unsigned long long>(), T,
                                                 dAgg1.as<unsigned long long>(), Sum64(), st)) {
            rc = GLS_ECUDA;
            break;
        }
        uint32_t flag = 0;
        unsigned long long total = 0;
        if (cudaMemcpyAsync(&flag, dFlag.p, 4, cudaMemcpyDeviceToHost, st) ||
            cudaMemcpyAsync(&total, dAt.as<unsigned long long>() + T - 1, 8, cudaMemcpyDeviceToHost, st) ||
            cudaStreamSynchronize(st)) {
            rc = GLS_ECUDA;
            break;
        }
        if (flag) {
            out->fallback = 1;
            break;
        }
        if (total == 0) break;
        if (!dSig.alloc((size_t)total * 4) || !dTime.alloc((size_t)total * 8) || !dVal.alloc(total) ||
            !dBusOut.alloc(total)) {
            rc = GLS_ENOMEM;
            break;
        }
        k_emit<<<grid, 256, 0, st>>>(B, dTok.as<uint32_t>(), dLen.as<uint32_t>(), dCls.as<uint8_t>(), T,
                                     dM3.as<uint4>(), di, dCnt.as<unsigned long long>(), dAt.as<unsigned long long>(),
                                     dSig.as<uint32_t>(),
                                     dTime.as<unsigned long long>(), dVal.as<uint8_t>(), dBusOut.as<uint8_t>());
        out->signal = static_cast<uint32_t *>(std::malloc((size_t)total * 4));
        out->time = static_cast<uint64_t *>(std::malloc((size_t)total * 8));
        out->value = static_cast<uint8_t *>(std::malloc(total));
        out->bus = static_cast<uint8_t *>(std::malloc(total));
        if (!out->signal || !out->time || !out->value || !out->bus) {
            rc = GLS_ENOMEM;
            break;
        }
        if (cudaMemcpyAsync(out->signal, dSig.p, (size_t)total * 4, cudaMemcpyDeviceToHost, st) ||
            cudaMemcpyAsync(out->time, dTime.p, (size_t)total * 8, cudaMemcpyDeviceToHost, st) ||
            cudaMemcpyAsync(out->value, dVal.p, total, cudaMemcpyDeviceToHost, st) ||
            cudaMemcpyAsync(out->bus, dBusOut.p, total, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st)) {
            rc = GLS_ECUDA;
            break;
        }
        out->n = total;
    } while (false);
    cudaStreamDestroy(st);
    if (rc) gls_vcd_free(out);
    return rc;
}

extern "C" void gls_vcd_free(gls_vcd_changes *out)
{
    if (!out) return;
    std::free(out->signal);
    std::free(out->time);
    std::free(out->value);
    std::free(out->bus);
    out->signal = nullptr;
    out->time = nullptr;
    out->value = nullptr;
    out->bus = nullptr;
    out->n = 0;
}
