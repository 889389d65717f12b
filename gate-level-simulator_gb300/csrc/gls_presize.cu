// Learned presize: per-gate features, MLP inference on the tensor cores
// (tcgen05, BF16 operands, FP32 accumulation in tensor memory) with an FP32
// CUDA-core twin, and FP32 training kernels (GEMM, Huber loss, Adam).
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include "gls_presize.h"

namespace gls {

// ------------------------------------------------------------- features
// Row of a gate output: its static features (cell, pins, delays, fan-out,
// truth-table sensitivity) with the input-net entries filled from the
// lengths of its input nets' change lists.
__device__ __forceinline__ void gate_features(const PresizeArgs &a, uint32_t r, float x[kIn])
{
    if (a.rows) {
#pragma unroll
        for (int k = 0; k < kIn; ++k) x[k] = a.rows[(uint64_t)r * kIn + k];
        return;
    }
    const uint32_t d = a.lo + r;
    const float4 *fs = reinterpret_cast<const float4 *>(a.feat_static + (uint64_t)d * kIn);
#pragma unroll
    for (int q = 0; q < kIn / 4; ++q) {
        const float4 v = __ldg(fs + q);
        x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
    }
    const DrvMeta &md = a.meta[d];
    float sum = 0.f, mx = 0.f, mn = 0.f, len[kMaxSlots], p1[kMaxSlots];
#pragma unroll
    for (int j = 0; j < kMaxSlots; ++j) {
        float l = 0.f, q = 0.5f;
        if (j < md.m) {
            const uint32_t net = md.net[j];
            const uint32_t n_ev = a.net_len[net];
            l = n_ev == 0xFFFFFFFFu ? 0.f : (float)n_ev;
            sum += l;
            mx = fmaxf(mx, l);
            mn = j == 0 ? l : fminf(mn, l);
            // share of the window the net spends at 1 (of its time at 0 or 1)
            const unsigned long long t0 = a.saif[3ull * net], t1 = a.saif[3ull * net + 1];
            if (t0 != ~0ull && t0 + t1 > 0) q = (float)((double)t1 / (double)(t0 + t1));
        }
        len[j] = l;
        p1[j] = q;
        if (j < 3) x[15 + j] = log1pf(l) * (1.f / 12.f);
    }
    x[18] = log1pf(sum) * (1.f / 12.f);
    x[19] = log1pf(mx) * (1.f / 12.f);
    x[20] = log1pf(mn) * (1.f / 12.f);
    // expected output changes with independent inputs: every input change
    // passes when the other inputs sensitize the output to it (the Boolean
    // difference of the truth table, weighted by their 1-probabilities)
    const uint8_t *lut = a.lut + md.lut_off;
    const int m = md.m;
    float est = 0.f, pone = 0.f, pmean = 0.f;
    for (uint32_t b = 0; b < (1u << m); ++b) {
        uint32_t idx = 0;
        for (int p = 0; p < md.n_pins; ++p)
            idx |= (((b >> ((md.pin_slot >> (3 * p)) & 7u)) & 1u) ? 3u : 0u) << (2 * p);
        const uint32_t F = __ldg(lut + idx);
        float w = 1.f;
        for (int j = 0; j < m; ++j) w *= ((b >> j) & 1u) ? p1[j] : 1.f - p1[j];
        if (F == kV1) pone += w;
        for (int j = 0; j < m; ++j) {
            if ((b >> j) & 1u) continue;
            uint32_t idx2 = 0;
            const uint32_t b2 = b | (1u << j);
            for (int p = 0; p < md.n_pins; ++p)
                idx2 |= (((b2 >> ((md.pin_slot >> (3 * p)) & 7u)) & 1u) ? 3u : 0u) << (2 * p);
            if (__ldg(lut + idx2) != F) {
                float wo = 1.f;   // probability of the other inputs' values
                for (int i = 0; i < m; ++i)
                    if (i != j) wo *= ((b >> i) & 1u) ? p1[i] : 1.f - p1[i];
                est += wo * len[j];
            }
        }
    }
    for (int j = 0; j < m; ++j) pmean += p1[j];
    x[21] = log1pf(est) * (1.f / 12.f);
    x[22] = pone;
    x[23] = m ? pmean / m : 0.f;
}

__device__ __forceinline__ uint32_t reserve_of(const PresizeArgs &a, float y)
{
    const float len = expm1f(fminf(fmaxf(y, 0.f), 30.f)) * (1.f + a.margin);
    const float r = ceilf(len) + (float)a.slack;
    return r >= 4.0e9f ? 0xFFFFFFF0u : (uint32_t)r;
}

// the window's own buffers when the rows are gate outputs of a batch of windows
__device__ __forceinline__ PresizeArgs for_window(const PresizeArgs &a)
{
    PresizeArgs b = a;
    if (a.wv) {
        const WinDev &w = a.wv[blockIdx.y];
        b.net_len = w.net_len;
        b.saif = w.saif;
        b.pred = w.pred;
        b.err = w.err;
    }
    return b;
}

__global__ void __launch_bounds__(256) k_features(PresizeArgs a, float *out)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.n) return;
    float x[kIn];
    gate_features(a, r, x);
#pragma unroll
    for (int k = 0; k < kIn; ++k) out[(uint64_t)r * kIn + k] = x[k];
}

// ------------------------------------------------ FP32 CUDA-core inference
// One thread per row; the FP32 weights sit in shared memory.
__global__ void __launch_bounds__(128) k_presize_f32(PresizeArgs a0)
{
    const PresizeArgs a = for_window(a0);
    extern __shared__ float sp[];
    for (uint32_t k = threadIdx.x; k < (uint32_t)kParams; k += blockDim.x) sp[k] = a.params[k];
    __syncthreads();
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.n) return;
    float x[kIn], h1[kHid];
    gate_features(a, r, x);
#pragma unroll 4
    for (int u = 0; u < kHid; ++u) {
        float z = sp[kOffB1 + u];
#pragma unroll
        for (int k = 0; k < kIn; ++k) z = fmaf(sp[kOffW1 + u * kIn + k], x[k], z);
        h1[u] = fmaxf(z, 0.f);
    }
    float y = sp[kOffB3];
    for (int u = 0; u < kHid; ++u) {
        float z = sp[kOffB2 + u];
#pragma unroll
        for (int v = 0; v < kHid; ++v) z = fmaf(sp[kOffW2 + u * kHid + v], h1[v], z);
        y = fmaf(sp[kOffW3 + u], fmaxf(z, 0.f), y);
    }
    if (a.y) a.y[r] = y;
    if (a.pred) a.pred[r] = reserve_of(a, y);
}

// -------------------------------------------------- tcgen05 inference
// One CTA of 128 threads per 128 rows: thread t builds row t's features and
// owns row t of both accumulators.  Layer 1 (128 x 32 by 32 x 128) and
// layer 2 (128 x 128 by 128 x 128) are tcgen05.mma kind::f16 with BF16
// operands in shared memory and the FP32 accumulator in tensor memory
// (128 lanes x 128 columns); the 128 -> 1 output layer runs on the CUDA
// cores from the tcgen05.ld of layer 2.
constexpr uint32_t kSmA1 = 0, kSmB1 = 8192, kSmB2 = kSmB1 + kImgW2, kSmA2 = kSmB1 + kImgBytes,
                   kSmBar = kSmA2 + kHid * kHid * 2, kSmTotal = kSmBar + 64;
static_assert(kSmB2 == 16384 && kSmA2 == 49152, "tensor-core kernel shared-memory map");
// instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kHid >> 3) << 17) | ((128u >> 4) << 24);
constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kWaitSpins = 1u << 20;

// shared-memory matrix descriptor: start address, leading (K-direction) and
// stride (8-row-group) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(tmem), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// bounded wait on an mbarrier phase: false after kWaitSpins polls
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (uint32_t it = 0; it < kWaitSpins; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__global__ void __launch_bounds__(128, 1) k_presize_tc(PresizeArgs a0)
{
    const PresizeArgs a = for_window(a0);
    extern __shared__ __align__(1024) uint8_t sm[];
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
    const uint32_t bar = sbase + kSmBar, tslot = sbase + kSmBar + 8;
    // weights: the prepared BF16 image goes to B1 | B2 unchanged
    {
        uint4 *dst = reinterpret_cast<uint4 *>(sm + kSmB1);
        for (uint32_t k = tid; k < kImgBytes / 16; k += 128) dst[k] = __ldg(a.img + k);
    }
    if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tslot), "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // A1: this thread's feature row in BF16, 16 bytes per 8 features
    const uint32_t r = blockIdx.x * 128 + tid;
    {
        float x[kIn];
        if (r < a.n) gate_features(a, r, x);
        else {
#pragma unroll
            for (int k = 0; k < kIn; ++k) x[k] = 0.f;
        }
#pragma unroll
        for (int k8 = 0; k8 < kIn / 8; ++k8) {
            uint4 q;
            q.x = pack_bf16(x[8 * k8 + 0], x[8 * k8 + 1]);
            q.y = pack_bf16(x[8 * k8 + 2], x[8 * k8 + 3]);
            q.z = pack_bf16(x[8 * k8 + 4], x[8 * k8 + 5]);
            q.w = pack_bf16(x[8 * k8 + 6], x[8 * k8 + 7]);
            *reinterpret_cast<uint4 *>(sm + kSmA1 + canon_off(tid, 8 * k8, kIn)) = q;
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(sm + kSmBar + 8);
    const uint32_t trow = tmem + ((warp * 32u) << 16);   // this warp's 32 lanes
    // layer 1: K = 32 in two K-steps of 16
    if (tid == 0) {
#pragma unroll
        for (uint32_t ks = 0; ks < kIn / 16; ++ks)
            mma_bf16(tmem, smem_desc(sbase + kSmA1 + ks * 256, 128, (kIn / 8) * 128),
                     smem_desc(sbase + kSmB1 + ks * 256, 128, (kIn / 8) * 128), ks);
        mma_commit(bar);
    }
    bool ok = __syncthreads_and(mbar_wait(bar, 0));
    fence_after();
    if (ok) {
        // hidden layer 1 = ReLU(acc + b1) -> A2 in BF16
#pragma unroll 1
        for (uint32_t c = 0; c < kHid / 32; ++c) {
            float v[32];
            tmem_ld32(trow + c * 32, v);
#pragma unroll
            for (int j8 = 0; j8 < 4; ++j8) {
                float h[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int col = c * 32 + j8 * 8 + j;
                    h[j] = fmaxf(v[j8 * 8 + j] + __ldg(a.params + kOffB1 + col), 0.f);
                }
                uint4 q;
                q.x = pack_bf16(h[0], h[1]);
                q.y = pack_bf16(h[2], h[3]);
                q.z = pack_bf16(h[4], h[5]);
                q.w = pack_bf16(h[6], h[7]);
                *reinterpret_cast<uint4 *>(sm + kSmA2 + canon_off(tid, c * 32 + j8 * 8, kHid)) = q;
            }
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    // layer 2: K = 128 in eight K-steps, accumulator columns reused
    if (ok && tid == 0) {
#pragma unroll
        for (uint32_t ks = 0; ks < kHid / 16; ++ks)
            mma_bf16(tmem, smem_desc(sbase + kSmA2 + ks * 256, 128, (kHid / 8) * 128),
                     smem_desc(sbase + kSmB2 + ks * 256, 128, (kHid / 8) * 128), ks);
        mma_commit(bar);
    }
    if (ok) ok = __syncthreads_and(mbar_wait(bar, 1));
    fence_after();
    if (ok) {
        float y = __ldg(a.params + kOffB3);
#pragma unroll 1
        for (uint32_t c = 0; c < kHid / 32; ++c) {
            float v[32];
            tmem_ld32(trow + c * 32, v);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int col = c * 32 + j;
                y = fmaf(__ldg(a.params + kOffW3 + col), fmaxf(v[j] + __ldg(a.params + kOffB2 + col), 0.f), y);
            }
        }
        if (r < a.n) {
            if (a.y) a.y[r] = y;
            if (a.pred) a.pred[r] = reserve_of(a, y);
        }
    } else if (tid == 0) {
        atomicOr(a.err, 1u);
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

void launch_features(const PresizeArgs &a, float *out, cudaStream_t st)
{
    if (!a.n) return;
    k_features<<<(a.n + 255) / 256, 256, 0, st>>>(a, out);
}

// the dynamic shared-memory limits of both inference kernels (the current
// device; called before any launch and outside stream capture)
void prepare_presize_kernels()
{
    cudaFuncSetAttribute(k_presize_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmTotal);
    cudaFuncSetAttribute(k_presize_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kParams * 4));
}

void launch_presize(const PresizeArgs &a, bool tensor_cores, cudaStream_t st)
{
    if (!a.n) return;
    const dim3 grid((a.n + 127) / 128, a.wv ? a.nwin : 1);
    if (tensor_cores) k_presize_tc<<<grid, 128, kSmTotal, st>>>(a);
    else k_presize_f32<<<grid, 128, kParams * 4, st>>>(a);
}

// ------------------------------------------------------------- training
// C(i, j) = sum_k A(i, k) B(k, j) with A(i, k) = A[i * as0 + k * as1],
// B(k, j) = B[k * bs0 + j * bs1] and row stride cs for C.  64 x 64 tiles,
// 256 threads with 4 x 4 outputs each.  With several K splits
// (gridDim.z) the partial sums are added into C with atomics (C cleared
// first).  Epilogues: kEpiStore; kEpiBiasRelu stores z = acc + bias[j] in C
// and max(z, 0) in C2; kEpiMask stores acc where mask(i, j) > 0, else 0.
constexpr int kEpiStore = 0, kEpiBiasRelu = 1, kEpiMask = 2;

template <int EPI>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, int kchunk, const float *__restrict__ A, long as0,
                                              long as1, const float *__restrict__ B, long bs0, long bs1,
                                              float *__restrict__ C, long cs, const float *__restrict__ bias,
                                              const float *__restrict__ mask, float *__restrict__ C2)
{
    __shared__ float As[16][65], Bs[16][65];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
    const int k0 = blockIdx.z * kchunk, k1 = min(K, k0 + kchunk);
    float acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = 0.f;
    for (int kb = k0; kb < k1; kb += 16) {
        for (int q = threadIdx.x; q < 1024; q += 256) {
            const int ii = q >> 4, kk = q & 15, gi = i0 + ii, gk = kb + kk;
            As[kk][ii] = (gi < M && gk < k1) ? A[(long)gi * as0 + (long)gk * as1] : 0.f;
        }
        for (int q = threadIdx.x; q < 1024; q += 256) {
            const int kk = q >> 6, jj = q & 63, gk = kb + kk, gj = j0 + jj;
            Bs[kk][jj] = (gk < k1 && gj < N) ? B[(long)gk * bs0 + (long)gj * bs1] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float av[4], bv[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) av[r] = As[kk][ty * 4 + r];
#pragma unroll
            for (int c = 0; c < 4; ++c) bv[c] = Bs[kk][tx * 4 + c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(av[r], bv[c], acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int gi = i0 + ty * 4 + r;
        if (gi >= M) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int gj = j0 + tx * 4 + c;
            if (gj >= N) continue;
            float *dst = C + (long)gi * cs + gj;
            if (EPI == kEpiStore) {
                if (gridDim.z > 1) atomicAdd(dst, acc[r][c]);
                else *dst = acc[r][c];
            } else if (EPI == kEpiBiasRelu) {
                const float z = acc[r][c] + bias[gj];
                *dst = z;
                C2[(long)gi * cs + gj] = fmaxf(z, 0.f);
            } else {
                *dst = mask[(long)gi * cs + gj] > 0.f ? acc[r][c] : 0.f;
            }
        }
    }
}

// y[i] = b + sum_j H[i][j] w[j] (one warp per row)
__global__ void __launch_bounds__(256) k_rowdot(int n, const float *__restrict__ H, const float *__restrict__ w,
                                                const float *__restrict__ b, float *__restrict__ y)
{
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= n) return;
    float s = 0.f;
    for (int j = lane; j < kHid; j += 32) s = fmaf(H[(long)row * kHid + j], w[j], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[row] = s + b[0];
}

// Huber loss on r = y - t: dy = scale * dloss/dy; the loss sum is added to *sum
__global__ void __launch_bounds__(256) k_loss(int n, const float *__restrict__ y, const float *__restrict__ t,
                                              float huber, float scale, float *__restrict__ dy, float *sum)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const float r = y[i] - t[i], ab = fabsf(r);
        const bool in = ab <= huber;
        l = in ? 0.5f * r * r : huber * (ab - 0.5f * huber);
        dy[i] = scale * (in ? r : copysignf(huber, r));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    __shared__ float ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += ws[k];
        atomicAdd(sum, s);
    }
}

// dZ2[i][j] = dy[i] w3[j] where Z2[i][j] > 0, else 0
__global__ void __launch_bounds__(256) k_dz2(int n, const float *__restrict__ dy, const float *__restrict__ w3,
                                             const float *__restrict__ Z2, float *__restrict__ dZ2)
{
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long)n * kHid) return;
    const int i = (int)(q / kHid), j = (int)(q % kHid);
    dZ2[q] = Z2[q] > 0.f ? dy[i] * w3[j] : 0.f;
}

// out[j] += sum_i D[i][j] (wt ? wt[i] : 1) over a block's rows
__global__ void __launch_bounds__(256) k_colsum(int n, int N, const float *__restrict__ D,
                                                const float *__restrict__ wt, float *__restrict__ out)
{
    const int j = threadIdx.x % N, rows_per = blockDim.x / N, sub = threadIdx.x / N;
    if (sub >= rows_per) return;
    const int chunk = (n + gridDim.x - 1) / gridDim.x, i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    float s = 0.f;
    for (int i = i0 + sub; i < i1; i += rows_per) s += D[(long)i * N + j] * (wt ? wt[i] : 1.f);
    atomicAdd(out + j, s);
}

__global__ void __launch_bounds__(256) k_adam(int P, float *__restrict__ p, const float *__restrict__ g,
                                              float *__restrict__ m, float *__restrict__ v, float lr, float c1,
                                              float c2)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    const float gk = g[k];
    const float mk = 0.9f * m[k] + 0.1f * gk, vk = 0.999f * v[k] + 0.001f * gk * gk;
    m[k] = mk;
    v[k] = vk;
    p[k] -= lr * (mk * c1) / (sqrtf(vk * c2) + 1e-8f);
}

// batch row i = data row (mul * (base + i) + add) mod n (a permutation when gcd(mul, n) = 1)
__global__ void __launch_bounds__(256) k_gather(int nb, uint64_t base, uint64_t mul, uint64_t add, uint64_t n,
                                                const float *__restrict__ X, const float *__restrict__ T,
                                                float *__restrict__ Xb, float *__restrict__ Tb)
{
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long)nb * kIn) return;
    const int i = (int)(q / kIn), k = (int)(q % kIn);
    const uint64_t src = (uint64_t)(((unsigned __int128)mul * (base + i) + add) % n);
    Xb[q] = X[src * kIn + k];
    if (k == 0) Tb[i] = T[src];
}

}  // namespace gls

// =============================================================== host side
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "gls_ctx.h"

using namespace gls;

namespace {

// round-to-nearest-even float -> bfloat16 bits
uint16_t to_bf16(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7FFFFFFFu) > 0x7F800000u) return 0x7FC0;
    return (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
}

// the BF16 weight image the tensor-core kernel copies to shared memory
std::vector<uint8_t> weight_image(const float *params)
{
    std::vector<uint8_t> img(kImgBytes, 0);
    for (uint32_t n = 0; n < (uint32_t)kHid; ++n) {
        for (uint32_t k = 0; k < (uint32_t)kIn; ++k) {
            const uint16_t b = to_bf16(params[kOffW1 + n * kIn + k]);
            std::memcpy(&img[kImgW1 + canon_off(n, k, kIn)], &b, 2);
        }
        for (uint32_t k = 0; k < (uint32_t)kHid; ++k) {
            const uint16_t b = to_bf16(params[kOffW2 + n * kHid + k]);
            std::memcpy(&img[kImgW2 + canon_off(n, k, kHid)], &b, 2);
        }
    }
    return img;
}

int setf(std::string *err, int code, const char *msg, cudaError_t e = cudaSuccess)
{
    if (err) *err = e == cudaSuccess ? std::string(msg) : std::string(msg) + ": " + cudaGetErrorString(e);
    return code;
}

}  // namespace

// ------------------------------------------------------------- trainer
struct gls_trainer {
    int device = 0;
    cudaStream_t st = nullptr;
    std::string err;
    uint64_t n = 0, seed = 0, adam_t = 0;
    uint32_t cap_batch = 0;
    DevBuf X, T, Xb, Tb, Z1, H1, Z2, H2, Y, DY, DZ2, DZ1, P, G, Mo, Vo, loss;
};

namespace {

int tr_alloc_batch(gls_trainer *tr, uint32_t nb)
{
    if (nb <= tr->cap_batch) return GLS_OK;
    const size_t h = (size_t)nb * kHid * 4;
    cudaError_t e = cudaSuccess;
    DevBuf *hb[] = {&tr->Z1, &tr->H1, &tr->Z2, &tr->H2, &tr->DZ2, &tr->DZ1};
    for (DevBuf *b : hb)
        if (e == cudaSuccess) e = b->ensure(h);
    if (e == cudaSuccess) e = tr->Xb.ensure((size_t)nb * kIn * 4);
    if (e == cudaSuccess) e = tr->Tb.ensure((size_t)nb * 4);
    if (e == cudaSuccess) e = tr->Y.ensure((size_t)nb * 4);
    if (e == cudaSuccess) e = tr->DY.ensure((size_t)nb * 4);
    if (e != cudaSuccess) return setf(&tr->err, GLS_ENOMEM, "trainer batch buffers", e);
    tr->cap_batch = nb;
    return GLS_OK;
}

template <int EPI>
void gemm(cudaStream_t st, int M, int N, int K, const float *A, long as0, long as1, const float *B, long bs0, long bs1,
          float *C, long cs, const float *bias = nullptr, const float *mask = nullptr, float *C2 = nullptr)
{
    int splits = 1;
    if (EPI == kEpiStore) splits = std::max(1, std::min(64, K / 512));   // split-K sums land by atomics in cleared C
    const int kchunk = ((K + splits - 1) / splits + 15) / 16 * 16;
    splits = (K + kchunk - 1) / kchunk;
    dim3 grid((N + 63) / 64, (M + 63) / 64, splits);
    k_gemm<EPI><<<grid, 256, 0, st>>>(M, N, K, kchunk, A, as0, as1, B, bs0, bs1, C, cs, bias, mask, C2);
}

// forward and backward over rows Xb/Tb (nb); gradients into G (cleared here), loss sum into loss[0]
void tr_step_grad(gls_trainer *tr, int nb, float huber)
{
    cudaStream_t st = tr->st;
    float *P = tr->P.as<float>(), *G = tr->G.as<float>();
    const float *Xb = tr->Xb.as<float>(), *Tb = tr->Tb.as<float>();
    float *Z1 = tr->Z1.as<float>(), *H1 = tr->H1.as<float>(), *Z2 = tr->Z2.as<float>(), *H2 = tr->H2.as<float>();
    float *Y = tr->Y.as<float>(), *DY = tr->DY.as<float>(), *DZ2 = tr->DZ2.as<float>(), *DZ1 = tr->DZ1.as<float>();
    cudaMemsetAsync(G, 0, (size_t)kParams * 4, st);
    gemm<kEpiBiasRelu>(st, nb, kHid, kIn, Xb, kIn, 1, P + kOffW1, 1, kIn, Z1, kHid, P + kOffB1, nullptr, H1);
    gemm<kEpiBiasRelu>(st, nb, kHid, kHid, H1, kHid, 1, P + kOffW2, 1, kHid, Z2, kHid, P + kOffB2, nullptr, H2);
    k_rowdot<<<(nb * 32 + 255) / 256, 256, 0, st>>>(nb, H2, P + kOffW3, P + kOffB3, Y);
    k_loss<<<(nb + 255) / 256, 256, 0, st>>>(nb, Y, Tb, huber, 1.f / nb, DY, tr->loss.as<float>());
    const int cb = std::max(1, std::min(256, nb / 64));
    k_colsum<<<cb, 256, 0, st>>>(nb, kHid, H2, DY, G + kOffW3);
    k_colsum<<<cb, 256, 0, st>>>(nb, 1, DY, nullptr, G + kOffB3);
    k_dz2<<<(unsigned)(((long)nb * kHid + 255) / 256), 256, 0, st>>>(nb, DY, P + kOffW3, Z2, DZ2);
    gemm<kEpiStore>(st, kHid, kHid, nb, DZ2, 1, kHid, H1, kHid, 1, G + kOffW2, kHid);
    k_colsum<<<cb, 256, 0, st>>>(nb, kHid, DZ2, nullptr, G + kOffB2);
    gemm<kEpiMask>(st, nb, kHid, kHid, DZ2, kHid, 1, P + kOffW2, kHid, 1, DZ1, kHid, nullptr, Z1);
    gemm<kEpiStore>(st, kHid, kIn, nb, DZ1, 1, kHid, Xb, kIn, 1, G + kOffW1, kIn);
    k_colsum<<<cb, 256, 0, st>>>(nb, kHid, DZ1, nullptr, G + kOffB1);
}

uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t gcd64(uint64_t a, uint64_t b)
{
    while (b) {
        const uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

}  // namespace

extern "C" int gls_trainer_create(int device, uint64_t seed, gls_trainer **out)
{
    if (!out) return GLS_EINVAL;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return GLS_ECUDA;
    gls_trainer *tr = new gls_trainer;
    tr->device = device;
    tr->seed = seed;
    cudaError_t e = cudaStreamCreateWithFlags(&tr->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = tr->P.ensure(kParams * 4);
    if (e == cudaSuccess) e = tr->G.ensure(kParams * 4);
    if (e == cudaSuccess) e = tr->Mo.ensure(kParams * 4);
    if (e == cudaSuccess) e = tr->Vo.ensure(kParams * 4);
    if (e == cudaSuccess) e = tr->loss.ensure(16);
    if (e != cudaSuccess) {
        delete tr;
        return GLS_ECUDA;
    }
    // He-uniform initialization from the seed
    std::vector<float> p(kParams, 0.f);
    uint64_t s = seed;
    auto uni = [&](float lim) { return (float)(((splitmix(s) >> 11) * 0x1.0p-53) * 2.0 - 1.0) * lim; };
    for (int k = 0; k < kHid * kIn; ++k) p[kOffW1 + k] = uni(std::sqrt(6.f / kIn));
    for (int k = 0; k < kHid * kHid; ++k) p[kOffW2 + k] = uni(std::sqrt(6.f / kHid));
    for (int k = 0; k < kHid; ++k) p[kOffW3 + k] = uni(std::sqrt(6.f / kHid)) * 0.1f;
    cudaMemcpy(tr->P.p, p.data(), kParams * 4, cudaMemcpyHostToDevice);
    cudaMemset(tr->Mo.p, 0, kParams * 4);
    cudaMemset(tr->Vo.p, 0, kParams * 4);
    *out = tr;
    return GLS_OK;
}

extern "C" int gls_trainer_destroy(gls_trainer *tr)
{
    if (!tr) return GLS_OK;
    cudaSetDevice(tr->device);
    DevBuf *all[] = {&tr->X, &tr->T, &tr->Xb, &tr->Tb, &tr->Z1, &tr->H1, &tr->Z2, &tr->H2, &tr->Y,
                     &tr->DY, &tr->DZ2, &tr->DZ1, &tr->P, &tr->G, &tr->Mo, &tr->Vo, &tr->loss};
    for (DevBuf *b : all) b->release();
    if (tr->st) cudaStreamDestroy(tr->st);
    delete tr;
    return GLS_OK;
}

extern "C" const char *gls_trainer_error(const gls_trainer *tr) { return tr ? tr->err.c_str() : "null trainer"; }

extern "C" int gls_trainer_set_data(gls_trainer *tr, const float *feat, const float *target, uint64_t n)
{
    if (!tr || !feat || !target || !n) return GLS_EINVAL;
    cudaSetDevice(tr->device);
    cudaError_t e = tr->X.ensure(n * kIn * 4);
    if (e == cudaSuccess) e = tr->T.ensure(n * 4);
    if (e != cudaSuccess) return setf(&tr->err, GLS_ENOMEM, "training data", e);
    e = cudaMemcpy(tr->X.p, feat, n * kIn * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(tr->T.p, target, n * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return setf(&tr->err, GLS_ECUDA, "upload training data", e);
    tr->n = n;
    // start the output bias at the mean target
    double mean = 0.0;
    for (uint64_t i = 0; i < n; ++i) mean += target[i];
    const float b3 = (float)(mean / (double)n);
    cudaMemcpy(tr->P.as<float>() + kOffB3, &b3, 4, cudaMemcpyHostToDevice);
    return GLS_OK;
}

extern "C" int gls_trainer_fit(gls_trainer *tr, const gls_train_opts *o, float *loss)
{
    if (!tr || !o || !o->batch || !tr->n) return GLS_EINVAL;
    cudaSetDevice(tr->device);
    const uint32_t nb_max = (uint32_t)std::min<uint64_t>(o->batch, tr->n);
    int rc = tr_alloc_batch(tr, nb_max);
    if (rc) return rc;
    uint64_t s = o->seed ^ 0x5DEECE66Dull;
    for (uint32_t ep = 0; ep < o->epochs; ++ep) {
        // a fresh pseudo-random permutation of the rows every epoch
        uint64_t mul = splitmix(s) % tr->n;
        if (mul == 0) mul = 1;
        while (gcd64(mul, tr->n) != 1) mul = mul + 1 < tr->n ? mul + 1 : 1;
        const uint64_t add = splitmix(s) % tr->n;
        cudaMemsetAsync(tr->loss.p, 0, 4, tr->st);
        for (uint64_t b0 = 0; b0 < tr->n; b0 += nb_max) {
            const int nb = (int)std::min<uint64_t>(nb_max, tr->n - b0);
            k_gather<<<(unsigned)(((long)nb * kIn + 255) / 256), 256, 0, tr->st>>>(
                nb, b0, mul, add, tr->n, tr->X.as<float>(), tr->T.as<float>(), tr->Xb.as<float>(), tr->Tb.as<float>());
            tr_step_grad(tr, nb, o->huber);
            ++tr->adam_t;
            const float c1 = 1.f / (1.f - std::pow(0.9f, (float)tr->adam_t));
            const float c2 = 1.f / (1.f - std::pow(0.999f, (float)tr->adam_t));
            k_adam<<<(kParams + 255) / 256, 256, 0, tr->st>>>(kParams, tr->P.as<float>(), tr->G.as<float>(),
                                                               tr->Mo.as<float>(), tr->Vo.as<float>(), o->lr, c1, c2);
        }
        float ls = 0.f;
        cudaMemcpyAsync(&ls, tr->loss.p, 4, cudaMemcpyDeviceToHost, tr->st);
        const cudaError_t e = cudaStreamSynchronize(tr->st);
        if (e != cudaSuccess) return setf(&tr->err, GLS_ECUDA, "training step", e);
        if (loss) loss[ep] = (float)(ls / (double)tr->n);
    }
    return GLS_OK;
}

extern "C" int gls_trainer_grad(gls_trainer *tr, uint64_t first, uint64_t n, float huber, float *grad, float *loss)
{
    if (!tr || !grad || !n || first + n > tr->n || n > 0x7FFFFFFFull) return GLS_EINVAL;
    cudaSetDevice(tr->device);
    int rc = tr_alloc_batch(tr, (uint32_t)n);
    if (rc) return rc;
    cudaMemcpyAsync(tr->Xb.p, tr->X.as<float>() + first * kIn, n * kIn * 4, cudaMemcpyDeviceToDevice, tr->st);
    cudaMemcpyAsync(tr->Tb.p, tr->T.as<float>() + first, n * 4, cudaMemcpyDeviceToDevice, tr->st);
    cudaMemsetAsync(tr->loss.p, 0, 4, tr->st);
    tr_step_grad(tr, (int)n, huber);
    cudaMemcpyAsync(grad, tr->G.p, kParams * 4, cudaMemcpyDeviceToHost, tr->st);
    float ls = 0.f;
    cudaMemcpyAsync(&ls, tr->loss.p, 4, cudaMemcpyDeviceToHost, tr->st);
    const cudaError_t e = cudaStreamSynchronize(tr->st);
    if (e != cudaSuccess) return setf(&tr->err, GLS_ECUDA, "gradient", e);
    if (loss) *loss = ls / (float)n;
    return GLS_OK;
}

extern "C" int gls_trainer_get_params(gls_trainer *tr, float *params)
{
    if (!tr || !params) return GLS_EINVAL;
    cudaSetDevice(tr->device);
    return cudaMemcpy(params, tr->P.p, kParams * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? GLS_OK : GLS_ECUDA;
}

extern "C" int gls_trainer_set_params(gls_trainer *tr, const float *params)
{
    if (!tr || !params) return GLS_EINVAL;
    cudaSetDevice(tr->device);
    if (cudaMemcpy(tr->P.p, params, kParams * 4, cudaMemcpyHostToDevice) != cudaSuccess) return GLS_ECUDA;
    cudaMemset(tr->Mo.p, 0, kParams * 4);
    cudaMemset(tr->Vo.p, 0, kParams * 4);
    tr->adam_t = 0;
    return GLS_OK;
}

// ------------------------------------------------- context-side presize
extern "C" int gls_set_presize_model(gls_ctx *ctx, const gls_presize_model *m)
{
    if (!ctx || !m) return GLS_EINVAL;
    if (!(m->margin >= 0.f) || m->margin > 100.f) return ctx_fail(ctx, GLS_EINVAL, "presize margin out of range");
    for (int k = 0; k < kParams; ++k)
        if (!std::isfinite(m->params[k])) return ctx_fail(ctx, GLS_EINVAL, "presize parameter %d is not finite", k);
    cudaSetDevice(ctx->opts.device);
    const std::vector<uint8_t> img = weight_image(m->params);
    cudaError_t e = ctx->mlp_params.ensure(kParams * 4);
    if (e == cudaSuccess) e = ctx->mlp_img.ensure(kImgBytes);
    if (e == cudaSuccess) e = ctx->aux.ensure(64);
    if (e == cudaSuccess) e = cudaMemcpy(ctx->mlp_params.p, m->params, kParams * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ctx->mlp_img.p, img.data(), kImgBytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "upload presize model: %s", cudaGetErrorString(e));
    ctx->margin = m->margin;
    ctx->slack = m->slack;
    ctx->have_model = true;
    ctx_drop_graphs(ctx);
    prepare_presize_kernels();
    return GLS_OK;
}

void ctx_presize_args(const gls_ctx *ctx, PresizeArgs *a)
{
    std::memset(a, 0, sizeof *a);
    a->feat_static = ctx->feat_static.as<float>();
    a->meta = ctx->meta.as<DrvMeta>();
    a->lut = ctx->lut.as<uint8_t>();
    a->params = ctx->mlp_params.as<float>();
    a->img = ctx->mlp_img.as<uint4>();
    a->margin = ctx->margin;
    a->slack = ctx->slack;
}

extern "C" int gls_presize_samples(gls_ctx *ctx, uint32_t window, float *feat, uint32_t *count, uint64_t cap,
                                   uint64_t *n)
{
    if (!ctx || !n) return GLS_EINVAL;
    if (!ctx->loaded) return ctx_fail(ctx, GLS_ESTATE, "presize_samples before load_netlist");
    if (window >= ctx->windows.size() || !ctx->windows[window]->done)
        return ctx_fail(ctx, GLS_ESTATE, "presize_samples: window %u has not run", window);
    *n = ctx->n_drv;
    if (!feat || !count) return GLS_OK;
    if (cap < ctx->n_drv) return ctx_fail(ctx, GLS_EINVAL, "presize_samples: room for %llu rows, %u needed",
                                          (unsigned long long)cap, ctx->n_drv);
    cudaSetDevice(ctx->opts.device);
    Window *w = ctx->windows[window];
    PresizeArgs a;
    ctx_presize_args(ctx, &a);
    a.net_len = w->net_len.as<uint32_t>();
    a.saif = w->saif.as<unsigned long long>();
    a.lo = 0;
    a.n = ctx->n_drv;
    DevBuf out;
    cudaError_t e = out.ensure((size_t)ctx->n_drv * kIn * 4);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ENOMEM, "presize_samples: %s", cudaGetErrorString(e));
    launch_features(a, out.as<float>(), ctx->stream);
    e = cudaMemcpyAsync(feat, out.p, (size_t)ctx->n_drv * kIn * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    out.release();
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "presize_samples: %s", cudaGetErrorString(e));
    // output lengths in driver order
    std::vector<uint32_t> len(ctx->n_nets);
    e = cudaMemcpy(len.data(), w->net_len.p, (size_t)ctx->n_nets * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "presize_samples: %s", cudaGetErrorString(e));
    std::vector<DrvMeta> meta(ctx->n_drv);
    e = cudaMemcpy(meta.data(), ctx->meta.p, (size_t)ctx->n_drv * sizeof(DrvMeta), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "presize_samples: %s", cudaGetErrorString(e));
    for (uint32_t d = 0; d < ctx->n_drv; ++d) count[d] = len[meta[d].out_net];
    return GLS_OK;
}

extern "C" int gls_presize_predict(gls_ctx *ctx, const gls_presize_model *m, const float *feat, uint64_t n, float *y,
                                   int tensor_cores)
{
    if (!ctx || !m || !feat || !y || !n || n > 0x7FFFFFFFull) return GLS_EINVAL;
    cudaSetDevice(ctx->opts.device);
    const std::vector<uint8_t> img = weight_image(m->params);
    DevBuf prm, im, rows, out, er;
    cudaError_t e = prm.ensure(kParams * 4);
    if (e == cudaSuccess) e = im.ensure(kImgBytes);
    if (e == cudaSuccess) e = rows.ensure(n * kIn * 4);
    if (e == cudaSuccess) e = out.ensure(n * 4);
    if (e == cudaSuccess) e = er.ensure(16);
    if (e == cudaSuccess) e = cudaMemcpy(prm.p, m->params, kParams * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(im.p, img.data(), kImgBytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(rows.p, feat, n * kIn * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(er.p, 0, 16);
    prepare_presize_kernels();
    uint32_t flag = 0;
    if (e == cudaSuccess) {
        PresizeArgs a;
        std::memset(&a, 0, sizeof a);
        a.rows = rows.as<float>();
        a.n = (uint32_t)n;
        a.params = prm.as<float>();
        a.img = im.as<uint4>();
        a.y = out.as<float>();
        a.err = er.as<uint32_t>();
        launch_presize(a, tensor_cores != 0, ctx->stream);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(y, out.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, er.p, 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    prm.release(); im.release(); rows.release(); out.release(); er.release();
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "presize_predict: %s", cudaGetErrorString(e));
    if (flag) return ctx_fail(ctx, GLS_ECUDA, "presize_predict: tensor-core kernel timed out waiting for its MMA");
    return GLS_OK;
}
