// gls_levelize: Kahn levels of an instance graph on the GPU.
//
// The reference levelizes in `process` (GenerateAdjacencyList,
// SetInDegrees, TopologyOrder; src/process.cpp:90-176): level 0 holds the
// instances without predecessors, and every later level takes, in instance
// order, the instances whose predecessors are all placed.  An instance's
// level is therefore the length of the longest predecessor chain that ends
// at it.  Here every sweep over the instances gives a level to each
// instance whose predecessors all have one (one more than the largest of
// theirs); levels given earlier in the same sweep are read at once, so a
// sweep can place several levels.  The host then buckets the instances by
// level in instance order (the reference's level packing, 423-566).
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <vector>
#include "gls.h"

namespace {

constexpr uint32_t kUnset = 0xFFFFFFFFu;

// pred[e] < n for every edge, else *bad = 1
__global__ void k_check_preds(uint64_t n_edges, uint32_t n, const uint32_t *__restrict__ pred, uint32_t *bad)
{
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_edges; e += (uint64_t)gridDim.x * blockDim.x)
        if (pred[e] >= n) *bad = 1;
}

// One sweep: an instance without a level takes one when all its
// predecessors have one.  A level word is written once, from kUnset to its
// final value, so a concurrent reader sees one or the other.
__global__ void k_level_sweep(uint32_t n, const uint64_t *__restrict__ ps, const uint32_t *__restrict__ pred,
                              uint32_t *lv, unsigned long long *placed)
{
    uint32_t mine = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (lv[i] != kUnset) continue;
        uint32_t m = 0;
        bool ready = true;
        for (uint64_t e = ps[i]; e < ps[i + 1]; ++e) {
            const uint32_t l = reinterpret_cast<volatile uint32_t *>(lv)[pred[e]];
            if (l == kUnset) { ready = false; break; }
            m = max(m, l + 1);
        }
        if (ready) {
            reinterpret_cast<volatile uint32_t *>(lv)[i] = m;
            ++mine;
        }
    }
    if (mine) atomicAdd(placed, (unsigned long long)mine);
}

struct Buf {
    void *p = nullptr;
    ~Buf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, n ? n : 16); }
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

}  // namespace

extern "C" int gls_levelize(int device, uint32_t n_inst, const uint64_t *pred_start, const uint32_t *pred,
                            uint32_t *order, uint32_t *level_start, uint32_t *n_levels)
{
    if (!order || !level_start || !n_levels || (n_inst && !pred_start)) return GLS_EINVAL;
    *n_levels = 0;
    level_start[0] = 0;
    if (n_inst == 0) return GLS_OK;
    // a monotone start table keeps every read of the predecessor list in range
    if (pred_start[0] != 0) return GLS_EINVAL;
    for (uint32_t i = 0; i < n_inst; ++i)
        if (pred_start[i + 1] < pred_start[i]) return GLS_EINVAL;
    const uint64_t n_edges = pred_start[n_inst];
    if (n_edges && !pred) return GLS_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return GLS_ECUDA;
    Buf d_ps, d_pred, d_lv, d_small;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return GLS_ECUDA;
    int rc = GLS_OK;
    std::vector<uint32_t> lv(n_inst);
    do {
        if (d_ps.alloc((size_t)(n_inst + 1) * 8) || d_pred.alloc(n_edges * 4) || d_lv.alloc((size_t)n_inst * 4) ||
            d_small.alloc(64)) {
            rc = GLS_ENOMEM;
            break;
        }
        if (cudaMemcpyAsync(d_ps.p, pred_start, (size_t)(n_inst + 1) * 8, cudaMemcpyHostToDevice, st) ||
            (n_edges && cudaMemcpyAsync(d_pred.p, pred, n_edges * 4, cudaMemcpyHostToDevice, st)) ||
            cudaMemsetAsync(d_lv.p, 0xFF, (size_t)n_inst * 4, st) || cudaMemsetAsync(d_small.p, 0, 64, st)) {
            rc = GLS_ECUDA;
            break;
        }
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        const uint32_t grid = (uint32_t)std::max(1, sms) * 8;
        uint32_t *bad = d_small.as<uint32_t>();
        unsigned long long *placed = reinterpret_cast<unsigned long long *>(d_small.as<uint32_t>() + 2);
        if (n_edges) k_check_preds<<<grid, 256, 0, st>>>(n_edges, n_inst, d_pred.as<uint32_t>(), bad);
        uint32_t h_bad = 0;
        if (cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st)) {
            rc = GLS_ECUDA;
            break;
        }
        if (h_bad) {   // a predecessor index out of range
            rc = GLS_EINVAL;
            break;
        }
        unsigned long long done = 0, before = 0;
        for (;;) {
            k_level_sweep<<<grid, 256, 0, st>>>(n_inst, d_ps.as<uint64_t>(), d_pred.as<uint32_t>(), d_lv.as<uint32_t>(),
                                                placed);
            if (cudaMemcpyAsync(&done, placed, 8, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st)) {
                rc = GLS_ECUDA;
                break;
            }
            if (done == n_inst) break;
            if (done == before) {   // nothing placed: the rest lies on or behind a loop
                rc = GLS_EINVAL;
                break;
            }
            before = done;
        }
        if (rc) break;
        if (cudaMemcpyAsync(lv.data(), d_lv.p, (size_t)n_inst * 4, cudaMemcpyDeviceToHost, st) ||
            cudaStreamSynchronize(st)) {
            rc = GLS_ECUDA;
            break;
        }
    } while (false);
    cudaStreamDestroy(st);
    if (rc) return rc;
    // level packing: the instances of every level in instance order
    uint32_t nl = 0;
    for (uint32_t i = 0; i < n_inst; ++i) nl = std::max(nl, lv[i] + 1);
    std::vector<uint32_t> at(nl + 1, 0);
    for (uint32_t i = 0; i < n_inst; ++i) ++at[lv[i] + 1];
    for (uint32_t k = 0; k < nl; ++k) at[k + 1] += at[k];
    for (uint32_t k = 0; k <= nl; ++k) level_start[k] = at[k];
    for (uint32_t i = 0; i < n_inst; ++i) order[at[lv[i]]++] = i;
    *n_levels = nl;
    return GLS_OK;
}
