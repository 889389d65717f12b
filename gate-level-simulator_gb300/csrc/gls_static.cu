// gls_run_level_static: one level of gate outputs simulated with no device
// allocation at all.
//
// Who needs this: callers that cannot call cudaMalloc while they simulate --
// for example a host application that owns all device memory through its
// own arena and forbids other allocations, or a latency-sensitive loop that
// cannot afford the implicit device synchronization a cudaMalloc/cudaFree
// may cause.  Such a caller keeps the event pool, the net table and the
// SAIF counters in its own buffers and hands them in; everything else the
// level kernels need (segment stacks and segment tables) lives in one
// file-scope static device array whose size is fixed when the library is
// loaded.
//
// The level kernels are the same ones gls_run launches; only where their
// scratch lives differs.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <string>
#include "gls.h"
#include "gls_ctx.h"
#include "gls_internal.h"

namespace gls {
namespace {

// Limits of one call (stated in include/gls.h).
constexpr uint32_t kStaticMaxOutputs = 16384;        // gate outputs per call
constexpr uint32_t kStaticMaxSegments = 65536;       // time segments per call
constexpr uint64_t kStaticMaxWords = 4194304;        // segment-stack words per call (16 MiB)

// Layout of the static scratch (byte offsets, each 256-byte aligned).
constexpr uint64_t al256(uint64_t x) { return (x + 255) & ~255ull; }
constexpr uint64_t kOffSmall = 0;   // 8 x u64: saved pool pointer, 4 counters, err, n_segs, presize overflows
constexpr uint64_t kOffWin = 64;                                             // the level kernels' WinDev
constexpr uint64_t kOffSegBase = al256(kOffWin + sizeof(WinDev));
constexpr uint64_t kOffSlot = al256(kOffSegBase + 4ull * (kStaticMaxOutputs + 1));
constexpr uint64_t kOffScr = al256(kOffSlot + 8ull * (kStaticMaxOutputs + 1));
constexpr uint64_t kOffSegs = al256(kOffScr + 8ull * (kStaticMaxOutputs + 1));
constexpr uint64_t kOffCopies = al256(kOffSegs + sizeof(SegRec) * kStaticMaxSegments);
constexpr uint64_t kOffWords = al256(kOffCopies + sizeof(CopyRec) * kStaticMaxSegments);
constexpr uint64_t kStaticBytes = al256(kOffWords + 4ull * kStaticMaxWords);

// Held by every GPU that loads the library, until the process exits.
static __device__ __align__(256) unsigned char g_level_scratch[kStaticBytes];

// The device address of g_level_scratch, resolved once per device: in host
// code the symbol's name is only a host-side stand-in for it.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {};

int scratch_address(int device, unsigned char **out, std::string &err)
{
    if (device < 0 || device >= kMaxDevices) {
        err = "device ordinal out of range for the static scratch table";
        return GLS_EINVAL;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void *p = nullptr;
        // With lazy module loading (the CUDA default) this lookup is what
        // loads the module and reserves the array on the device, so it can
        // fail for lack of device memory when a caller's arena already holds
        // all of it.
        const cudaError_t e = cudaGetSymbolAddress(&p, g_level_scratch);
        if (e != cudaSuccess) {
            err = std::string("cudaGetSymbolAddress of the static scratch failed: ") + cudaGetErrorString(e);
            if (e == cudaErrorMemoryAllocation) {
                cudaGetLastError();   // reset the last-error state (an allocation failure is not sticky)
                err += " (the 20 MiB static array could not be reserved: make the first call before an arena "
                       "takes the remaining device memory)";
                return GLS_ENOMEM;
            }
            return GLS_ECUDA;
        }
        g_addr[device] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[device];
    return GLS_OK;
}

}  // namespace
}  // namespace gls

using namespace gls;

extern "C" int gls_run_level_static(gls_ctx *ctx, uint32_t level, uint32_t first, uint32_t count, uint32_t *d_pool,
                                    uint64_t pool_cap, unsigned long long *d_top, uint64_t *d_net_off,
                                    uint32_t *d_net_len, unsigned long long *d_saif, uint64_t t_begin,
                                    uint64_t t_end)
{
    if (!ctx) return GLS_EINVAL;
    if (!ctx->loaded) return ctx_fail(ctx, GLS_ESTATE, "run_level_static before load_netlist");
    if (!d_pool || !d_top || !d_net_off || !d_net_len || !d_saif)
        return ctx_fail(ctx, GLS_EINVAL, "run_level_static: null device buffer");
    if (t_end <= t_begin) return ctx_fail(ctx, GLS_EINVAL, "run_level_static: window end must exceed begin");
    if (level + 1 >= ctx->drv_level_start.size())
        return ctx_fail(ctx, GLS_EINVAL, "run_level_static: level %u out of range", level);
    const uint32_t lo = ctx->drv_level_start[level], hi = ctx->drv_level_start[level + 1];
    if ((uint64_t)first + count > hi - lo)
        return ctx_fail(ctx, GLS_EINVAL, "run_level_static: outputs [%u, %llu) outside level %u (%u outputs)", first,
                        (unsigned long long)first + count, level, hi - lo);
    if (count > kStaticMaxOutputs)
        return ctx_fail(ctx, GLS_ERANGE, "run_level_static: %u gate outputs in one call; the static scratch holds %u",
                        count, kStaticMaxOutputs);
    if (count == 0) return GLS_OK;
    cudaError_t e = cudaSetDevice(ctx->opts.device);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    unsigned char *base = nullptr;
    std::string err;
    int rc = scratch_address(ctx->opts.device, &base, err);
    if (rc) return ctx_fail(ctx, rc, "%s", err.c_str());
    unsigned long long *small = reinterpret_cast<unsigned long long *>(base + kOffSmall);
    // every call starts from cleared flags and counters (the array keeps the
    // previous call's contents otherwise)
    e = cudaMemsetAsync(small, 0, 64, ctx->stream);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "clear static flags: %s", cudaGetErrorString(e));
    // the caller's pool pointer as it was, put back if the level fails, so
    // that a failed call (e.g. GLS_ERANGE, retried with fewer outputs) uses
    // up no pool space; small[0] holds it
    e = cudaMemcpyAsync(small, d_top, 8, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "save pool pointer: %s", cudaGetErrorString(e));
    WinDev d;
    std::memset(&d, 0, sizeof d);
    d.net_off = d_net_off;
    d.net_len = d_net_len;
    d.pool = d_pool;
    d.saif = d_saif;
    d.top = d_top;
    d.counters = small + 1;
    d.err = reinterpret_cast<uint32_t *>(small + 5);
    d.n_segs = reinterpret_cast<uint32_t *>(small + 6);
    d.n_over = small + 7;
    d.seg_base = reinterpret_cast<uint32_t *>(base + kOffSegBase);
    d.slot = reinterpret_cast<uint64_t *>(base + kOffSlot);
    d.scr = reinterpret_cast<uint64_t *>(base + kOffScr);
    d.segs = reinterpret_cast<SegRec *>(base + kOffSegs);
    d.copies = reinterpret_cast<CopyRec *>(base + kOffCopies);
    d.scratch = reinterpret_cast<uint32_t *>(base + kOffWords);
    d.cap = pool_cap;
    d.scr_cap = kStaticMaxWords;
    d.seg_cap = kStaticMaxSegments;
    d.t_begin = t_begin;
    d.t_end = t_end;
    LevelArgs a;
    ctx_level_args(ctx, &a);
    a.alloc_mode = kAllocBound;   // the caller's pool: slots reserved up front
    a.lo = lo + first;
    a.hi = a.lo + count;
    // the descriptor goes into its slot of the static array (no allocation)
    WinDev *dw = reinterpret_cast<WinDev *>(base + kOffWin);
    e = cudaMemcpyAsync(dw, &d, sizeof d, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "upload static descriptor: %s", cudaGetErrorString(e));
    launch_plan(dw, d, 1, a, ctx->stream);
    for (int c = 0; c < kClasses; ++c) {
        // the fan-in class ranges of the level, clipped to [first, first + count)
        const uint32_t c0 = ctx->cls_start[(kClasses + 1) * level + c], c1 = ctx->cls_start[(kClasses + 1) * level + c + 1];
        const uint32_t d0 = std::max(c0, first), d1 = std::min(c1, first + count);
        if (d1 > d0) launch_sim(dw, d, 1, a, c, d0 - first, d1 - first, ctx->sm_count, ctx->stream);
    }
    launch_link(dw, d, 1, a, 0, count, ctx->stream);
    launch_copy(dw, d, 1, a, 0, count, ctx->sm_count, ctx->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "level kernel launch: %s", cudaGetErrorString(e));
    unsigned long long st[8];
    e = cudaMemcpyAsync(st, small, sizeof st, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "run_level_static: %s", cudaGetErrorString(e));
    const uint32_t ef = (uint32_t)st[5];
    if (ef) {
        // k_link and k_copy skip a failed level, so net_off, net_len and the
        // SAIF counters are untouched; only the pool pointer may have moved
        e = cudaMemcpyAsync(d_top, small, 8, cudaMemcpyDeviceToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctx_fail(ctx, GLS_ECUDA, "restore pool pointer: %s", cudaGetErrorString(e));
        if (ef & kErrScratch)
            return ctx_fail(ctx, GLS_ERANGE,
                            "run_level_static: the outputs' fan-in events need more than the %llu-word static "
                            "segment scratch; pass fewer outputs per call",
                            (unsigned long long)kStaticMaxWords);
        if (ef & kErrSegCap)
            return ctx_fail(ctx, GLS_ERANGE, "run_level_static: more than %u time segments; pass fewer outputs per call",
                            kStaticMaxSegments);
        if (ef & kErrPool)
            return ctx_fail(ctx, GLS_EOVERFLOW, "run_level_static: the caller's event pool (%llu words) is full",
                            (unsigned long long)pool_cap);
        if (ef & kErrTime) return ctx_fail(ctx, GLS_ERANGE, "run_level_static: an output time passed 2^30-2");
        return ctx_fail(ctx, GLS_EINVAL, "run_level_static: simulation error flags 0x%x", ef);
    }
    return GLS_OK;
}
