// Host-side context of libgls, shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include "gls.h"
#include "gls_internal.h"

namespace glsh {

// Host threads kept for the context's lifetime: parallel_for(n, f) calls
// f(0) .. f(n-1) on them and on the caller, and returns when all are done.
// (A call per window would otherwise start and join its threads each time.)
class WorkPool {
public:
    explicit WorkPool(unsigned threads)
    {
        try {
            for (unsigned i = 0; i < threads; ++i) th_.emplace_back([this] { loop(); });
        } catch (...) {   // the threads started so far end before the error leaves
            shutdown();
            throw;
        }
    }
    ~WorkPool() { shutdown(); }
    unsigned threads() const { return (unsigned)th_.size() + 1; }
    void parallel_for(unsigned n, const std::function<void(unsigned)> &f)
    {
        {
            std::lock_guard<std::mutex> l(mu_);
            f_ = &f;
            n_ = n;
            next_ = 0;
            left_ = n;
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> l(mu_);
        done_.wait(l, [this] { return left_ == 0; });
        f_ = nullptr;
    }

private:
    void shutdown()
    {
        {
            std::lock_guard<std::mutex> l(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_)
            if (t.joinable()) t.join();
        th_.clear();
    }
    void work()
    {
        for (;;) {
            unsigned i;
            const std::function<void(unsigned)> *f;
            {
                std::lock_guard<std::mutex> l(mu_);
                if (!f_ || next_ >= n_) return;
                i = next_++;
                f = f_;
            }
            (*f)(i);
            std::lock_guard<std::mutex> l(mu_);
            if (--left_ == 0) done_.notify_all();
        }
    }
    void loop()
    {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> l(mu_);
                cv_.wait(l, [&] { return stop_ || (gen_ != seen && f_ && next_ < n_); });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(unsigned)> *f_ = nullptr;
    unsigned n_ = 0, next_ = 0, left_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n)
    {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n ? n : 16);
        if (e == cudaSuccess) bytes = n ? n : 16;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

struct PinBuf {   // page-locked host staging, reused across windows
    void *p = nullptr;
    size_t bytes = 0;
    bool ensure(size_t n)
    {
        if (n <= bytes && p) return true;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        if (cudaHostAlloc(&p, n ? n : 16, cudaHostAllocDefault) != cudaSuccess) return false;
        bytes = n ? n : 16;
        return true;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T> T *as() const { return static_cast<T *>(p); }
};

// One window's per-level work space: segment tables, slot offsets and the
// segment stacks.  Sequential runs share set 0; a wave of windows run
// together takes one set per window.
struct LevelScratch {
    DevBuf seg_base, slot, scr, res, pred, segs, copies, scratch;
    // the per-gate-output tables of odd levels: the next level's plan fills
    // one set while the previous level's copy still reads the other
    DevBuf seg_base1, slot1, scr1, res1;
    uint32_t seg_cap = 0;
    uint64_t scr_cap = 0;
    uint32_t width = 0;
    cudaError_t ensure(uint32_t w, uint32_t segs_need, uint64_t words_need)
    {
        cudaError_t e = cudaSuccess;
        if (w > width) {
            const size_t n = (size_t)w + 1;
            if (e == cudaSuccess) e = seg_base.ensure(n * 4);
            if (e == cudaSuccess) e = slot.ensure(n * 8);
            if (e == cudaSuccess) e = scr.ensure(n * 8);
            if (e == cudaSuccess) e = res.ensure(n * 4);
            if (e == cudaSuccess) e = pred.ensure(n * 4);
            if (e == cudaSuccess) e = seg_base1.ensure(n * 4);
            if (e == cudaSuccess) e = slot1.ensure(n * 8);
            if (e == cudaSuccess) e = scr1.ensure(n * 8);
            if (e == cudaSuccess) e = res1.ensure(n * 4);
            if (e == cudaSuccess) width = w;
        }
        if (e == cudaSuccess && segs_need > seg_cap) {
            // room for the segment records of either event-word width
            e = segs.ensure((size_t)segs_need * gls::kSegRecMax);
            if (e == cudaSuccess) e = copies.ensure((size_t)segs_need * sizeof(gls::CopyRec));
            if (e == cudaSuccess) seg_cap = segs_need;
        }
        if (e == cudaSuccess && words_need > scr_cap) {
            e = scratch.ensure(words_need * 4);
            if (e == cudaSuccess) scr_cap = words_need;
        }
        return e;
    }
    void release()
    {
        DevBuf *all[] = {&seg_base, &slot, &scr, &res, &pred, &segs, &copies, &scratch,
                         &seg_base1, &slot1, &scr1, &res1};
        for (DevBuf *b : all) b->release();
        seg_cap = 0;
        scr_cap = 0;
        width = 0;
    }
};

struct Window {
    std::vector<uint32_t> stim_nets;
    std::vector<uint64_t> stim_off;     // aligned pool offset per stimulus net
    std::vector<uint32_t> stim_len;
    uint64_t stim_events = 0;           // aligned extent of the stimulus in the pool
    PinBuf h_words;                     // packed stimulus events (kept to re-upload on pool growth)
    PinBuf h_off, h_len;                // initial net table
    uint64_t t_begin = 0, t_end = 0;
    uint64_t cap = 0;
    DevBuf pool, net_off, net_len, init_off, init_len, saif, small, stim_dev;
    DevBuf dwin;                        // the window's WinDev on the device (sequential runs)
    bool done = false;
    bool uploaded = false;              // device buffers hold this stimulus (uploaded when the window first runs)
    bool saif_only = false;             // pool released after a batched run: SAIF counts and lengths kept
    // 64-bit event words: a stimulus time or a gate output past 2^30 - 2
    // (the pool, the stimulus staging and the level stacks hold 8 bytes per
    // event; the window runs alone, through the thread-per-segment kernels)
    bool w64 = false;
    uint64_t word_bytes() const { return w64 ? 8 : 4; }
};

}  // namespace glsh
using namespace glsh;

struct gls_ctx {
    gls_opts opts{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // fan-in classes of a level run concurrently: side streams fork after the
    // plan and join before the link (GLS_SIM_CONCURRENT=0 runs them in turn)
    cudaStream_t side[gls::kClasses] = {};
    cudaStream_t side_prio[gls::kClasses] = {};   // the same with priority rising with fan-in
    cudaEvent_t fork_ev = nullptr, join_ev[gls::kClasses] = {};
    cudaEvent_t link_ev[gls::kClasses] = {}, copy_ev[gls::kClasses] = {};
    cudaEvent_t slots_ev = nullptr;          // learned mode, split plan: the level's slots are placed
    cudaStream_t stim_side = nullptr;        // the stimulus SAIF beside the first levels
    cudaEvent_t stim_fork = nullptr, stim_join = nullptr;
    bool plan_overlap = true;        // the next level's plan runs beside this level's copies (GLS_PLAN_OVERLAP)
    bool concurrent = true;
    bool wide_first = false;         // launch the widest fan-in class first (GLS_WIDE_FIRST)
    bool class_priority = false;     // wider classes on higher-priority side streams (GLS_CLASS_PRIORITY)
    uint32_t sim_variant = 0;        // thread-per-segment gate kernel: bit 0 256-thread blocks, bit 1 wider loads
    float bal_weight = 0.f;          // learned balance of segments in use (0: off)
    float bal_weight_on = 0.5f;      // its factor when GLS_SCHED_LEARNED_BALANCE is set (GLS_BALANCE_WEIGHT)
    bool pipeline = true;            // with concurrent classes: each class links and copies on its own stream
    uint32_t copy_lanes = 8;         // lanes per segment of the copy kernel (GLS_COPY_LANES: 4, 8, 16, 32)
    int sm_count = 0;
    std::string err;
    bool loaded = false;
    uint32_t n_nets = 0;
    uint32_t n_drv = 0;
    std::vector<uint32_t> drv_level_start;   // per level, into drivers
    std::vector<uint32_t> cls_start;         // per level kClasses+1 entries: fan-in class ranges, level-relative
    uint32_t max_width = 0;
    uint64_t pins_total = 0;
    std::vector<uint8_t> driven;             // net driven by a gate output
    std::vector<uint32_t> ext_inputs;        // nets read by gates and driven by no gate
    DevBuf meta, arcs, ndel, lut, slut;
    std::vector<LevelScratch *> lsc;         // level work spaces ([0]: sequential runs)
    uint32_t seg_cap = 0;                    // segment-table size new work spaces get
    uint64_t scr_cap = 0;                    // stack words new work spaces get
    uint32_t def_delay = 1;
    uint32_t warp_mask = 0;          // fan-in classes run by the warp-per-segment kernel (GLS_SIM_WARP_MASK)
    uint32_t seg_per_sm = 2048;      // time segments per SM and fan-in class for the thread-per-segment kernel
    uint32_t seg_target_w = 0;       // segments per class for those kernels (GLS_SIM_WARP_SEGS per SM)
    uint64_t pool_gap = 0;           // unused events between the stimulus and the first gate output (GLS_POOL_GAP_EVENTS)
    double pool_ratio = 0.0;         // gate-output pool events per (mean stimulus list x input pins) seen so far
    // learned presize (GLS_ALLOC_LEARNED)
    DevBuf feat_static;              // per driver x 32 static features
    DevBuf mlp_params, mlp_img;      // FP32 parameters and the BF16 weight image
    DevBuf aux;                      // small device scratch of the presize calls (error word)
    bool have_model = false;
    float margin = 0.f;
    uint32_t slack = 0;
    std::vector<Window *> windows;
    std::vector<Window *> spare;     // cleared windows whose buffers are reused
    gls_stats stats{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> prof;   // per-launch events when opts.profile
    size_t prof_used = 0;
    // batched runs: the wave's window descriptors (host pinned, device) and
    // the captured launch graphs, one per wave shape
    PinBuf hwave;
    PinBuf pin_out;                  // staging of SAIF counts and lengths read back to the host
    WorkPool *pool = nullptr;        // host threads that pack stimuli (made on first use)
    DevBuf dwave;
    DevBuf wave_e;                   // per level: a wave's fan-in events per class
    std::vector<DevBuf> spare_bufs;  // device buffers of windows that ran saif_only, reused by later windows
    struct WaveGraph {
        uint32_t nwin, max_stim, warp_mask, alloc_mode, seg_per_sm, flags;   // flags: GLS_SCHED_*
        cudaGraphExec_t exec;
        uint32_t launches;
        bool same(const WaveGraph &o) const
        {
            return nwin == o.nwin && max_stim == o.max_stim && warp_mask == o.warp_mask &&
                   alloc_mode == o.alloc_mode && seg_per_sm == o.seg_per_sm && flags == o.flags;
        }
    };
    std::vector<WaveGraph> graphs;
};


// Sets the context's error message and returns `code`.
int ctx_fail(gls_ctx *c, int code, const char *fmt, ...);
// The per-level kernel arguments that do not depend on the level.
void ctx_level_args(const gls_ctx *ctx, gls::LevelArgs *a);
namespace gls { struct PresizeArgs; }
// The presize-kernel arguments of the installed model (rows, range and outputs left empty).
void ctx_presize_args(const gls_ctx *ctx, gls::PresizeArgs *a);
// Forget the captured wave graphs (they bake in tables and options).
void ctx_drop_graphs(gls_ctx *ctx);
