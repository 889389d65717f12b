// C ABI of libgls: context, netlist upload, stimulus windows, level loop.
//
// The run of one window replaces the per-level host loop of the reference
// GPU tool (src/simulate.cu:2027-3254).  Nothing goes back to the host
// between levels: every net's change list stays in the device event pool,
// and a level's fan-in is read in place by the next level's kernels.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <thread>
#include <string>
#include <vector>
#include "gls.h"
#include "gls_internal.h"
#include "gls_ctx.h"
#include "gls_presize.h"

using namespace gls;

namespace {

int fail(gls_ctx *c, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

}  // namespace

int ctx_fail(gls_ctx *c, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

void ctx_level_args(const gls_ctx *ctx, LevelArgs *a)
{
    a->meta = ctx->meta.as<DrvMeta>();
    a->slut = ctx->slut.as<uint4>();
    a->arcs = ctx->arcs.as<ArcDev>();
    a->ndel = ctx->ndel.as<NetDelay>();
    a->lut = ctx->lut.as<uint8_t>();
    a->lo = a->hi = 0;
    a->seg_events = ctx->opts.seg_events;
    a->seg_target = (uint32_t)ctx->sm_count * ctx->seg_per_sm;
    a->seg_target_w = ctx->seg_target_w;
    a->warp_mask = ctx->warp_mask;
    a->def_delay = ctx->def_delay;
    a->alloc_mode = (uint32_t)ctx->opts.alloc_mode;
    a->copy_lanes = ctx->copy_lanes;
    a->sim_variant = ctx->sim_variant;
    a->bal_weight = ctx->bal_weight;
    a->wave_e = nullptr;
    a->wide = 0;
    a->plan_part = 0;
}

namespace {

int cuda_fail(gls_ctx *c, cudaError_t e, const char *what)
{
    return fail(c, e == cudaErrorMemoryAllocation ? GLS_ENOMEM : GLS_ECUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

#define CK(call, what)                                        \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

uint64_t round4(uint64_t x) { return (x + 3) & ~3ull; }

}  // namespace

extern "C" int gls_abi_version(void) { return GLS_ABI_VERSION; }

extern "C" const char *gls_last_error(const gls_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" int gls_create(const gls_opts *opts, gls_ctx **out)
{
    if (!out) return GLS_EINVAL;
    *out = nullptr;
    gls_ctx *ctx = new gls_ctx();
    if (opts) ctx->opts = *opts;
    else {
        ctx->opts.delay_factor = 1.0;
    }
    if (ctx->opts.delay_factor <= 0.0) ctx->opts.delay_factor = 1.0;
    if ((ctx->opts.calc_mode != GLS_CALC_FIXED && ctx->opts.calc_mode != GLS_CALC_LITERAL) ||
        ctx->opts.alloc_mode < GLS_ALLOC_BOUND || ctx->opts.alloc_mode > GLS_ALLOC_LEARNED) {
        delete ctx;
        return GLS_EINVAL;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0 || ctx->opts.device < 0 || ctx->opts.device >= ndev) {
        delete ctx;
        return GLS_ECUDA;
    }
    e = cudaSetDevice(ctx->opts.device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->opts.device);
    if (e == cudaSuccess) {
        if (ctx->opts.stream) ctx->stream = (cudaStream_t)ctx->opts.stream;
        else {
            e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
            ctx->own_stream = true;
        }
    }
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (const char *v = getenv("GLS_CLASS_PRIORITY")) ctx->class_priority = strtoul(v, nullptr, 0) != 0;
    if (const char *v = getenv("GLS_WIDE_FIRST")) ctx->wide_first = strtoul(v, nullptr, 0) != 0;
    if (const char *v = getenv("GLS_BALANCE_WEIGHT")) {   // sets the factor, and turns the balance on
        ctx->bal_weight_on = std::max(0.f, strtof(v, nullptr));
        ctx->bal_weight = ctx->bal_weight_on;
    }
    for (int c = 0; c < kClasses && e == cudaSuccess; ++c) {
        // two sets: default priority, and priority rising with fan-in (a schedule option)
        const int prio = c >= 2 ? prio_hi : (c == 1 ? (prio_lo + prio_hi) / 2 : prio_lo);
        e = cudaStreamCreateWithFlags(&ctx->side[c], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ctx->side_prio[c], cudaStreamNonBlocking, prio);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->join_ev[c], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->link_ev[c], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->copy_ev[c], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->slots_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stim_side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->stim_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->stim_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e != cudaSuccess) {
        delete ctx;
        return GLS_ECUDA;
    }
    ctx->def_delay = (uint32_t)std::min<uint64_t>((uint64_t)(1.0 * ctx->opts.delay_factor), kMaxDelay);
    // tuning knobs: which fan-in classes (bit 0: one input net, 1: two,
    // 2: three) run warp-per-segment, and how many segments per SM those
    // classes are cut into
    if (const char *v = getenv("GLS_SIM_WARP_MASK")) ctx->warp_mask = (uint32_t)strtoul(v, nullptr, 0) & 7u;
    if (const char *v = getenv("GLS_SIM_CONCURRENT")) ctx->concurrent = strtoul(v, nullptr, 0) != 0;
    if (const char *v = getenv("GLS_SIM_PIPELINE")) ctx->pipeline = strtoul(v, nullptr, 0) != 0;
    if (const char *v = getenv("GLS_PLAN_OVERLAP")) ctx->plan_overlap = strtoul(v, nullptr, 0) != 0;
    if (const char *v = getenv("GLS_COPY_LANES")) ctx->copy_lanes = (uint32_t)strtoul(v, nullptr, 0);
    uint32_t per_sm = 128;
    if (const char *v = getenv("GLS_SIM_WARP_SEGS")) per_sm = std::max(1u, (uint32_t)strtoul(v, nullptr, 0));
    ctx->seg_target_w = (uint32_t)ctx->sm_count * per_sm;
    // testing knob: leave this many unused events after the stimulus, so
    // that gate outputs sit at large pool offsets (64-bit indexing)
    if (const char *v = getenv("GLS_POOL_GAP_EVENTS")) ctx->pool_gap = (strtoull(v, nullptr, 0) + 3) & ~3ull;
    *out = ctx;
    return GLS_OK;
}

static void free_window(Window *w)
{
    w->pool.release(); w->net_off.release(); w->net_len.release();
    w->init_off.release(); w->init_len.release(); w->saif.release(); w->small.release();
    w->stim_dev.release();
    w->dwin.release();
    w->h_words.release(); w->h_off.release(); w->h_len.release();
    delete w;
}

extern "C" int gls_clear_windows(gls_ctx *ctx)
{
    if (!ctx) return GLS_EINVAL;
    cudaSetDevice(ctx->opts.device);
    cudaStreamSynchronize(ctx->stream);
    for (Window *w : ctx->windows) {
        w->done = false;
        ctx->spare.push_back(w);
    }
    ctx->windows.clear();
    return GLS_OK;
}

void ctx_drop_graphs(gls_ctx *ctx)
{
    for (auto &g : ctx->graphs) cudaGraphExecDestroy(g.exec);
    ctx->graphs.clear();
}

// a window's large device buffers go; its SAIF counts, lengths and flags stay
// a window's large device buffers go to the context's spares (saif_only);
// its SAIF counts, lengths and flags stay
static void release_window_pool(gls_ctx *ctx, Window *w)
{
    DevBuf *bufs[] = {&w->pool, &w->net_off, &w->init_off, &w->init_len, &w->stim_dev};
    for (DevBuf *b : bufs) {
        if (b->p) ctx->spare_bufs.push_back(*b);
        b->p = nullptr;
        b->bytes = 0;
    }
    w->uploaded = false;
}

static void free_spares(gls_ctx *ctx)
{
    for (DevBuf &b : ctx->spare_bufs) b.release();
    ctx->spare_bufs.clear();
}

static uint64_t spare_bytes(const gls_ctx *ctx)
{
    uint64_t t = 0;
    for (const DevBuf &b : ctx->spare_bufs) t += b.bytes;
    return t;
}

// dst holds at least `bytes`: kept if it does, else the smallest spare that
// does, else a new allocation (spares are freed first if memory is short)
static cudaError_t take_buf(gls_ctx *ctx, DevBuf &dst, size_t bytes)
{
    if (dst.p && dst.bytes >= bytes) return cudaSuccess;
    size_t best = SIZE_MAX;
    for (size_t k = 0; k < ctx->spare_bufs.size(); ++k)
        if (ctx->spare_bufs[k].bytes >= bytes && (best == SIZE_MAX || ctx->spare_bufs[k].bytes < ctx->spare_bufs[best].bytes))
            best = k;
    if (best != SIZE_MAX) {
        if (dst.p) ctx->spare_bufs.push_back(dst);
        dst = ctx->spare_bufs[best];
        ctx->spare_bufs.erase(ctx->spare_bufs.begin() + (long)best);
        return cudaSuccess;
    }
    cudaError_t e = dst.ensure(bytes);
    if (e == cudaErrorMemoryAllocation && !ctx->spare_bufs.empty()) {
        cudaGetLastError();
        free_spares(ctx);
        e = dst.ensure(bytes);
    }
    return e;
}

extern "C" int gls_destroy(gls_ctx *ctx)
{
    if (!ctx) return GLS_EINVAL;
    gls_clear_windows(ctx);
    for (Window *w : ctx->spare) free_window(w);
    ctx->spare.clear();
    ctx->meta.release(); ctx->arcs.release(); ctx->ndel.release(); ctx->lut.release(); ctx->slut.release();
    ctx_drop_graphs(ctx);
    ctx->hwave.release();
    ctx->pin_out.release();
    ctx->dwave.release();
    ctx->wave_e.release();
    free_spares(ctx);
    delete ctx->pool;
    ctx->pool = nullptr;
    for (LevelScratch *l : ctx->lsc) {
        l->release();
        delete l;
    }
    ctx->lsc.clear();
    ctx->feat_static.release(); ctx->mlp_params.release(); ctx->mlp_img.release(); ctx->aux.release();
    for (cudaEvent_t e : ctx->prof) cudaEventDestroy(e);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    for (int c = 0; c < kClasses; ++c) {
        if (ctx->side[c]) cudaStreamDestroy(ctx->side[c]);
        if (ctx->side_prio[c]) cudaStreamDestroy(ctx->side_prio[c]);
        if (ctx->join_ev[c]) cudaEventDestroy(ctx->join_ev[c]);
        if (ctx->link_ev[c]) cudaEventDestroy(ctx->link_ev[c]);
        if (ctx->copy_ev[c]) cudaEventDestroy(ctx->copy_ev[c]);
    }
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->slots_ev) cudaEventDestroy(ctx->slots_ev);
    if (ctx->stim_side) cudaStreamDestroy(ctx->stim_side);
    if (ctx->stim_fork) cudaEventDestroy(ctx->stim_fork);
    if (ctx->stim_join) cudaEventDestroy(ctx->stim_join);
    delete ctx;
    return GLS_OK;
}

extern "C" int gls_load_netlist(gls_ctx *ctx, const gls_netlist *nl)
{
    if (!ctx || !nl) return GLS_EINVAL;
    if (!nl->cells || !nl->prims || !nl->level_start || !nl->inst_cell || !nl->inst_pin_start ||
        !nl->inst_pin_net || !nl->inst_arc_start || (!nl->arcs && nl->inst_arc_start[nl->n_inst]))
        return fail(ctx, GLS_EINVAL, "netlist: null array");
    cudaSetDevice(ctx->opts.device);
    if (nl->level_start[0] != 0 || nl->level_start[nl->n_levels] != nl->n_inst)
        return fail(ctx, GLS_EINVAL, "netlist: level_start must span all instances");
    for (uint32_t c = 0; c < nl->n_cells; ++c) {
        const gls_cell &cl = nl->cells[c];
        if (cl.n_in > kMaxPins) return fail(ctx, GLS_EINVAL, "cell %u: %u inputs (max %d)", c, cl.n_in, kMaxPins);
        if ((uint64_t)cl.prim_start + cl.n_prim > nl->n_prims) return fail(ctx, GLS_EINVAL, "cell %u: primitive range", c);
    }
    // truth tables, one per (cell, output), built on first use
    std::map<std::pair<uint32_t, int>, uint32_t> lut_of;
    std::vector<uint8_t> h_lut;
    std::vector<DrvMeta> h_meta;
    std::vector<ArcDev> h_arcs;
    std::vector<NetDelay> h_ndel;
    std::vector<int32_t> drv_level_of_net(nl->n_nets, -1);
    ctx->drv_level_start.assign(1, 0);
    ctx->cls_start.clear();
    ctx->pins_total = 0;
    std::vector<uint8_t> consumed(nl->n_nets, 0);
    std::vector<uint32_t> fanout(nl->n_nets, 0), cell_of_net(nl->n_nets, 0xFFFFFFFFu);
    for (uint32_t L = 0; L < nl->n_levels; ++L) {
        for (uint32_t i = nl->level_start[L]; i < nl->level_start[L + 1]; ++i) {
            const uint32_t cid = nl->inst_cell[i];
            if (cid >= nl->n_cells) return fail(ctx, GLS_EINVAL, "instance %u: bad cell", i);
            const gls_cell &cl = nl->cells[cid];
            const uint32_t p0 = nl->inst_pin_start[i];
            if (nl->inst_pin_start[i + 1] - p0 != (uint32_t)cl.n_in + cl.n_out)
                return fail(ctx, GLS_EINVAL, "instance %u: pin count", i);
            const uint32_t *pins = nl->inst_pin_net + p0;
            DrvMeta md;
            std::memset(&md, 0, sizeof md);
            int m = 0;
            bool ident = true;
            for (int p = 0; p < cl.n_in; ++p) {
                const uint32_t net = pins[p];
                if (net >= nl->n_nets) return fail(ctx, GLS_EINVAL, "instance %u: bad net", i);
                consumed[net] = 1;
                ++fanout[net];
                int slotp = -1;
                for (int j = 0; j < m; ++j) if (md.net[j] == net) slotp = j;
                if (slotp < 0) {
                    if (m == kMaxSlots) return fail(ctx, GLS_EINVAL, "instance %u: too many fan-in nets", i);
                    md.net[m] = net;
                    slotp = m++;
                }
                if (slotp != p) ident = false;
                md.pin_slot |= (uint32_t)slotp << (3 * p);
                if (drv_level_of_net[net] >= (int32_t)L)
                    return fail(ctx, GLS_EINVAL, "instance %u (level %u) reads net %u produced at level %d", i, L, net,
                                drv_level_of_net[net]);
            }
            md.m = (uint8_t)m;
            md.n_pins = cl.n_in;
            md.flags = ident ? kFlagIdent : 0;
            ctx->pins_total += cl.n_in;
            for (int o = 0; o < cl.n_out; ++o) {
                DrvMeta d = md;
                const uint32_t onet = pins[cl.n_in + o];
                if (onet >= nl->n_nets) return fail(ctx, GLS_EINVAL, "instance %u: bad output net", i);
                if (drv_level_of_net[onet] >= 0) return fail(ctx, GLS_EINVAL, "net %u has two drivers", onet);
                drv_level_of_net[onet] = (int32_t)L;
                cell_of_net[onet] = cid;
                d.out_net = onet;
                if (o == 0) d.flags |= kFlagFirstOut;
                auto key = std::make_pair(cid, o);
                auto it = lut_of.find(key);
                if (it == lut_of.end()) {
                    const uint32_t off = (uint32_t)h_lut.size();
                    h_lut.resize(off + (1u << (2 * cl.n_in)));
                    int rc = gls_cell_lut(&cl, nl->prims, o, ctx->opts.calc_mode, h_lut.data() + off,
                                          1u << (2 * cl.n_in));
                    if (rc) return fail(ctx, rc, "cell %u: bad primitive program", cid);
                    it = lut_of.emplace(key, off).first;
                }
                d.lut_off = it->second;
                d.arc_off = (uint32_t)h_arcs.size();
                uint32_t na = 0;
                for (uint32_t a = nl->inst_arc_start[i]; a < nl->inst_arc_start[i + 1]; ++a) {
                    const gls_arc &A = nl->arcs[a];
                    if (A.out_pin != o) continue;
                    if (A.edge > 2) return fail(ctx, GLS_EINVAL, "instance %u: arc edge %u", i, A.edge);
                    if (A.in_pin >= cl.n_in) continue;   // never related: its net is not an input
                    const uint32_t slotp = (md.pin_slot >> (3 * A.in_pin)) & 7u;
                    const double r = A.rise * ctx->opts.delay_factor, f = A.fall * ctx->opts.delay_factor;
                    if (!(r >= 0.0) || !(f >= 0.0) || r >= 4294967295.0 || f >= 4294967295.0)
                        return fail(ctx, GLS_ERANGE, "instance %u: delay out of range", i);
                    ArcDev ad;
                    ad.info = (uint32_t)A.edge | (slotp << 2);
                    ad.rise = (uint32_t)std::min<uint64_t>((uint64_t)r, kMaxDelay);
                    ad.fall = (uint32_t)std::min<uint64_t>((uint64_t)f, kMaxDelay);
                    ad.pad = 0;
                    h_arcs.push_back(ad);
                    ++na;
                }
                if (na > 255) return fail(ctx, GLS_EINVAL, "instance %u: too many arcs", i);
                d.n_arcs = (uint8_t)na;
                // per-net delay table when every net's arcs are regular
                bool regular = true;
                NetDelay nd[kMaxSlots];
                for (int j = 0; j < m; ++j) {
                    uint32_t rf[2][2] = {{kInf, kInf}, {kInf, kInf}};   // [edge][rise/fall]
                    int nboth = 0, npos = 0, nneg = 0;
                    for (uint32_t k = 0; k < na; ++k) {
                        const ArcDev &A = h_arcs[d.arc_off + k];
                        if ((int)(A.info >> 2) != j) continue;
                        const int edge = A.info & 3u;
                        if (edge == 2) {
                            ++nboth;
                            rf[0][0] = rf[1][0] = A.rise;
                            rf[0][1] = rf[1][1] = A.fall;
                        } else {
                            ++(edge == 0 ? npos : nneg);
                            rf[edge][0] = A.rise;
                            rf[edge][1] = A.fall;
                        }
                    }
                    const bool ok = (nboth == 0 && npos == 0 && nneg == 0) || (nboth == 1 && npos == 0 && nneg == 0) ||
                                    (nboth == 0 && npos == 1 && nneg == 1);
                    if (!ok) regular = false;
                    for (int e = 0; e < 2; ++e) {
                        const uint32_t r = rf[e][0], f = rf[e][1];
                        nd[j].d[e * 4 + 0] = r;
                        nd[j].d[e * 4 + 1] = f;
                        nd[j].d[e * 4 + 2] = std::max(r, f);
                        nd[j].d[e * 4 + 3] = std::min(r, f);
                    }
                }
                d.dt_off = (uint32_t)h_ndel.size();
                if (regular) {
                    d.flags |= kFlagRegular;
                    for (int j = 0; j < m; ++j) h_ndel.push_back(nd[j]);
                }
                h_meta.push_back(d);
            }
        }
        // order the level's gate outputs by fan-in class (stable)
        const uint32_t lv0 = ctx->drv_level_start.back();
        std::stable_sort(h_meta.begin() + lv0, h_meta.end(), [](const DrvMeta &x, const DrvMeta &y) {
            return fanin_class(x.m) < fanin_class(y.m);
        });
        uint32_t c0 = 0;
        for (int c = 0; c < kClasses; ++c) {
            ctx->cls_start.push_back(c0);
            while (lv0 + c0 < h_meta.size() && fanin_class(h_meta[lv0 + c0].m) == c) ++c0;
        }
        ctx->cls_start.push_back((uint32_t)(h_meta.size() - lv0));
        ctx->drv_level_start.push_back((uint32_t)h_meta.size());
    }
    ctx->n_nets = nl->n_nets;
    ctx->n_drv = (uint32_t)h_meta.size();
    ctx->max_width = 0;
    for (size_t L = 0; L + 1 < ctx->drv_level_start.size(); ++L)
        ctx->max_width = std::max(ctx->max_width, ctx->drv_level_start[L + 1] - ctx->drv_level_start[L]);
    ctx->driven.assign(nl->n_nets, 0);
    ctx->ext_inputs.clear();
    for (uint32_t n = 0; n < nl->n_nets; ++n) {
        ctx->driven[n] = drv_level_of_net[n] >= 0;
        if (consumed[n] && !ctx->driven[n]) ctx->ext_inputs.push_back(n);
    }
    if (h_arcs.empty()) h_arcs.push_back(ArcDev{0, 0, 0, 0});
    if (h_ndel.empty()) h_ndel.push_back(NetDelay{{kInf, kInf, kInf, kInf, kInf, kInf, kInf, kInf}});
    if (h_lut.empty()) h_lut.push_back(kVX);
    if (h_meta.empty()) h_meta.push_back(DrvMeta{});
    // static presize features per gate output (feature order in gls.h)
    std::vector<float> h_feat(h_meta.size() * kIn, 0.f);
    for (size_t d = 0; d < ctx->n_drv; ++d) {
        const DrvMeta &md = h_meta[d];
        float *f = &h_feat[d * kIn];
        const uint32_t cid = cell_of_net[md.out_net];
        if (cid < 13) f[cid] = 1.f;
        f[13] = md.n_pins / 6.f;
        f[14] = md.m / 6.f;
        double sr = 0, sf = 0;
        uint32_t mn = 0xFFFFFFFFu, mx = 0;
        for (uint32_t k = 0; k < md.n_arcs; ++k) {
            const ArcDev &A = h_arcs[md.arc_off + k];
            sr += A.rise;
            sf += A.fall;
            mn = std::min(mn, std::min(A.rise, A.fall));
            mx = std::max(mx, std::max(A.rise, A.fall));
        }
        const double na = md.n_arcs ? md.n_arcs : 1;
        if (!md.n_arcs) { sr = sf = ctx->def_delay; mn = mx = ctx->def_delay; }
        f[24] = (float)(sr / na / 100.0);
        f[25] = (float)(sf / na / 100.0);
        f[26] = (float)(mn / 100.0);
        f[27] = (float)(mx / 100.0);
        f[28] = (float)(std::log1p((double)fanout[md.out_net]) / 6.0);
        // share of single-input changes (0 <-> 1) that change the output
        const uint8_t *lut = &h_lut[md.lut_off];
        uint32_t changes = 0, trials = 0;
        for (uint32_t c = 0; c < (1u << md.n_pins); ++c) {
            uint32_t idx = 0;
            for (int p = 0; p < md.n_pins; ++p) idx |= (((c >> p) & 1u) ? 3u : 0u) << (2 * p);
            for (int p = 0; p < md.n_pins; ++p) {
                changes += lut[idx] != lut[idx ^ (3u << (2 * p))];
                ++trials;
            }
        }
        f[29] = trials ? (float)changes / trials : 0.f;
        f[30] = (md.flags & kFlagRegular) ? 1.f : 0.f;
        f[31] = 1.f;
    }
    // per gate output with at most 3 input nets: its truth table indexed by
    // the input nets' values (what the gate kernels keep in registers)
    std::vector<uint4> h_slut(h_meta.size(), make_uint4(0, 0, 0, 0));
    for (size_t d = 0; d < ctx->n_drv; ++d) {
        const DrvMeta &md = h_meta[d];
        if (md.m > 3) continue;
        uint32_t words[4] = {0, 0, 0, 0};
        const uint32_t entries = 1u << (2 * std::max<int>(md.m, 1));
        for (uint32_t x = 0; x < entries; ++x) {
            uint32_t idx = 0;
            for (int p = 0; p < md.n_pins; ++p)
                idx |= ((x >> (2 * ((md.pin_slot >> (3 * p)) & 7u))) & 3u) << (2 * p);
            words[x >> 4] |= (uint32_t)(h_lut[md.lut_off + idx] & 3u) << (2 * (x & 15u));
        }
        h_slut[d] = make_uint4(words[0], words[1], words[2], words[3]);
    }
    CK(ctx->slut.ensure(h_slut.size() * sizeof(uint4)), "alloc slot truth tables");
    CK(cudaMemcpy(ctx->slut.p, h_slut.data(), h_slut.size() * sizeof(uint4), cudaMemcpyHostToDevice),
       "upload slot truth tables");
    CK(ctx->feat_static.ensure(h_feat.size() * 4), "alloc presize features");
    CK(cudaMemcpy(ctx->feat_static.p, h_feat.data(), h_feat.size() * 4, cudaMemcpyHostToDevice),
       "upload presize features");
    CK(ctx->meta.ensure(h_meta.size() * sizeof(DrvMeta)), "alloc meta");
    CK(ctx->arcs.ensure(h_arcs.size() * sizeof(ArcDev)), "alloc arcs");
    CK(ctx->ndel.ensure(h_ndel.size() * sizeof(NetDelay)), "alloc net delays");
    CK(ctx->lut.ensure(h_lut.size()), "alloc lut");
    CK(cudaMemcpy(ctx->meta.p, h_meta.data(), h_meta.size() * sizeof(DrvMeta), cudaMemcpyHostToDevice), "upload meta");
    CK(cudaMemcpy(ctx->arcs.p, h_arcs.data(), h_arcs.size() * sizeof(ArcDev), cudaMemcpyHostToDevice), "upload arcs");
    CK(cudaMemcpy(ctx->ndel.p, h_ndel.data(), h_ndel.size() * sizeof(NetDelay), cudaMemcpyHostToDevice),
       "upload net delays");
    CK(cudaMemcpy(ctx->lut.p, h_lut.data(), h_lut.size(), cudaMemcpyHostToDevice), "upload lut");
    ctx_drop_graphs(ctx);   // they hold the previous netlist's tables
    free_spares(ctx);
    ctx->seg_cap = std::max<uint32_t>(1u << 21, 8 * ctx->max_width + 64);
    if (ctx->lsc.empty()) ctx->lsc.push_back(new LevelScratch);
    for (LevelScratch *l : ctx->lsc) l->release();
    CK(ctx->lsc[0]->ensure(ctx->max_width, ctx->seg_cap, ctx->scr_cap), "alloc level work space");
    ctx->loaded = true;
    return GLS_OK;
}

// mean stimulus list length x input pins: what the gate-output pool scales with
static double pool_scale(const gls_ctx *ctx, const Window *w)
{
    const double avg = w->stim_nets.empty() ? 4.0 : (double)w->stim_events / (double)w->stim_nets.size();
    return avg * (double)ctx->pins_total;
}

// the pool a window is given: its estimate, raised to what earlier windows
// of this netlist needed (unless the caller fixed the size)
static uint64_t projected_cap(const gls_ctx *ctx, const Window *w)
{
    uint64_t cap = w->cap;
    if (!ctx->opts.pool_events && ctx->pool_ratio > 0.0) {
        const uint64_t need = w->stim_events + ctx->pool_gap + 8ull * ctx->n_drv + 1024 +
                              (uint64_t)(1.1 * ctx->pool_ratio * pool_scale(ctx, w));
        cap = std::max(cap, need);
    }
    return cap;
}

// Device buffers of a window filled from its host staging.  Without `sync`
// the copies only precede later work on the context's stream.
static int upload_window(gls_ctx *ctx, Window *w, bool sync = true)
{
    const uint64_t n = ctx->n_nets;
    w->cap = std::max(w->cap, projected_cap(ctx, w));
    const uint64_t wb = w->word_bytes();
    if (w->pool.p && w->pool.bytes < w->cap * wb) w->pool.release();
    CK(take_buf(ctx, w->pool, w->cap * wb), "alloc event pool");
    CK(take_buf(ctx, w->net_off, n * 8), "alloc net_off");
    CK(w->net_len.ensure(n * 4), "alloc net_len");
    CK(take_buf(ctx, w->init_off, n * 8), "alloc init_off");
    CK(take_buf(ctx, w->init_len, n * 4), "alloc init_len");
    CK(w->saif.ensure(n * 24), "alloc saif");
    CK(w->small.ensure(256), "alloc counters");
    CK(take_buf(ctx, w->stim_dev, w->stim_nets.size() * 4 + 16), "alloc stim nets");
    if (w->stim_events)
        CK(cudaMemcpyAsync(w->pool.p, w->h_words.p, w->stim_events * wb, cudaMemcpyHostToDevice, ctx->stream),
           "upload stimulus");
    if (!w->h_off.ensure(n * 8) || !w->h_len.ensure(n * 4)) return fail(ctx, GLS_ENOMEM, "pinned staging");
    uint64_t *off = w->h_off.as<uint64_t>();
    uint32_t *len = w->h_len.as<uint32_t>();
    std::memset(off, 0, n * 8);
    std::memset(len, 0xFF, n * 4);
    for (size_t k = 0; k < w->stim_nets.size(); ++k) {
        off[w->stim_nets[k]] = w->stim_off[k];
        len[w->stim_nets[k]] = w->stim_len[k];
    }
    CK(cudaMemcpyAsync(w->init_off.p, off, n * 8, cudaMemcpyHostToDevice, ctx->stream), "upload offsets");
    CK(cudaMemcpyAsync(w->init_len.p, len, n * 4, cudaMemcpyHostToDevice, ctx->stream), "upload lengths");
    if (!w->stim_nets.empty())
        CK(cudaMemcpyAsync(w->stim_dev.p, w->stim_nets.data(), w->stim_nets.size() * 4, cudaMemcpyHostToDevice,
                           ctx->stream),
           "upload stim nets");
    if (sync) CK(cudaStreamSynchronize(ctx->stream), "upload sync");
    w->uploaded = true;
    return GLS_OK;
}

extern "C" int gls_add_window(gls_ctx *ctx, const gls_stimulus *st, uint64_t t_begin, uint64_t t_end,
                              uint32_t *window_id)
{
    if (!ctx || !st) return GLS_EINVAL;
    if (!ctx->loaded) return fail(ctx, GLS_ESTATE, "add_window before load_netlist");
    if (t_end <= t_begin) return fail(ctx, GLS_EINVAL, "window end %llu must exceed begin %llu",
                                      (unsigned long long)t_end, (unsigned long long)t_begin);
    if (st->n_nets && (!st->net || !st->ev_start || !st->time || !st->value))
        return fail(ctx, GLS_EINVAL, "stimulus: null array");
    cudaSetDevice(ctx->opts.device);
    Window *w;
    if (!ctx->spare.empty()) {
        w = ctx->spare.back();
        ctx->spare.pop_back();
    } else {
        w = new Window();
    }
    w->done = false;
    w->w64 = false;
    w->t_begin = t_begin;
    w->t_end = t_end;
    std::vector<uint8_t> seen(ctx->n_nets, 0);
    std::vector<uint64_t> at(st->n_nets + 1, 0);
    for (uint32_t k = 0; k < st->n_nets; ++k) {
        const uint32_t net = st->net[k];
        if (net >= ctx->n_nets) { ctx->spare.push_back(w); return fail(ctx, GLS_EINVAL, "stimulus net %u out of range", net); }
        if (seen[net]) { ctx->spare.push_back(w); return fail(ctx, GLS_EINVAL, "stimulus net %u given twice", net); }
        if (ctx->driven[net]) { ctx->spare.push_back(w); return fail(ctx, GLS_EINVAL, "stimulus net %u is driven by a gate", net); }
        seen[net] = 1;
        if (st->ev_start[k + 1] < st->ev_start[k]) { ctx->spare.push_back(w); return fail(ctx, GLS_EINVAL, "stimulus ev_start not monotone"); }
        at[k + 1] = at[k] + round4(st->ev_start[k + 1] - st->ev_start[k]);
    }
    for (uint32_t net : ctx->ext_inputs)
        if (!seen[net]) { ctx->spare.push_back(w); return fail(ctx, GLS_EINVAL, "net %u is read by a gate but has no stimulus", net); }
    const uint64_t total = at[st->n_nets];
    if (!w->h_words.ensure(total * 4)) {
        ctx->spare.push_back(w);
        return fail(ctx, GLS_ENOMEM, "pinned staging of %llu events", (unsigned long long)total);
    }
    // validate and pack (time << 2 | value), each net on a 4-event boundary;
    // large stimuli are packed by several host threads.  32-bit words hold
    // times up to 2^30 - 2; a later time repacks the stimulus in 64-bit words.
    std::atomic<int> bad(0);
    std::atomic<uint32_t> bad_net(0);
    std::atomic<bool> long_times(false);
    // The loops carry no early exit so that the compiler vectorizes them; a
    // net's faults are reported in the order value, time range, time order.
    auto pack = [&](auto *hw, uint32_t k0, uint32_t k1) {
        using Wd = typename std::remove_pointer<decltype(hw)>::type;
        for (uint32_t k = k0; k < k1; ++k) {
            const uint64_t a = st->ev_start[k], cnt = st->ev_start[k + 1] - a;
            const uint32_t *tt = st->time + a;
            const uint8_t *vv = st->value + a;
            Wd *o = hw + at[k];
            uint32_t ev = 0, et = 0, ew = 0, eo = 0;
            if (cnt) {   // one pass over the times: the order check reads the word before from cache
                ev |= vv[0] > 3 ? 1u : 0u;
                ew |= tt[0] > kMaxTime ? 1u : 0u;
                et |= tt[0] > kMaxTimeWide ? 1u : 0u;
                o[0] = ((Wd)tt[0] << 2) | (Wd)(vv[0] & 3u);
            }
            for (uint64_t e = 1; e < cnt; ++e) {
                const uint32_t t = tt[e], v = vv[e];
                ev |= v > 3 ? 1u : 0u;
                ew |= t > kMaxTime ? 1u : 0u;
                et |= t > kMaxTimeWide ? 1u : 0u;
                eo |= t <= tt[e - 1] ? 1u : 0u;
                o[e] = ((Wd)t << 2) | (Wd)(v & 3u);
            }
            for (uint64_t e = cnt; e < round4(cnt); ++e) o[e] = EvW<Wd>::kInfW;
            if (ew) long_times = true;
            if (ev | et | eo) {
                bad = ev ? 1 : (et ? 2 : 3);
                bad_net = st->net[k];
                return;
            }
        }
    };
    const unsigned hc = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (total > (1u << 20) && hc > 1 && st->n_nets > 4 * hc && !ctx->pool) {
        try {
            ctx->pool = new WorkPool(hc - 1);
        } catch (...) {   // no threads to be had: pack on this one
            ctx->pool = nullptr;
        }
    }
    if (total > (1u << 20) && ctx->pool && st->n_nets > 4 * ctx->pool->threads()) {
        // parts of about equal event counts: part q starts at the first net
        // whose packed offset reaches q * total / parts
        const unsigned parts = 4 * ctx->pool->threads();
        std::vector<uint32_t> first(parts + 1, st->n_nets);
        for (unsigned q = 0; q < parts; ++q)
            first[q] = (uint32_t)(std::lower_bound(at.begin(), at.end() - 1, total * q / parts) - at.begin());
        ctx->pool->parallel_for(parts, [&](unsigned q) {
            pack(w->h_words.as<uint32_t>(), first[q], std::max(first[q], first[q + 1]));
        });
    } else {
        pack(w->h_words.as<uint32_t>(), 0, st->n_nets);
    }
    if (!bad && long_times) {
        if (!w->h_words.ensure(total * 8)) {
            ctx->spare.push_back(w);
            return fail(ctx, GLS_ENOMEM, "pinned staging of %llu events", (unsigned long long)total);
        }
        w->w64 = true;
        pack(w->h_words.as<WideWord>(), 0, st->n_nets);
    }
    if (bad) {
        ctx->spare.push_back(w);
        const int b = bad;
        return fail(ctx, b == 2 ? GLS_ERANGE : GLS_EINVAL, "stimulus net %u: %s", (unsigned)bad_net,
                    b == 1 ? "value above 3" : b == 2 ? "time beyond the largest event time (2^32-2)"
                                             : "times not strictly increasing");
    }
    w->stim_nets.assign(st->net, st->net + st->n_nets);
    w->stim_off.assign(at.begin(), at.end() - 1);
    w->stim_len.resize(st->n_nets);
    for (uint32_t k = 0; k < st->n_nets; ++k) w->stim_len[k] = (uint32_t)(st->ev_start[k + 1] - st->ev_start[k]);
    w->stim_events = total;
    // initial pool capacity: stimulus plus an estimate of every gate's slot
    uint64_t cap = ctx->opts.pool_events;
    if (!cap) {
        // gate outputs take about as many events as one input on average; an
        // upper-bound slot reserves the sum over the inputs
        const double avg = st->n_nets ? (double)total / st->n_nets : 4.0;
        const double f = ctx->opts.alloc_mode == GLS_ALLOC_BOUND ? 2.5 : 1.3;
        cap = total + (uint64_t)(f * avg * (double)ctx->pins_total) + 8ull * ctx->n_drv + 1024;
        size_t fr = 0, tot = 0;
        // a reused window that already holds this much needs no limit
        if (cap + ctx->pool_gap > w->cap && cudaMemGetInfo(&fr, &tot) == cudaSuccess) {
            const uint64_t limit = (uint64_t)(fr * 0.6) / 5;
            if (cap > limit) cap = std::max<uint64_t>(limit, total + 1024);
        }
    }
    w->cap = std::max<uint64_t>(std::max<uint64_t>(cap, total + 1024) + ctx->pool_gap, w->cap);
    // level scratch: the widest level's fan-in events, estimated from the stimulus
    {
        const double avg = st->n_nets ? (double)total / st->n_nets : 4.0;
        const double fan = std::max(1.0, (double)ctx->pins_total / std::max<uint32_t>(1, ctx->n_drv));
        uint64_t want = (uint64_t)(2.0 * avg * fan * ctx->max_width) + 16ull * ctx->max_width + 4096;
        if (want > ctx->scr_cap) {
            ctx->scr_cap = want;
            CK(ctx->lsc[0]->ensure(ctx->max_width, ctx->seg_cap, ctx->scr_cap), "alloc level scratch");
        }
    }
    // device buffers are filled when the window first runs
    w->uploaded = false;
    w->saif_only = false;
    ctx->windows.push_back(w);
    if (window_id) *window_id = (uint32_t)(ctx->windows.size() - 1);
    return GLS_OK;
}

// parity 1: the per-gate-output tables of odd levels
static WinDev make_windev(gls_ctx *ctx, Window *w, const LevelScratch &ls, int parity = 0)
{
    WinDev d;
    std::memset(&d, 0, sizeof d);
    d.net_off = w->net_off.as<uint64_t>();
    d.net_len = w->net_len.as<uint32_t>();
    d.pool = w->pool.as<uint32_t>();
    d.saif = w->saif.as<unsigned long long>();
    unsigned long long *sm = w->small.as<unsigned long long>();
    d.top = sm;
    d.counters = sm + 1;     // 4 counters
    d.err = reinterpret_cast<uint32_t *>(sm + 5);
    d.n_segs = reinterpret_cast<uint32_t *>(sm + 6);
    d.n_over = sm + 7;
    d.res = (parity ? ls.res1 : ls.res).as<uint32_t>();
    d.pred = ls.pred.as<uint32_t>();
    d.stim_nets = w->stim_dev.as<uint32_t>();
    d.n_stim = (uint32_t)w->stim_nets.size();
    d.seg_base = (parity ? ls.seg_base1 : ls.seg_base).as<uint32_t>();
    d.slot = (parity ? ls.slot1 : ls.slot).as<uint64_t>();
    d.scr = (parity ? ls.scr1 : ls.scr).as<uint64_t>();
    d.segs = ls.segs.as<SegRec>();   // SegRecT<WideWord> records in a window of 64-bit words
    d.copies = ls.copies.as<CopyRec>();
    d.scratch = ls.scratch.as<uint32_t>();
    d.scr_cap = ls.scr_cap * 4 / w->word_bytes();   // the stacks are sized in 32-bit words
    d.cap = w->cap;
    d.seg_cap = ls.seg_cap;
    d.t_begin = w->t_begin;
    d.t_end = w->t_end;
    return d;
}

// profiling: events recorded between kernel launches (opts.profile)
static cudaEvent_t prof_event(gls_ctx *ctx)
{
    if (ctx->prof_used == ctx->prof.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ctx->prof.push_back(e);
    }
    return ctx->prof[ctx->prof_used++];
}

static void prof_mark(gls_ctx *ctx)
{
    if (!ctx->opts.profile) return;
    cudaEvent_t e = prof_event(ctx);
    if (e) cudaEventRecord(e, ctx->stream);
}

// Clear a window's outputs and counters before it runs.
static int reset_window(gls_ctx *ctx, Window *w)
{
    const uint64_t n = ctx->n_nets;
    CK(cudaMemcpyAsync(w->net_off.p, w->init_off.p, n * 8, cudaMemcpyDeviceToDevice, ctx->stream), "reset offsets");
    CK(cudaMemcpyAsync(w->net_len.p, w->init_len.p, n * 4, cudaMemcpyDeviceToDevice, ctx->stream), "reset lengths");
    CK(cudaMemsetAsync(w->saif.p, 0xFF, n * 24, ctx->stream), "reset saif");
    unsigned long long small[8] = {w->stim_events + ctx->pool_gap, 0, 0, 0, 0, 0, 0, 0};
    CK(cudaMemcpyAsync(w->small.p, small, sizeof small, cudaMemcpyHostToDevice, ctx->stream), "reset counters");
    return GLS_OK;
}

// The launches of a run of nwin windows: stimulus SAIF, then per level the
// presize (learned mode), plan, simulate per fan-in class, link and copy.
// dw[p] / h[p] are the descriptors (device array / window 0 on the host)
// whose per-gate-output tables serve levels of parity p.  With `prof` the
// kernel classes are bracketed with events (not during stream capture).
static int enqueue_levels(gls_ctx *ctx, const WinDev *const dw[2], const WinDev *const h[2], uint32_t nwin,
                          uint32_t max_stim, bool prof, uint32_t *launches, bool w64 = false)
{
    LevelArgs a;
    ctx_level_args(ctx, &a);
    if (w64) {   // a window of 64-bit words runs alone, through the thread-per-segment kernels
        if (nwin != 1) return fail(ctx, GLS_EINVAL, "64-bit event windows run one at a time");
        a.wide = 1;
        a.warp_mask = 0;
        a.sim_variant = 0;
    }
    // Overlapped levels: every class runs simulate, link and copy on its own
    // stream; the main stream plans the next level as soon as every class
    // has linked (the plan needs the new lists' lengths and places, and
    // writes the other set of per-gate-output tables), while the copies
    // still run; a class's next simulation waits for every class's copy.
    // Learned mode splits the plan: the presize reads SAIF counts that the
    // copies add, so the segments and stacks are planned beside the copies,
    // and only the presize and the slot placement run between the copies
    // and the next level's simulations.  (The learned balance sizes segments
    // from the predictions: it keeps the plan whole, after the copies.)
    const bool learned = a.alloc_mode == kAllocLearned;
    const bool split = learned && ctx->bal_weight <= 0.f;
    const bool overlap_ok = ctx->concurrent && ctx->pipeline && ctx->plan_overlap && !(prof && ctx->opts.profile) &&
                            (!learned || split);
    if (prof) prof_mark(ctx);
    if (overlap_ok && !learned) {
        // the stimulus nets' SAIF beside the levels (nothing else reads or
        // writes their counts; learned mode's presize reads them)
        CK(cudaEventRecord(ctx->stim_fork, ctx->stream), "stim fork");
        CK(cudaStreamWaitEvent(ctx->stim_side, ctx->stim_fork, 0), "stim fork wait");
        launch_stim_saif(dw[0], *h[0], nwin, max_stim, w64, ctx->stim_side);
        CK(cudaEventRecord(ctx->stim_join, ctx->stim_side), "stim join");
    } else {
        launch_stim_saif(dw[0], *h[0], nwin, max_stim, w64, ctx->stream);
    }
    ++*launches;
    if (prof) prof_mark(ctx);
    const size_t nlev = ctx->drv_level_start.size() - 1;
    if (nwin > 1) {
        // per level, the wave's fan-in events per class: segments are cut to
        // one size across the windows of the wave
        CK(ctx->wave_e.ensure(nlev * kClasses * 8 + 8), "alloc wave totals");
        CK(cudaMemsetAsync(ctx->wave_e.p, 0, nlev * kClasses * 8, ctx->stream), "clear wave totals");
    }
    bool copied[kClasses] = {false, false, false, false};   // the class copied at the previous level
    for (size_t L = 0; L < nlev; ++L) {
        a.lo = ctx->drv_level_start[L];
        a.hi = ctx->drv_level_start[L + 1];
        if (a.hi == a.lo) continue;
        const WinDev *dwL = dw[L & 1];
        const WinDev &hL = *h[L & 1];
        a.wave_e = nwin > 1 ? ctx->wave_e.as<unsigned long long>() + L * kClasses : nullptr;
        if (nwin > 1) {
            launch_wave_events(dwL, nwin, a, ctx->stream);
            ++*launches;
        }
        int n_cls = 0;
        for (int c = 0; c < kClasses; ++c)
            n_cls += ctx->cls_start[(kClasses + 1) * L + c + 1] > ctx->cls_start[(kClasses + 1) * L + c];
        const bool overlap = overlap_ok && n_cls > 0;
        const bool split_level = learned && overlap;
        auto presize = [&]() {   // the level's presize predictions (tensor cores), before its slots are placed
            PresizeArgs pa;
            ctx_presize_args(ctx, &pa);
            pa.wv = dwL;
            pa.nwin = nwin;
            pa.lo = a.lo;
            pa.n = a.hi - a.lo;
            launch_presize(pa, true, ctx->stream);
            ++*launches;
        };
        if (learned && !split_level) presize();
        a.plan_part = split_level ? 1u : 0u;
        launch_plan(dwL, hL, nwin, a, ctx->stream);
        a.plan_part = 0;
        if (prof) prof_mark(ctx);
        // Concurrent: the fan-in classes simulate on their own streams, so
        // one class's blocks fill another's tail (linking and copying every
        // class together after the join measured faster than per class).
        // Profiled runs keep the classes apart.
        const bool fork = overlap || (ctx->concurrent && !(prof && ctx->opts.profile) && n_cls > 1);
        if (fork) CK(cudaEventRecord(ctx->fork_ev, ctx->stream), "fork");
        if (overlap) {
            // every class stream waits for the plan and for every class's
            // copy of the previous level, before any class records anew
            for (int c = 0; c < kClasses; ++c) {
                if (ctx->cls_start[(kClasses + 1) * L + c + 1] <= ctx->cls_start[(kClasses + 1) * L + c]) continue;
                cudaStream_t st = ctx->class_priority ? ctx->side_prio[c] : ctx->side[c];
                CK(cudaStreamWaitEvent(st, ctx->fork_ev, 0), "fork wait");
                for (int c2 = 0; c2 < kClasses; ++c2)
                    if (copied[c2]) CK(cudaStreamWaitEvent(st, ctx->copy_ev[c2], 0), "copy wait");
            }
        }
        if (split_level) {
            // the presize and the slots after the previous level's copies
            // (the main stream has waited for the links only)
            for (int c2 = 0; c2 < kClasses; ++c2)
                if (copied[c2]) CK(cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[c2], 0), "copy wait");
            presize();
            a.plan_part = 2;
            launch_plan(dwL, hL, nwin, a, ctx->stream);
            a.plan_part = 0;
            ++*launches;
            CK(cudaEventRecord(ctx->slots_ev, ctx->stream), "slots placed");
        }
        bool first = true;
        bool linked[kClasses] = {false, false, false, false};
        for (int ci = 0; ci < kClasses; ++ci) {
            // wider gates first when the classes run together: they carry
            // the most events per gate, so their chain sets the level's length
            const int c = (fork && ctx->wide_first) ? kClasses - 1 - ci : ci;
            const uint32_t d0 = ctx->cls_start[(kClasses + 1) * L + c], d1 = ctx->cls_start[(kClasses + 1) * L + c + 1];
            if (d1 <= d0) continue;
            // the first class on the main stream, the others beside it
            // (overlapped: every class beside it)
            cudaStream_t st = ctx->stream;
            if (overlap) {
                st = ctx->class_priority ? ctx->side_prio[c] : ctx->side[c];
            } else if (fork && (!first || ctx->class_priority)) {
                st = ctx->class_priority ? ctx->side_prio[c] : ctx->side[c];
                CK(cudaStreamWaitEvent(st, ctx->fork_ev, 0), "fork wait");
            }
            // the gate kernels fill every SM until their last segment: the
            // presize and the slots go first, else they would wait for them
            if (split_level) CK(cudaStreamWaitEvent(st, ctx->slots_ev, 0), "slots wait");
            launch_sim(dwL, hL, nwin, a, c, d0, d1, ctx->sm_count, st);
            ++*launches;
            if (fork && ctx->pipeline) {   // the class's link and copy right behind it
                launch_link(dwL, hL, nwin, a, d0, d1, st);
                if (overlap) {
                    CK(cudaEventRecord(ctx->link_ev[c], st), "link done");
                    linked[c] = true;
                }
                launch_copy(dwL, hL, nwin, a, d0, d1, ctx->sm_count, st);
                if (overlap) CK(cudaEventRecord(ctx->copy_ev[c], st), "copy done");
                *launches += 2;
            }
            if (st != ctx->stream && !overlap) {
                CK(cudaEventRecord(ctx->join_ev[c], st), "join");
                CK(cudaStreamWaitEvent(ctx->stream, ctx->join_ev[c], 0), "join wait");
            }
            first = false;
        }
        if (overlap) {
            // the next plan waits for the links only
            for (int c = 0; c < kClasses; ++c) {
                if (linked[c]) CK(cudaStreamWaitEvent(ctx->stream, ctx->link_ev[c], 0), "link wait");
                copied[c] = linked[c];
            }
        } else {
            // this level's kernels are all on or joined to the main stream
            for (int c = 0; c < kClasses; ++c) copied[c] = false;
        }
        if (prof) prof_mark(ctx);
        if (!(fork && ctx->pipeline)) {
            launch_link(dwL, hL, nwin, a, 0, a.hi - a.lo, ctx->stream);
            launch_copy(dwL, hL, nwin, a, 0, a.hi - a.lo, ctx->sm_count, ctx->stream);
            *launches += 2;
        }
        if (prof) prof_mark(ctx);
        ++*launches;   // the plan
    }
    // the last level's copies and the stimulus SAIF join the main stream
    for (int c = 0; c < kClasses; ++c)
        if (copied[c]) CK(cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[c], 0), "final join");
    if (overlap_ok && !learned) CK(cudaStreamWaitEvent(ctx->stream, ctx->stim_join, 0), "stim join wait");
    CK(cudaGetLastError(), "kernel launch");
    return GLS_OK;
}

static int enqueue_window(gls_ctx *ctx, Window *w, uint32_t *launches)
{
    int rc = w->uploaded ? GLS_OK : upload_window(ctx, w);
    if (rc) return rc;
    w->saif_only = false;
    rc = reset_window(ctx, w);
    if (rc) return rc;
    const WinDev d[2] = {make_windev(ctx, w, *ctx->lsc[0], 0), make_windev(ctx, w, *ctx->lsc[0], 1)};
    CK(w->dwin.ensure(sizeof d), "alloc window descriptor");
    CK(cudaMemcpyAsync(w->dwin.p, d, sizeof d, cudaMemcpyHostToDevice, ctx->stream), "upload window descriptor");
    const WinDev *dw[2] = {w->dwin.as<WinDev>(), w->dwin.as<WinDev>() + 1};
    const WinDev *hp[2] = {&d[0], &d[1]};
    return enqueue_levels(ctx, dw, hp, 1, d[0].n_stim, true, launches, w->w64);
}

// Totals of a run over its windows.
struct RunAcc {
    uint64_t gate_ev = 0, out_ev = 0, segs = 0, pool_ev = 0, pool_bytes = 0, fanin_ev = 0, over_ev = 0, wide = 0;
    double total_ms = 0.0;
    uint32_t launches = 0;
};

// The window's stimulus repacked in 64-bit event words and uploaded again.
static int widen_window(gls_ctx *ctx, Window *w)
{
    const uint64_t n = w->stim_events;
    std::vector<uint32_t> narrow(w->h_words.as<uint32_t>(), w->h_words.as<uint32_t>() + n);
    if (!w->h_words.ensure(n * 8)) return fail(ctx, GLS_ENOMEM, "pinned staging of %llu events", (unsigned long long)n);
    WideWord *o = w->h_words.as<WideWord>();
    for (uint64_t e = 0; e < n; ++e)
        o[e] = narrow[e] == kInf ? EvW<WideWord>::kInfW : (WideWord)narrow[e];
    w->w64 = true;
    w->pool.release();
    return upload_window(ctx, w);
}

// Read a window's flags after its run; on a full pool or work space, grow it
// and run the window again on its own (level work space 0), until it fits.
static int settle_window(gls_ctx *ctx, Window *w, RunAcc &acc)
{
    for (int attempt = 0;; ++attempt) {
        unsigned long long small[8];
        CK(cudaMemcpy(small, w->small.p, sizeof small, cudaMemcpyDeviceToHost), "read status");
        const uint32_t err = (uint32_t)small[5];
        if (!err) {
            const double sc = pool_scale(ctx, w);
            if (sc > 0.0 && small[0] > w->stim_events + ctx->pool_gap)
                ctx->pool_ratio = std::max(ctx->pool_ratio,
                                           (double)(small[0] - w->stim_events - ctx->pool_gap) / sc);
            acc.over_ev += small[7];
            acc.gate_ev += small[1];
            acc.out_ev += small[2];
            acc.segs += small[3];
            acc.fanin_ev += small[4];
            acc.pool_ev += small[0];
            acc.pool_bytes += w->cap * w->word_bytes();
            acc.wide += w->w64 ? 1 : 0;
            break;
        }
        if (err & kErrPresize) return fail(ctx, GLS_ECUDA, "presize kernel timed out waiting for its tensor-core MMA");
        if ((err & kErrTime) && !w->w64) {
            // a gate output past 2^30 - 2: the window again in 64-bit words
            int rc = widen_window(ctx, w);
            if (rc) return rc;
        } else if (err & (kErrRegion | kErrEmptied | kErrTime)) {
            return fail(ctx, err & kErrTime ? GLS_ERANGE : GLS_EINVAL,
                        "simulation error flags 0x%x (%s)", err,
                        err & kErrTime ? "output time beyond the largest event time (2^32-2)"
                                       : err & kErrEmptied ? "output list emptied by a zero delay at time 0"
                                                           : "segment region overflow");
        }
        if (attempt > 12) return fail(ctx, GLS_EOVERFLOW, "event pool could not grow enough");
        if (err & kErrSegCap) ctx->seg_cap = std::max<uint32_t>(ctx->seg_cap, ctx->lsc[0]->seg_cap) * 2;
        if (err & kErrScratch) ctx->scr_cap = std::max<uint64_t>(ctx->scr_cap, ctx->lsc[0]->scr_cap) * 2;
        {
            const cudaError_t e = ctx->lsc[0]->ensure(ctx->max_width, ctx->seg_cap, ctx->scr_cap);
            if (e != cudaSuccess)
                return fail(ctx, GLS_ENOMEM, "grow level work space to %llu stack words / %u segments (flags 0x%x): %s",
                            (unsigned long long)ctx->scr_cap, ctx->seg_cap, err, cudaGetErrorString(e));
        }
        if ((err & kErrPool) && !(err & kErrTime)) {
            w->cap *= 2;
            w->pool.release();
            int rc = upload_window(ctx, w);
            if (rc) return fail(ctx, GLS_EOVERFLOW, "event pool growth to %llu events failed: %s",
                                (unsigned long long)w->cap, ctx->err.c_str());
            ctx->stats.overflow_retries++;
        }
        uint32_t l2 = 0;
        ctx->prof_used = 0;   // per-kernel times then cover the successful run only
        CK(cudaEventRecord(ctx->ev0, ctx->stream), "event");
        int rc = enqueue_window(ctx, w, &l2);
        if (rc) return rc;
        CK(cudaEventRecord(ctx->ev1, ctx->stream), "event");
        CK(cudaStreamSynchronize(ctx->stream), "rerun");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        acc.total_ms += ms;
        acc.launches += l2;
    }
    w->done = true;
    return GLS_OK;
}

static void publish_stats(gls_ctx *ctx, const RunAcc &acc, const double kms[4])
{
    ctx->stats.gate_events = acc.gate_ev;
    ctx->stats.output_events = acc.out_ev;
    ctx->stats.segments = acc.segs;
    ctx->stats.pool_events = acc.pool_ev;
    ctx->stats.pool_bytes = acc.pool_bytes;
    ctx->stats.kernel_ms = acc.total_ms;
    ctx->stats.launches = acc.launches;
    ctx->stats.n_windows = (uint32_t)ctx->windows.size();
    ctx->stats.stim_ms = kms[0];
    ctx->stats.plan_ms = kms[1];
    ctx->stats.sim_ms = kms[2];
    ctx->stats.combine_ms = kms[3];
    ctx->stats.fanin_bytes = acc.fanin_ev * 5;
    ctx->stats.presize_overflows = acc.over_ev;
    ctx->stats.pool_used = acc.pool_ev;
    ctx->stats.wide_windows = acc.wide;
}

extern "C" int gls_run(gls_ctx *ctx)
{
    if (!ctx) return GLS_EINVAL;
    if (!ctx->loaded) return fail(ctx, GLS_ESTATE, "run before load_netlist");
    if (ctx->opts.alloc_mode == GLS_ALLOC_LEARNED && !ctx->have_model)
        return fail(ctx, GLS_ESTATE, "GLS_ALLOC_LEARNED needs gls_set_presize_model before gls_run");
    cudaSetDevice(ctx->opts.device);
    uint32_t launches = 0;
    ctx->prof_used = 0;
    CK(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    for (Window *w : ctx->windows) {
        int rc = enqueue_window(ctx, w, &launches);
        if (rc) return rc;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    CK(cudaStreamSynchronize(ctx->stream), "run");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    double total_ms = ms;
    double kms[4] = {0, 0, 0, 0};   // stim, plan, sim, combine
    if (ctx->opts.profile) {
        // per window: [stim start, stim end, then per level: after plan, after sim, after combine]
        size_t k = 0;
        const size_t nlev = ctx->drv_level_start.size() - 1;
        for (size_t wi = 0; wi < ctx->windows.size() && k + 1 < ctx->prof_used; ++wi) {
            float x = 0.f;
            cudaEventElapsedTime(&x, ctx->prof[k], ctx->prof[k + 1]);
            kms[0] += x;
            cudaEvent_t prev = ctx->prof[k + 1];
            k += 2;
            for (size_t L = 0; L < nlev; ++L) {
                if (ctx->drv_level_start[L + 1] == ctx->drv_level_start[L]) continue;
                if (k + 2 >= ctx->prof_used) break;
                cudaEventElapsedTime(&x, prev, ctx->prof[k]); kms[1] += x;
                cudaEventElapsedTime(&x, ctx->prof[k], ctx->prof[k + 1]); kms[2] += x;
                cudaEventElapsedTime(&x, ctx->prof[k + 1], ctx->prof[k + 2]); kms[3] += x;
                prev = ctx->prof[k + 2];
                k += 3;
            }
        }
    }
    RunAcc acc;
    acc.total_ms = total_ms;
    acc.launches = launches;
    for (Window *w : ctx->windows) {
        int rc = settle_window(ctx, w, acc);
        if (rc) return rc;
    }
    publish_stats(ctx, acc, kms);
    return GLS_OK;
}

static void apply_schedule(gls_ctx *ctx, uint32_t seg_per_sm, uint32_t warp_mask, uint32_t flags)
{
    ctx->seg_per_sm = seg_per_sm;
    ctx->warp_mask = warp_mask;
    ctx->class_priority = flags & GLS_SCHED_CLASS_PRIORITY;
    ctx->sim_variant = ((flags & GLS_SCHED_BLOCK256) ? 1u : 0u) | ((flags & GLS_SCHED_WIDE_LOADS) ? 2u : 0u);
    ctx->bal_weight = (flags & GLS_SCHED_LEARNED_BALANCE) ? ctx->bal_weight_on : 0.f;
}

static uint32_t schedule_flags(const gls_ctx *ctx)
{
    return (ctx->class_priority ? GLS_SCHED_CLASS_PRIORITY : 0u) | ((ctx->sim_variant & 1u) ? GLS_SCHED_BLOCK256 : 0u) |
           ((ctx->sim_variant & 2u) ? GLS_SCHED_WIDE_LOADS : 0u) | (ctx->bal_weight > 0.f ? GLS_SCHED_LEARNED_BALANCE : 0u);
}

// Checks and buffers of a batched run; *B receives the windows per wave.
static int batch_setup(gls_ctx *ctx, const gls_batch_opts &o, uint64_t *B)
{
    if (!ctx->loaded) return fail(ctx, GLS_ESTATE, "run before load_netlist");
    if (ctx->opts.alloc_mode == GLS_ALLOC_LEARNED && !ctx->have_model)
        return fail(ctx, GLS_ESTATE, "GLS_ALLOC_LEARNED needs gls_set_presize_model before gls_run_batched");
    cudaSetDevice(ctx->opts.device);
    const size_t nw = ctx->windows.size();
    if (o.saif_only)
        for (Window *w : ctx->windows) release_window_pool(ctx, w);
    // windows per wave: all of them, or with saif_only as many as free device
    // memory holds (each needs its pool, net tables and a level work space)
    uint64_t b = std::min<uint64_t>(std::max<size_t>(nw, 1), kMaxWave);
    if (o.max_wave) b = std::min<uint64_t>(b, o.max_wave);
    if (o.saif_only) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        fr += spare_bytes(ctx);
        uint64_t per = 0;
        for (Window *w : ctx->windows) per = std::max<uint64_t>(per, projected_cap(ctx, w) * w->word_bytes());
        per += (uint64_t)ctx->n_nets * 48 + (uint64_t)(ctx->max_width + 1) * 32 +
               (uint64_t)ctx->seg_cap * (sizeof(SegRec) + sizeof(CopyRec)) + ctx->scr_cap * 4;
        const uint64_t fit = std::max<uint64_t>(1, (uint64_t)(0.85 * (double)fr) / std::max<uint64_t>(per, 1));
        b = std::max<uint64_t>(1, std::min(b, fit));
    }
    while (ctx->lsc.size() < b) ctx->lsc.push_back(new LevelScratch);
    for (uint64_t k = 0; k < b; ++k)
        CK(ctx->lsc[k]->ensure(ctx->max_width, ctx->seg_cap, ctx->scr_cap), "alloc level work spaces");
    // two descriptor sets: the per-gate-output tables of even and odd levels
    if (!ctx->hwave.ensure(2 * kMaxWave * sizeof(WinDev))) return fail(ctx, GLS_ENOMEM, "pinned wave descriptors");
    CK(ctx->dwave.ensure(2 * kMaxWave * sizeof(WinDev)), "alloc wave descriptors");
    // allocated here, never inside a stream capture
    CK(ctx->wave_e.ensure((ctx->drv_level_start.size() - 1) * kClasses * 8 + 8), "alloc wave totals");
    *B = b;
    return GLS_OK;
}

// One wave: windows [w0, w0 + nwin) together; *ms receives its device time
// (upload of new stimuli excluded, reruns of windows that outgrew a buffer
// included in acc).
static int run_wave(gls_ctx *ctx, size_t w0, uint32_t nwin, const gls_batch_opts &o, RunAcc &acc, float *ms,
                    cudaEvent_t e0, cudaEvent_t e1)
{
    WinDev *hw = ctx->hwave.as<WinDev>();
    uint32_t max_stim = 0;
    for (uint32_t k = 0; k < nwin; ++k)
        CK(ctx->lsc[k]->ensure(ctx->max_width, ctx->seg_cap, ctx->scr_cap), "alloc level work spaces");
    for (uint32_t k = 0; k < nwin; ++k) {
        Window *w = ctx->windows[w0 + k];
        int rc = w->uploaded ? GLS_OK : upload_window(ctx, w, false);
        if (rc == GLS_OK) rc = reset_window(ctx, w);
        if (rc) return rc;
        w->saif_only = false;
        hw[k] = make_windev(ctx, w, *ctx->lsc[k], 0);
        hw[kMaxWave + k] = make_windev(ctx, w, *ctx->lsc[k], 1);
        max_stim = std::max(max_stim, hw[k].n_stim);
    }
    CK(cudaEventRecord(e0, ctx->stream), "event");
    for (int p = 0; p < 2; ++p)
        CK(cudaMemcpyAsync(ctx->dwave.as<WinDev>() + p * kMaxWave, hw + p * kMaxWave, nwin * sizeof(WinDev),
                           cudaMemcpyHostToDevice, ctx->stream),
           "upload wave descriptors");
    const WinDev *dw[2] = {ctx->dwave.as<WinDev>(), ctx->dwave.as<WinDev>() + kMaxWave};
    const WinDev *hp[2] = {&hw[0], &hw[kMaxWave]};
    if (o.use_graph && nwin > 1) {
        // one graph per wave shape; the descriptors it reads are rewritten per wave
        gls_ctx::WaveGraph key{nwin, max_stim, ctx->warp_mask, (uint32_t)ctx->opts.alloc_mode, ctx->seg_per_sm,
                               schedule_flags(ctx), nullptr, 0};
        cudaGraphExec_t ge = nullptr;
        uint32_t l = 0;
        for (auto &g : ctx->graphs)
            if (g.same(key)) {
                ge = g.exec;
                l = g.launches;
            }
        if (!ge) {
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
            int rc = GLS_OK;
            if (e == cudaSuccess) {
                rc = enqueue_levels(ctx, dw, hp, nwin, max_stim, false, &l);
                const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
                if (rc == GLS_OK && e2 != cudaSuccess) e = e2;
            }
            if (rc == GLS_OK && e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
            if (g) cudaGraphDestroy(g);
            if (rc) return rc;
            if (e != cudaSuccess) return fail(ctx, GLS_ECUDA, "capture wave graph: %s", cudaGetErrorString(e));
            key.exec = ge;
            key.launches = l;
            ctx->graphs.push_back(key);
        }
        CK(cudaGraphLaunch(ge, ctx->stream), "graph launch");
        acc.launches += l;
    } else {
        int rc = enqueue_levels(ctx, dw, hp, nwin, max_stim, false, &acc.launches,
                                nwin == 1 && ctx->windows[w0]->w64);
        if (rc) return rc;
    }
    CK(cudaEventRecord(e1, ctx->stream), "event");
    CK(cudaStreamSynchronize(ctx->stream), "wave");
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    *ms = t;
    // windows that finished first (and, with saif_only, give their pools
    // back), then the ones that outgrew a buffer, rerun alone with more room
    std::vector<uint32_t> again;
    for (uint32_t k = 0; k < nwin; ++k) {
        Window *w = ctx->windows[w0 + k];
        unsigned long long small[8];
        CK(cudaMemcpy(small, w->small.p, sizeof small, cudaMemcpyDeviceToHost), "read status");
        if (small[5]) {
            again.push_back(k);
            continue;
        }
        int rc = settle_window(ctx, w, acc);
        if (rc) return rc;
        if (o.saif_only) {
            release_window_pool(ctx, w);
            w->saif_only = true;
        }
    }
    if (!again.empty())   // room for the reruns: the other windows' work spaces come back next wave
        for (size_t k = 1; k < ctx->lsc.size(); ++k) ctx->lsc[k]->release();
    for (uint32_t k : again) {
        Window *w = ctx->windows[w0 + k];
        int rc = settle_window(ctx, w, acc);
        if (rc) return rc;
        if (o.saif_only) {
            release_window_pool(ctx, w);
            w->saif_only = true;
        }
    }
    return GLS_OK;
}

extern "C" int gls_run_batched(gls_ctx *ctx, const gls_batch_opts *opts)
{
    if (!ctx) return GLS_EINVAL;
    gls_batch_opts o{0, 1, 0};
    if (opts) o = *opts;
    uint64_t B = 1;
    int rc = batch_setup(ctx, o, &B);
    if (rc) return rc;
    RunAcc acc;
    const double kms[4] = {0, 0, 0, 0};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    for (size_t w0 = 0; w0 < ctx->windows.size() && rc == GLS_OK;) {
        uint64_t nwin = std::min<uint64_t>(B, ctx->windows.size() - w0);
        if (o.saif_only) {
            // pools grow with what earlier windows needed: refit the wave to free memory
            size_t fr = 0, tot = 0;
            cudaMemGetInfo(&fr, &tot);
            fr += spare_bytes(ctx);
            uint64_t per = 1;
            for (uint64_t k = 0; k < nwin; ++k) {
                const Window *w = ctx->windows[w0 + k];
                per = std::max<uint64_t>(per, projected_cap(ctx, w) * w->word_bytes() + (uint64_t)ctx->n_nets * 48);
            }
            nwin = std::max<uint64_t>(1, std::min<uint64_t>(nwin, (uint64_t)(0.85 * (double)fr) / per));
        }
        // a window of 64-bit event words runs alone; a wave stops before one
        if (ctx->windows[w0]->w64) {
            nwin = 1;
        } else {
            for (uint64_t k = 1; k < nwin; ++k)
                if (ctx->windows[w0 + k]->w64) {
                    nwin = k;
                    break;
                }
        }
        float ms = 0.f;
        rc = run_wave(ctx, w0, (uint32_t)nwin, o, acc, &ms, e0, e1);
        acc.total_ms += ms;
        w0 += nwin;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    publish_stats(ctx, acc, kms);
    return GLS_OK;
}

extern "C" int gls_set_schedule(gls_ctx *ctx, uint32_t seg_per_sm, uint32_t warp_mask, uint32_t flags)
{
    if (!ctx) return GLS_EINVAL;
    const uint32_t all = GLS_SCHED_CLASS_PRIORITY | GLS_SCHED_BLOCK256 | GLS_SCHED_WIDE_LOADS | GLS_SCHED_LEARNED_BALANCE;
    if (seg_per_sm < 64 || seg_per_sm > 65536 || warp_mask > 7 || (flags & ~all))
        return fail(ctx, GLS_EINVAL, "schedule out of range: %u segments per SM, warp mask %u, flags %u", seg_per_sm,
                    warp_mask, flags);
    apply_schedule(ctx, seg_per_sm, warp_mask, flags);
    ctx_drop_graphs(ctx);
    return GLS_OK;
}

extern "C" int gls_autotune(gls_ctx *ctx, const gls_batch_opts *opts, gls_tune_result *res)
{
    if (!ctx) return GLS_EINVAL;
    if (ctx->windows.empty()) return fail(ctx, GLS_ESTATE, "autotune needs at least one added window");
    gls_batch_opts o{0, 1, 0};
    if (opts) o = *opts;
    uint64_t B = 1;
    int rc = batch_setup(ctx, o, &B);
    if (rc) return rc;
    const uint32_t nwin = (uint32_t)std::min<uint64_t>(B, ctx->windows.size());
    // Stage 1: time segments per SM for the thread-per-segment kernel times
    // which fan-in classes run warp-per-segment.  Stage 2, on the best of
    // those: class-stream priority, the gate kernel's block size and load
    // width (the variants change nothing but speed).
    static const uint32_t kSegs[] = {1024, 2048, 4096};
    static const uint32_t kMasks[] = {0, 1, 7};
    static const uint32_t kFlags2[] = {GLS_SCHED_CLASS_PRIORITY, GLS_SCHED_BLOCK256, GLS_SCHED_WIDE_LOADS,
                                       GLS_SCHED_BLOCK256 | GLS_SCHED_WIDE_LOADS};
    gls_tune_result r;
    std::memset(&r, 0, sizeof r);
    float best = 1e30f;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    const uint32_t keep_segs = ctx->seg_per_sm, keep_mask = ctx->warp_mask, keep_flags = schedule_flags(ctx);
    uint32_t c = 0;
    auto trial = [&](uint32_t segs, uint32_t mask, uint32_t flags) {
        apply_schedule(ctx, segs, mask, flags);
        RunAcc acc;
        float t = 1e30f;
        // the first run of a shape captures its graph; the best of the next two counts
        for (int rep = 0; rep < 3 && rc == GLS_OK; ++rep) {
            float tr = 0.f;
            rc = run_wave(ctx, 0, nwin, o, acc, &tr, e0, e1);
            if (rep) t = std::min(t, tr);
        }
        r.ms[c] = t;
        r.seg_per_sm[c] = segs;
        r.warp_mask[c] = mask;
        r.flags[c] = flags;
        if (rc == GLS_OK && t < best) {
            best = t;
            r.best = c;
        }
        ++c;
    };
    for (uint32_t ms_i = 0; ms_i < 3 && rc == GLS_OK; ++ms_i)
        for (uint32_t s_i = 0; s_i < 3 && rc == GLS_OK; ++s_i) trial(kSegs[s_i], kMasks[ms_i], 0);
    const uint32_t segs1 = r.seg_per_sm[r.best], mask1 = r.warp_mask[r.best];
    for (uint32_t f : kFlags2) {
        if (rc != GLS_OK) break;
        trial(segs1, mask1, f);
    }
    if (rc == GLS_OK && ctx->opts.alloc_mode == GLS_ALLOC_LEARNED) trial(segs1, mask1, GLS_SCHED_LEARNED_BALANCE);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    r.n = c;
    r.windows = nwin;
    if (rc) {
        apply_schedule(ctx, keep_segs, keep_mask, keep_flags);
        return rc;
    }
    apply_schedule(ctx, r.seg_per_sm[r.best], r.warp_mask[r.best], r.flags[r.best]);
    if (res) *res = r;
    return GLS_OK;
}

// A large host copy split over the context's worker threads (the SAIF table
// of a 2M-net design is 48 MB: one thread copies it at a fraction of the
// memory bandwidth).
static void host_copy(gls_ctx *ctx, void *dst, const void *src, size_t bytes)
{
    if (bytes < (8u << 20) || !ctx->pool) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const unsigned parts = ctx->pool->threads();
    const size_t step = ((bytes + parts - 1) / parts + 63) & ~(size_t)63;
    ctx->pool->parallel_for(parts, [&](unsigned q) {
        const size_t a = std::min(bytes, q * step), b = std::min(bytes, a + step);
        if (b > a) std::memcpy(static_cast<char *>(dst) + a, static_cast<const char *>(src) + a, b - a);
    });
}

static Window *get_done(gls_ctx *ctx, uint32_t window)
{
    if (window >= ctx->windows.size()) return nullptr;
    Window *w = ctx->windows[window];
    return w->done ? w : nullptr;
}

extern "C" int gls_saif_counts(gls_ctx *ctx, uint32_t window, uint64_t *t0, uint64_t *t1, uint64_t *tx)
{
    if (!ctx || !t0 || !t1 || !tx) return GLS_EINVAL;
    Window *w = get_done(ctx, window);
    if (!w) return fail(ctx, GLS_ESTATE, "window %u not simulated", window);
    cudaSetDevice(ctx->opts.device);
    // through pinned staging: a pageable destination would go through the
    // driver's bounce buffers at a fraction of the link's speed
    const size_t bytes = (size_t)ctx->n_nets * 24;
    if (!ctx->pin_out.ensure(bytes)) return fail(ctx, GLS_ENOMEM, "pinned staging for SAIF counts");
    CK(cudaMemcpyAsync(ctx->pin_out.p, w->saif.p, bytes, cudaMemcpyDeviceToHost, ctx->stream), "read saif");
    CK(cudaStreamSynchronize(ctx->stream), "read saif");
    const uint64_t *buf = ctx->pin_out.as<uint64_t>();
    auto part = [&](uint32_t n0, uint32_t n1) {
        for (uint32_t n = n0; n < n1; ++n) {
            t0[n] = buf[3ull * n];
            t1[n] = buf[3ull * n + 1];
            tx[n] = buf[3ull * n + 2];
        }
    };
    if (ctx->n_nets < (1u << 18) || !ctx->pool) {
        part(0, ctx->n_nets);
    } else {   // large designs: split over the worker threads, like host_copy
        const unsigned parts = ctx->pool->threads();
        const uint32_t step = (ctx->n_nets + parts - 1) / parts;
        ctx->pool->parallel_for(parts, [&](unsigned q) {
            part(std::min(ctx->n_nets, q * step), std::min(ctx->n_nets, (q + 1) * step));
        });
    }
    return GLS_OK;
}

extern "C" int gls_saif_table(gls_ctx *ctx, uint32_t window, uint64_t *t3)
{
    if (!ctx || !t3) return GLS_EINVAL;
    Window *w = get_done(ctx, window);
    if (!w) return fail(ctx, GLS_ESTATE, "window %u not simulated", window);
    cudaSetDevice(ctx->opts.device);
    // the device keeps the counters in this layout: one copy through pinned staging
    const size_t bytes = (size_t)ctx->n_nets * 24;
    if (!ctx->pin_out.ensure(bytes)) return fail(ctx, GLS_ENOMEM, "pinned staging for SAIF counts");
    CK(cudaMemcpyAsync(ctx->pin_out.p, w->saif.p, bytes, cudaMemcpyDeviceToHost, ctx->stream), "read saif");
    CK(cudaStreamSynchronize(ctx->stream), "read saif");
    host_copy(ctx, t3, ctx->pin_out.p, bytes);
    return GLS_OK;
}

extern "C" int gls_waveform_lengths(gls_ctx *ctx, uint32_t window, uint32_t *len)
{
    if (!ctx || !len) return GLS_EINVAL;
    Window *w = get_done(ctx, window);
    if (!w) return fail(ctx, GLS_ESTATE, "window %u not simulated", window);
    cudaSetDevice(ctx->opts.device);
    const size_t bytes = (size_t)ctx->n_nets * 4;
    if (!ctx->pin_out.ensure(bytes)) return fail(ctx, GLS_ENOMEM, "pinned staging for lengths");
    CK(cudaMemcpyAsync(ctx->pin_out.p, w->net_len.p, bytes, cudaMemcpyDeviceToHost, ctx->stream), "read lengths");
    CK(cudaStreamSynchronize(ctx->stream), "read lengths");
    std::memcpy(len, ctx->pin_out.p, bytes);
    return GLS_OK;
}

extern "C" int gls_waveform(gls_ctx *ctx, uint32_t window, uint32_t net, uint32_t *time, uint8_t *value,
                            uint64_t cap, uint64_t *n)
{
    if (!ctx || !n) return GLS_EINVAL;
    Window *w = get_done(ctx, window);
    if (!w) return fail(ctx, GLS_ESTATE, "window %u not simulated", window);
    if (net >= ctx->n_nets) return fail(ctx, GLS_EINVAL, "net %u out of range", net);
    if (w->saif_only) return fail(ctx, GLS_ESTATE, "window %u ran with saif_only: its waveforms were not kept", window);
    cudaSetDevice(ctx->opts.device);
    uint64_t off = 0;
    uint32_t len = 0;
    CK(cudaMemcpy(&off, w->net_off.as<uint64_t>() + net, 8, cudaMemcpyDeviceToHost), "read offset");
    CK(cudaMemcpy(&len, w->net_len.as<uint32_t>() + net, 4, cudaMemcpyDeviceToHost), "read length");
    if (len == 0xFFFFFFFFu) {
        *n = UINT64_MAX;
        return GLS_OK;
    }
    *n = len;
    const uint64_t k = std::min<uint64_t>(cap, len);
    if (k && (time || value)) {
        if (w->w64) {
            std::vector<WideWord> words(k);
            CK(cudaMemcpy(words.data(), w->pool.as<WideWord>() + off, k * 8, cudaMemcpyDeviceToHost), "read events");
            for (uint64_t e = 0; e < k; ++e) {
                if (time) time[e] = ev_time(words[e]);
                if (value) value[e] = (uint8_t)ev_val(words[e]);
            }
        } else {
            std::vector<uint32_t> words(k);
            CK(cudaMemcpy(words.data(), w->pool.as<uint32_t>() + off, k * 4, cudaMemcpyDeviceToHost), "read events");
            for (uint64_t e = 0; e < k; ++e) {
                if (time) time[e] = ev_time(words[e]);
                if (value) value[e] = (uint8_t)ev_val(words[e]);
            }
        }
    }
    return GLS_OK;
}

extern "C" int gls_stats_get(gls_ctx *ctx, gls_stats *st)
{
    if (!ctx || !st) return GLS_EINVAL;
    *st = ctx->stats;
    return GLS_OK;
}
