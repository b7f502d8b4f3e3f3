// ft_capi.cu — the C ABI of include/footile_gpu.h: context state (footile's
// Plotter settings), device buffers, work-item planning and kernel launches.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>

#include <nvtx3/nvToolsExt.h>
#include <string>
#include <vector>

#include "../../include/ft_fmath.h"
#include "ft_adjoint.cuh"
#include "ft_kernels.cuh"

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) {
            cudaDeviceSynchronize();  // earlier asynchronous work may still use the old buffer
            cudaFree(p);
        }
        p = nullptr;
        cap = 0;
        size_t want = std::max(bytes, (size_t)256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

}  // namespace

struct ft_batch;

namespace {
// A planned batch: the descriptors it was planned for, its work items on the host and the
// device, and the plan knobs; kept while the same batch comes back.
struct PlanSlot {
    std::vector<ft_path_desc> paths;
    std::vector<ftk::WorkItem> h_items, h_items_w;
    DevBuf items, items_w;
    int smem = -1, stroke = -1, wside = -1;
    uint64_t split = 0;
    void release() {
        items.release();
        items_w.release();
    }
};
}  // namespace

struct ft_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // Plotter state (plotter.rs:96-115)
    float tolerance = 0.3f;
    float xf[6] = {1, 0, 0, 0, 1, 0};
    int join = FT_JOIN_MITER;
    float miter_limit = 4.0f;
    float s_width = 1.0f;   // host copy, valid unless sw_on_device
    bool sw_on_device = false;
    int sw_cur = 0;         // the current slot of sw_chain
    // device buffers
    DevBuf ops, paths, overflow, status, sw_out, rasters, queue, scratch, sw_chain;
    DevBuf pool, pool_used, bandoff, crec;  // ordered composite
    DevBuf figbins;                         // one path's figure state and band counts (split binning)
    DevBuf mask;                            // a single large Rgba8p call's Matte8 coverage
    DevBuf gbuf;                            // one fill path's grid-wide figure build
    size_t gb_raw_cap = 0;                  // its raw vertex capacity (grows on demand)
    size_t gs_sraw_cap = 0;                 // a stroke path's raw stroke point capacity (grows on demand)
    DevBuf srgb_lut, conv_src, conv_dst;    // ft_convert
    PlanSlot plan;                                   // the last batch's plan
    std::vector<std::unique_ptr<PlanSlot>> chunk_plans;  // host batches in pipelined chunks
    cudaStream_t s_in = nullptr, s_out = nullptr;    // their copy streams
    std::vector<cudaEvent_t> ev_chunk;               // copied in / drawn, per chunk
    uint32_t last_n_paths = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_comp = nullptr;  // before the tile compositor of the last call
    bool comp_timed = false;        // the last call ran the tile compositor (ev_comp .. ev1)

    bool timed = false;
    uint64_t launches = 0;
    int sm_count = 0;
    int max_smem = 0;
    uint32_t fig_cap = 0;  // vertices per figure of a fill above footile's 65,535 (0: footile's cap)
    ft_tuning tune{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool tuned = false;  // `tune` replaces the built-in plan defaults
    std::string err;
};

static int composite_impl(ft_ctx* c, int32_t stroke, int32_t rule, const ft_op* ops, uint32_t n_ops_total,
                          const ft_path_desc* paths, uint32_t n_paths, int32_t fmt, uint8_t* raster, uint32_t w,
                          uint32_t h, uint32_t stride, int32_t where, float* sw_out);

namespace {

// An NVTX range over one stage of a call (a profiler's timeline shows the path's stages;
// without a tool attached the calls return at once).
struct Stage {
    explicit Stage(const char* name) { nvtxRangePushA(name); }
    ~Stage() { nvtxRangePop(); }
    Stage(const Stage&) = delete;
    Stage& operator=(const Stage&) = delete;
};

int fail(ft_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(ft_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? FT_ERR_NOMEM : FT_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define FT_CU(call, what)                                 \
    do {                                                  \
        cudaError_t _e = (call);                          \
        if (_e != cudaSuccess) return cuda_fail(c, _e, what); \
    } while (0)

// Plan knobs: the context's tuning (ft_set_tuning / ft_autotune_batch) overrides the
// built-in default.
// Dynamic shared memory for a batch whose widest raster row is `max_w` pixels.
int choose_smem(const ft_ctx* c, uint32_t max_w) {
    const int wp = (int)((max_w + 3) & ~3u);
    int smem;
    if (c->tuned && c->tune.cta_smem_bytes > 0) {
        smem = c->tune.cta_smem_bytes;
    } else if (wp <= 512) {
        smem = 48 * 1024;  // four CTAs per SM
    } else {
        smem = ftk::RASTER_FIXED_SMEM + 16 * wp * 4;
    }
    smem = std::max(smem, ftk::RASTER_FIXED_SMEM + wp * 4);
    smem = std::max(smem, (int)(40 * 1024));  // room for the build-phase buffers
    smem = std::min(smem, c->max_smem);
    return smem;
}

// Shared memory of the ordered composite's figure builds (k_cbuild): 48 KB (four CTAs
// per SM), more only when a tall raster's band histogram needs it.  The CTA rasteriser's
// tile knob (cta_smem_bytes) does not apply: it sizes bands of rows, which a build has
// none of, and a larger value only takes resident CTAs from the builds.
int build_smem(const ft_ctx* c, int n_bands) {
    const size_t need = ((size_t)(n_bands + 1) * sizeof(int) + 1023) & ~(size_t)1023;
    return (int)std::min<size_t>(std::max<size_t>(48 * 1024, need), (size_t)c->max_smem);
}

// Largest canvas side the warp rasteriser takes (0 disables it).
int warp_max_side(const ft_ctx* c) {
    const int v = c->tuned ? c->tune.warp_max_side : ftk::WARP_MAX_SIDE;
    return std::max(0, std::min(v, ftk::WARP_MAX_SIDE));
}

// Paths of at least this many pixels are split into row ranges.
uint64_t split_px(const ft_ctx* c) {
    if (c->tuned && c->tune.split_px > 0) return (uint64_t)c->tune.split_px;
    return (uint64_t)(1u << 20);
}

// Resident CTAs per SM of the persistent rasterisers.
int grid_cap(const ft_ctx* c, int per_sm) {
    if (c->tuned && c->tune.grid_per_sm > 0) per_sm = std::min(per_sm, (int)c->tune.grid_per_sm);
    return c->sm_count * per_sm;
}

// Work items of the device queues: small paths go whole to the warp rasteriser,
// large paths are split into row ranges of whole bands for the CTA rasteriser.
// Both lists are ordered longest first.
void plan_items(ft_ctx* c, const ft_path_desc* paths, uint32_t n_paths, int smem, std::vector<ftk::WorkItem>& out,
                std::vector<ftk::WorkItem>& out_w, bool stroke) {
    out.clear();
    out_w.clear();
    const int area_bytes = smem - ftk::RASTER_FIXED_SMEM;
    const uint64_t big_px = split_px(c);
    // few paths cannot fill the GPU one warp or one CTA each: split their rows instead
    const bool few = n_paths < (uint32_t)std::max(2 * c->sm_count, 1);
    const uint32_t wside = (stroke || few) ? 0u : (uint32_t)warp_max_side(c);  // strokes use the CTA kernel
    for (uint32_t i = 0; i < n_paths; i++) {
        const ft_path_desc& d = paths[i];
        const uint32_t wp = (d.width + 3) & ~3u;
        uint32_t R = wp ? (uint32_t)(area_bytes / (int)(wp * 4)) : 1;
        R = std::max(1u, std::min(R, std::max(d.height, 1u)));
        if (d.width <= wside && d.height <= wside) {
            out_w.push_back(ftk::WorkItem{i, 0, d.height, R});
            continue;
        }
        uint32_t rows_per_item = std::max(d.height, 1u);
        if ((uint64_t)d.width * d.height >= big_px && c->sm_count > 0) {
            uint32_t target = (d.height + (uint32_t)c->sm_count - 1) / (uint32_t)c->sm_count;
            rows_per_item = std::max(R, ((target + R - 1) / R) * R);
        } else if (few && c->sm_count > 0) {
            // every item rebuilds the figure, so keep items at least 16 rows tall
            const uint32_t parts = std::max(1u, (uint32_t)(2 * c->sm_count) / std::max(n_paths, 1u));
            rows_per_item = std::max(16u, (d.height + parts - 1) / parts);
        }
        for (uint32_t r = 0; r < std::max(d.height, 1u); r += rows_per_item)
            out.push_back(ftk::WorkItem{i, r, std::min(d.height, r + rows_per_item), R});
    }
    auto order = [&](std::vector<ftk::WorkItem>& v) {
        std::vector<std::pair<uint64_t, uint32_t>> key(v.size());
        for (size_t k = 0; k < v.size(); k++) {
            const ft_path_desc& d = paths[v[k].path];
            key[k] = {(uint64_t)d.n_ops * 64 + (uint64_t)d.width * (v[k].row_end - v[k].row_begin) / 8, (uint32_t)k};
        }
        std::stable_sort(key.begin(), key.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
        std::vector<ftk::WorkItem> sorted(v.size());
        for (size_t k = 0; k < v.size(); k++) sorted[k] = v[key[k].second];
        v.swap(sorted);
    };
    order(out);
    order(out_w);
}

int check_path(ft_ctx* c, const ft_path_desc& d, int fmt, uint64_t raster_bytes, uint64_t n_ops_total) {
    const uint32_t bpp = fmt == FT_RGBA8P ? 4 : 1;
    if (d.width > FT_MAX_WIDTH) return fail(c, FT_ERR_CAP, "raster wider than FT_MAX_WIDTH");
    if ((uint64_t)d.op_begin + d.n_ops > n_ops_total) return fail(c, FT_ERR_ARG, "path ops out of range");
    if (d.height > 0 && d.width > 0) {
        if ((uint64_t)d.stride < (uint64_t)d.width * bpp) return fail(c, FT_ERR_ARG, "stride smaller than a row");
        const uint64_t end = d.raster_offset + (uint64_t)(d.height - 1) * d.stride + (uint64_t)d.width * bpp;
        if (end > raster_bytes) return fail(c, FT_ERR_ARG, "raster region out of range");
        if (fmt == FT_RGBA8P && ((d.raster_offset | d.stride) & 3))
            return fail(c, FT_ERR_ARG, "Rgba8p rasters need 4-byte aligned rows");
    }
    return FT_OK;
}

// Kernel parameters for a planned launch.
void fill_params(ft_ctx* c, ftk::KParams& p, int stroke, int rule, int fmt, int smem) {
    memset(&p, 0, sizeof(p));
    for (int i = 0; i < 6; i++) p.xf[i] = c->xf[i];
    const float t = std::max(c->tolerance, 0.01f);
    p.tol_sq = t * t;
    p.join = c->join;
    p.miter_limit = c->miter_limit;
    p.miter_g = ft_miter_angle(c->miter_limit);
    p.rule = rule;
    p.fmt = fmt;
    p.stroke = stroke;
    p.smem_bytes = smem;
    p.pt_cap = ftk::PT_CAP;
    p.L = ftk::scr_layout(ftk::PT_CAP);
}

int grid_for(ft_ctx* c, int smem, uint32_t n_items, bool stroke) {
    const int grid = grid_cap(c, ftk::raster_blocks_per_sm(smem, stroke));
    return std::max(1, std::min(grid, (int)std::max(n_items, 1u)));
}

// Grid of the warp rasteriser.
int grid_for_warp(ft_ctx* c, uint32_t n_items_w) {
    const int grid = grid_cap(c, ftk::raster_warp_blocks_per_sm());
    const int need = (int)((n_items_w + ftk::NWARP - 1) / ftk::NWARP);
    return std::max(1, std::min(grid, std::max(need, 1)));
}

// Enqueue the two rasterisers for prepared parameters: warps for small paths,
// then CTAs for large paths and for small ones a warp could not hold.
cudaError_t enqueue(const ftk::KParams& p, int grid_b, int grid_w, int smem, cudaStream_t st, uint64_t* launches,
                    int sm_count) {
    cudaError_t e = cudaSuccess;
    if (p.n_items_w) {
        e = ftk::launch_raster_warp(p, grid_w, st);
        if (e != cudaSuccess) return e;
        (*launches)++;
    }
    if (p.n_items || p.n_items_w) {
        e = ftk::launch_raster(p, grid_b, smem, st, grid_b <= sm_count);
        if (e == cudaSuccess) (*launches)++;
    }
    return e;
}

// Queue, statuses, launch.  `ops_d` / `rasters_d` are device pointers.
// Plan (or reuse the plan of `slot`), upload and launch one batch on the context stream;
// per-path statuses go to status_d.
int run_plan(ft_ctx* c, PlanSlot& slot, int stroke, int rule, const ft_op* ops_d, const ft_path_desc* paths,
             uint32_t n_paths, int fmt, uint8_t* rasters_d, const float* sw_chain, float* sw_out, int32_t* status_d,
             bool events = true, bool host_rasters = false) {
    uint32_t max_w = 1;
    for (uint32_t i = 0; i < n_paths; i++) max_w = std::max(max_w, paths[i].width);
    const int smem = choose_smem(c, max_w);
    // a batch that comes back unchanged (same descriptors and plan knobs) keeps its
    // planned and uploaded work items
    const bool same_plan = slot.smem == smem && slot.stroke == stroke && slot.wside == warp_max_side(c) &&
                           slot.split == split_px(c) && slot.paths.size() == n_paths &&
                           (n_paths == 0 || memcmp(slot.paths.data(), paths, sizeof(ft_path_desc) * n_paths) == 0);
    if (!same_plan) {
        slot.smem = -1;  // invalid until the new items are on the device
        plan_items(c, paths, n_paths, smem, slot.h_items, slot.h_items_w, stroke != 0);
    }
    const uint32_t n_items = (uint32_t)slot.h_items.size(), n_items_w = (uint32_t)slot.h_items_w.size();
    FT_CU(c->paths.ensure(sizeof(ft_path_desc) * std::max(n_paths, 1u)), "alloc paths");
    if (!same_plan) {
        FT_CU(slot.items.ensure(sizeof(ftk::WorkItem) * std::max(n_items, 1u)), "alloc items");
        FT_CU(slot.items_w.ensure(sizeof(ftk::WorkItem) * std::max(n_items_w, 1u)), "alloc items");
    }
    FT_CU(c->overflow.ensure(sizeof(uint32_t) * std::max(n_items_w, 1u)), "alloc overflow list");
    FT_CU(c->queue.ensure(256), "alloc queue");
    const int grid = n_items_w ? std::max(grid_for(c, smem, n_items, stroke), c->sm_count)
                               : grid_for(c, smem, n_items, stroke);
    const int grid_w = grid_for_warp(c, n_items_w);
    FT_CU(c->scratch.ensure(ftk::SCRATCH_BYTES_PER_CTA * (size_t)std::max(grid, grid_w)), "alloc scratch");
    FT_CU(cudaMemcpyAsync(c->paths.p, paths, sizeof(ft_path_desc) * n_paths, cudaMemcpyHostToDevice, c->stream),
          "upload paths");
    if (!same_plan) {
        if (n_items)
            FT_CU(cudaMemcpyAsync(slot.items.p, slot.h_items.data(), sizeof(ftk::WorkItem) * n_items,
                                  cudaMemcpyHostToDevice, c->stream),
                  "upload items");
        if (n_items_w)
            FT_CU(cudaMemcpyAsync(slot.items_w.p, slot.h_items_w.data(), sizeof(ftk::WorkItem) * n_items_w,
                                  cudaMemcpyHostToDevice, c->stream),
                  "upload items");
        slot.paths.assign(paths, paths + n_paths);
        slot.smem = smem;
        slot.stroke = stroke;
        slot.wside = warp_max_side(c);
        slot.split = split_px(c);
    }
    FT_CU(cudaMemsetAsync(c->queue.p, 0, 256, c->stream), "reset queue");
    if (n_paths) FT_CU(cudaMemsetAsync(status_d, 0, sizeof(int32_t) * n_paths, c->stream), "reset status");
    c->last_n_paths = n_paths;
    if (n_items == 0 && n_items_w == 0) return FT_OK;
    ftk::KParams p;
    fill_params(c, p, stroke, rule, fmt, smem);
    p.ops = ops_d;
    p.paths = static_cast<const ft_path_desc*>(c->paths.p);
    p.items = static_cast<const ftk::WorkItem*>(slot.items.p);
    p.n_items = n_items;
    p.items_w = static_cast<const ftk::WorkItem*>(slot.items_w.p);
    p.n_items_w = n_items_w;
    p.overflow = static_cast<uint32_t*>(c->overflow.p);
    p.queue = static_cast<uint32_t*>(c->queue.p);
    p.rasters = rasters_d;
    p.host_rasters = host_rasters ? 1 : 0;
    p.status = status_d;
    p.sw_out = sw_out;
    p.sw_chain = sw_chain;
    p.scratch = static_cast<unsigned char*>(c->scratch.p);
    c->comp_timed = false;
    if (events) FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
    FT_CU(enqueue(p, grid, grid_w, smem, c->stream, &c->launches, c->sm_count), "launch rasteriser");
    if (events) {
        FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
        c->timed = true;
    }
    return FT_OK;
}

int run(ft_ctx* c, int stroke, int rule, const ft_op* ops_d, const ft_path_desc* paths, uint32_t n_paths, int fmt,
        uint8_t* rasters_d, const float* sw_chain, float* sw_out, bool host_rasters = false) {
    FT_CU(c->status.ensure(sizeof(int32_t) * std::max(n_paths, 1u)), "alloc status");
    return run_plan(c, c->plan, stroke, rule, ops_d, paths, n_paths, fmt, rasters_d, sw_chain, sw_out,
                    static_cast<int32_t*>(c->status.p), true, host_rasters);
}

bool valid_ops_host(const ft_op* ops, uint64_t n) {
    for (uint64_t i = 0; i < n; i++)
        if (ops[i].kind < FT_OP_CLOSE || ops[i].kind > FT_OP_PEN_WIDTH) return false;
    return true;
}

int single(ft_ctx* c, int stroke, int32_t rule, const ft_op* ops, uint32_t n_ops, int32_t fmt, const uint8_t clr[4],
           uint8_t* raster, uint32_t w, uint32_t h, uint32_t stride, int32_t where) {
    if (!c) return FT_ERR_ARG;
    if ((rule != FT_NONZERO && rule != FT_EVENODD) || (fmt != FT_MATTE8 && fmt != FT_RGBA8P) ||
        (where != FT_HOST && where != FT_DEVICE))
        return fail(c, FT_ERR_ARG, "bad rule, format or location");
    if ((n_ops && !ops) || (w && h && !raster)) return fail(c, FT_ERR_ARG, "null buffer");
    FT_CU(cudaSetDevice(c->device), "set device");
    ft_path_desc d;
    memset(&d, 0, sizeof(d));
    d.op_begin = 0;
    d.n_ops = n_ops;
    d.width = w;
    d.height = h;
    d.raster_offset = 0;
    d.stride = stride;
    d.s_width = c->s_width;
    if (clr) memcpy(d.clr, clr, 4);
    const uint32_t bpp = fmt == FT_RGBA8P ? 4 : 1;
    const uint64_t raster_bytes = h ? (uint64_t)(h - 1) * stride + (uint64_t)w * bpp : 0;
    int st = check_path(c, d, fmt, raster_bytes, n_ops);
    if (st != FT_OK) return st;
    // pen-width chain (plotter.rs:151-153): two slots used in turn, the call reads the
    // current one and its kernels write the width after the call into the other, which
    // becomes current when the call is enqueued (no copy between calls)
    FT_CU(c->sw_chain.ensure(2 * sizeof(float)), "alloc pen width");
    float* sw_in = static_cast<float*>(c->sw_chain.p) + c->sw_cur;
    float* sw_next = static_cast<float*>(c->sw_chain.p) + (c->sw_cur ^ 1);
    if (!c->sw_on_device) {
        FT_CU(cudaMemcpyAsync(sw_in, &c->s_width, sizeof(float), cudaMemcpyHostToDevice, c->stream), "pen width");
        c->sw_on_device = true;
    }
    const ft_op* ops_d = ops;
    uint8_t* ras_d = raster;
    if (where == FT_HOST) {
        if (!valid_ops_host(ops, n_ops)) return fail(c, FT_ERR_ARG, "unknown path op kind");
        FT_CU(c->ops.ensure(sizeof(ft_op) * std::max(n_ops, 1u)), "alloc ops");
        FT_CU(c->rasters.ensure(std::max(raster_bytes, (uint64_t)1)), "alloc raster");
        if (n_ops)
            FT_CU(cudaMemcpyAsync(c->ops.p, ops, sizeof(ft_op) * n_ops, cudaMemcpyHostToDevice, c->stream),
                  "upload ops");
        if (raster_bytes)
            FT_CU(cudaMemcpyAsync(c->rasters.p, raster, raster_bytes, cudaMemcpyHostToDevice, c->stream),
                  "upload raster");
        ops_d = static_cast<const ft_op*>(c->ops.p);
        ras_d = static_cast<uint8_t*>(c->rasters.p);
    } else if ((reinterpret_cast<uintptr_t>(ops) & 15) || (fmt == FT_RGBA8P && (reinterpret_cast<uintptr_t>(raster) & 3))) {
        return fail(c, FT_ERR_ARG, "device ops need 16-byte alignment, Rgba8p rasters 4-byte alignment");
    }
    const bool uncapped = !stroke && c->fig_cap > (uint32_t)ftk::PT_CAP;
    if ((uncapped || (uint64_t)w * h >= split_px(c)) && ftk::composite_bands_smem(1, (int)w) <= c->max_smem) {
        // a large canvas, or an un-capped fill: build the figure once and bin its edges,
        // then one CTA per band of rows (the ordered compositor with a single call)
        float sw0 = c->s_width;
        FT_CU(cudaMemcpyAsync(&sw0, sw_in, sizeof(float), cudaMemcpyDeviceToHost, c->stream), "pen width");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
        d.s_width = sw0;
        st = composite_impl(c, stroke, rule, ops_d, n_ops, &d, 1, fmt, ras_d, w, h, stride, FT_DEVICE, sw_next);
    } else {
        st = run(c, stroke, rule, ops_d, &d, 1, fmt, ras_d, sw_in, sw_next);
    }
    if (st != FT_OK) return st;
    c->sw_cur ^= 1;
    if (where == FT_HOST) {
        if (raster_bytes)
            FT_CU(cudaMemcpyAsync(raster, c->rasters.p, raster_bytes, cudaMemcpyDeviceToHost, c->stream),
                  "download raster");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
        int32_t s0 = 0;
        FT_CU(cudaMemcpy(&s0, c->status.p, sizeof(int32_t), cudaMemcpyDeviceToHost), "status");
        if (s0 != FT_OK) return fail(c, s0, s0 == FT_ERR_DEPTH ? "subdivision depth cap reached"
                                                               : "non-finite curve control point or bad op");
    }
    return FT_OK;
}

}  // namespace


struct ft_batch {
    int stroke = 0, rule = 0, fmt = 0, smem = 0, grid = 0, grid_w = 0;
    uint32_t n_paths = 0, n_items = 0, n_items_w = 0;
    uint64_t ops_needed = 0, bytes_needed = 0;
    DevBuf paths, items, items_w, overflow, status, queue, scratch;
    ftk::KParams params;
    const void* g_ops = nullptr;
    void* g_ras = nullptr;
    cudaStream_t g_stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    void release() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        paths.release();
        items.release();
        items_w.release();
        overflow.release();
        status.release();
        queue.release();
        scratch.release();
    }
};

extern "C" {

FT_API int ft_batch_create(ft_ctx* c, int32_t stroke, int32_t rule, const ft_path_desc* paths, uint32_t n_paths,
                           int32_t fmt, ft_batch** out) {
    if (!c || !out) return FT_ERR_ARG;
    *out = nullptr;
    if ((rule != FT_NONZERO && rule != FT_EVENODD) || (fmt != FT_MATTE8 && fmt != FT_RGBA8P))
        return fail(c, FT_ERR_ARG, "bad rule or format");
    if (stroke) rule = FT_NONZERO;  // Plotter::stroke fills the outline NonZero (plotter.rs:364)
    if (n_paths && !paths) return fail(c, FT_ERR_ARG, "null path list");
    FT_CU(cudaSetDevice(c->device), "set device");
    ft_batch* b = new ft_batch();
    b->stroke = stroke;
    b->rule = rule;
    b->fmt = fmt;
    b->n_paths = n_paths;
    uint32_t max_w = 1;
    const uint32_t bpp = fmt == FT_RGBA8P ? 4 : 1;
    for (uint32_t i = 0; i < n_paths; i++) {
        const ft_path_desc& d = paths[i];
        int st = check_path(c, d, fmt, UINT64_MAX, UINT64_MAX);
        if (st != FT_OK) {
            delete b;
            return st;
        }
        max_w = std::max(max_w, d.width);
        b->ops_needed = std::max(b->ops_needed, (uint64_t)d.op_begin + d.n_ops);
        if (d.width && d.height)
            b->bytes_needed = std::max(b->bytes_needed, d.raster_offset + (uint64_t)(d.height - 1) * d.stride +
                                                            (uint64_t)d.width * bpp);
    }
    b->smem = choose_smem(c, max_w);
    std::vector<ftk::WorkItem> items, items_w;
    plan_items(c, paths, n_paths, b->smem, items, items_w, stroke != 0);
    b->n_items = (uint32_t)items.size();
    b->n_items_w = (uint32_t)items_w.size();
    b->grid = b->n_items_w ? std::max(grid_for(c, b->smem, b->n_items, stroke), c->sm_count)
                           : grid_for(c, b->smem, b->n_items, stroke);
    b->grid_w = grid_for_warp(c, b->n_items_w);
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = b->paths.ensure(sizeof(ft_path_desc) * std::max(n_paths, 1u));
    if (e == cudaSuccess) e = b->items.ensure(sizeof(ftk::WorkItem) * std::max(b->n_items, 1u));
    if (e == cudaSuccess) e = b->items_w.ensure(sizeof(ftk::WorkItem) * std::max(b->n_items_w, 1u));
    if (e == cudaSuccess) e = b->overflow.ensure(sizeof(uint32_t) * std::max(b->n_items_w, 1u));
    if (e == cudaSuccess) e = b->status.ensure(sizeof(int32_t) * std::max(n_paths, 1u));
    if (e == cudaSuccess) e = b->queue.ensure(256);
    if (e == cudaSuccess) e = b->scratch.ensure(ftk::SCRATCH_BYTES_PER_CTA * (size_t)std::max(b->grid, b->grid_w));
    if (e == cudaSuccess && n_paths)
        e = cudaMemcpyAsync(b->paths.p, paths, sizeof(ft_path_desc) * n_paths, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && b->n_items)
        e = cudaMemcpyAsync(b->items.p, items.data(), sizeof(ftk::WorkItem) * b->n_items, cudaMemcpyHostToDevice,
                            c->stream);
    if (e == cudaSuccess && b->n_items_w)
        e = cudaMemcpyAsync(b->items_w.p, items_w.data(), sizeof(ftk::WorkItem) * b->n_items_w,
                            cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        b->release();
        delete b;
        return cuda_fail(c, e, "batch setup");
    }
    fill_params(c, b->params, stroke, rule, fmt, b->smem);
    b->params.paths = static_cast<const ft_path_desc*>(b->paths.p);
    b->params.items = static_cast<const ftk::WorkItem*>(b->items.p);
    b->params.n_items = b->n_items;
    b->params.items_w = static_cast<const ftk::WorkItem*>(b->items_w.p);
    b->params.n_items_w = b->n_items_w;
    b->params.overflow = static_cast<uint32_t*>(b->overflow.p);
    b->params.queue = static_cast<uint32_t*>(b->queue.p);
    b->params.status = static_cast<int32_t*>(b->status.p);
    b->params.scratch = static_cast<unsigned char*>(b->scratch.p);
    ftk::raster_blocks_per_sm(b->smem, stroke != 0);  // sets the kernels' shared-memory attributes outside capture
    ftk::raster_warp_blocks_per_sm();
    *out = b;
    return FT_OK;
}

FT_API int ft_batch_launch(ft_ctx* c, ft_batch* b, const ft_op* ops, uint32_t n_ops_total, uint8_t* rasters,
                           uint64_t raster_bytes) {
    Stage stage_("ft_batch_launch");
    if (!c || !b) return FT_ERR_ARG;
    if (n_ops_total < b->ops_needed || raster_bytes < b->bytes_needed)
        return fail(c, FT_ERR_ARG, "ops or raster buffer smaller than the batch needs");
    if ((reinterpret_cast<uintptr_t>(ops) & 15) || (b->fmt == FT_RGBA8P && (reinterpret_cast<uintptr_t>(rasters) & 3)))
        return fail(c, FT_ERR_ARG, "device ops need 16-byte alignment, Rgba8p rasters 4-byte alignment");
    FT_CU(cudaSetDevice(c->device), "set device");
    b->params.ops = ops;
    b->params.rasters = rasters;
    if (c->stream == nullptr || c->stream == cudaStreamLegacy || c->stream == cudaStreamPerThread) {
        // the legacy and per-thread default streams cannot be captured: launch directly
        c->comp_timed = false;
        FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
        FT_CU(cudaMemsetAsync(b->queue.p, 0, 256, c->stream), "reset queue");
        FT_CU(cudaMemsetAsync(b->status.p, 0, sizeof(int32_t) * std::max(b->n_paths, 1u), c->stream), "reset status");
        FT_CU(enqueue(b->params, b->grid, b->grid_w, b->smem, c->stream, &c->launches, c->sm_count),
              "launch rasteriser");
        FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
        c->timed = true;
        return FT_OK;
    }
    if (!b->exec || b->g_ops != ops || b->g_ras != rasters || b->g_stream != c->stream) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        cudaGraph_t g = nullptr;
        FT_CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        cudaError_t e1 = cudaMemsetAsync(b->queue.p, 0, 256, c->stream);
        cudaError_t e2 = cudaMemsetAsync(b->status.p, 0, sizeof(int32_t) * std::max(b->n_paths, 1u), c->stream);
        uint64_t nl = 0;
        cudaError_t e3 = enqueue(b->params, b->grid, b->grid_w, b->smem, c->stream, &nl, c->sm_count);
        cudaError_t e4 = cudaStreamEndCapture(c->stream, &g);
        if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e4 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(c, e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3 != cudaSuccess ? e3 : e4,
                             "capture batch graph");
        }
        cudaError_t e5 = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e5 != cudaSuccess) return cuda_fail(c, e5, "instantiate batch graph");
        b->g_ops = ops;
        b->g_ras = rasters;
        b->g_stream = c->stream;
    }
    c->comp_timed = false;
    FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
    FT_CU(cudaGraphLaunch(b->exec, c->stream), "launch batch graph");
    FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
    c->timed = true;
    c->launches += (b->n_items_w ? 1 : 0) + ((b->n_items || b->n_items_w) ? 1 : 0);
    return FT_OK;
}

FT_API int ft_batch_launch_status(ft_ctx* c, ft_batch* b, int32_t* status, uint32_t n) {
    if (!c || !b || (n && !status)) return FT_ERR_ARG;
    FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    const uint32_t k = std::min(n, b->n_paths);
    if (k) FT_CU(cudaMemcpy(status, b->status.p, sizeof(int32_t) * k, cudaMemcpyDeviceToHost), "status");
    for (uint32_t i = k; i < n; i++) status[i] = FT_OK;
    return FT_OK;
}

FT_API void ft_batch_destroy(ft_batch* b) {
    if (!b) return;
    b->release();
    delete b;
}


FT_API int ft_set_tuning(ft_ctx* c, const ft_tuning* t) {
    if (!c) return FT_ERR_ARG;
    if (!t) {
        c->tune = ft_tuning{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        c->tuned = false;
        return FT_OK;
    }
    if (t->warp_max_side < 0 || t->warp_max_side > ftk::WARP_MAX_SIDE || t->cta_smem_bytes < 0 ||
        (t->cta_smem_bytes && t->cta_smem_bytes < 40 * 1024) || t->cta_smem_bytes > c->max_smem ||
        t->split_px < 0 || t->grid_per_sm < 0 || t->band_rows < 0 || t->band_rows > ftk::NWARP ||
        t->pool_edges < 0 || t->host_chunks < 0 || t->host_chunks > 16 || t->host_mapped < 0 || t->host_mapped > 2 ||
        (t->tile_w != 0 && t->tile_w != 128 && t->tile_w != 256 && t->tile_w != 512 && t->tile_w != 1024) ||
        t->tile_stage < 0 || t->tile_stage > 2 || t->fig_build < 0 || t->fig_build > 2)
        return fail(c, FT_ERR_ARG, "tuning out of range");
    c->tune = *t;
    c->tuned = true;
    return FT_OK;
}

FT_API int ft_get_tuning(ft_ctx* c, ft_tuning* t) {
    if (!c || !t) return FT_ERR_ARG;
    if (c->tuned) {
        *t = c->tune;
    } else {
        *t = ft_tuning{ftk::WARP_MAX_SIDE, 0, 1 << 20, 0, 0, 0, 0, 0, 0, 0, 0};
    }
    return FT_OK;
}

FT_API int ft_ctx_create(int device, ft_ctx** out) {
    if (!out) return FT_ERR_ARG;
    *out = nullptr;
    ft_ctx* c = new ft_ctx();
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_comp);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        delete c;
        return FT_ERR_CUDA;
    }
    c->own_stream = true;
    c->max_smem = ftk::raster_max_smem();
    *out = c;
    return FT_OK;
}

FT_API void ft_ctx_destroy(ft_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->plan.release();
    for (auto& sl : c->chunk_plans) sl->release();
    for (cudaEvent_t e : c->ev_chunk) cudaEventDestroy(e);
    if (c->s_in) cudaStreamDestroy(c->s_in);
    if (c->s_out) cudaStreamDestroy(c->s_out);
    DevBuf* bufs[] = {&c->ops,     &c->paths,   &c->overflow,
                      &c->status,  &c->sw_out,  &c->rasters, &c->queue,   &c->scratch,
                      &c->sw_chain, &c->pool,   &c->pool_used, &c->bandoff, &c->crec,
                      &c->srgb_lut, &c->conv_src, &c->conv_dst, &c->figbins, &c->mask};
    for (DevBuf* b : bufs) b->release();
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev_comp) cudaEventDestroy(c->ev_comp);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

FT_API int ft_set_stream(ft_ctx* c, void* s) {
    if (!c) return FT_ERR_ARG;
    if (c->own_stream && c->stream) {
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
    }
    c->stream = static_cast<cudaStream_t>(s);
    c->own_stream = false;
    return FT_OK;
}

FT_API int ft_set_tolerance(ft_ctx* c, float t) {
    if (!c) return FT_ERR_ARG;
    c->tolerance = std::max(t, 0.01f);
    return FT_OK;
}

FT_API int ft_set_transform(ft_ctx* c, const float m[6]) {
    if (!c || !m) return FT_ERR_ARG;
    for (int i = 0; i < 6; i++) c->xf[i] = m[i];
    return FT_OK;
}

FT_API int ft_set_join(ft_ctx* c, int32_t join, float miter_limit) {
    if (!c || join < FT_JOIN_MITER || join > FT_JOIN_ROUND) return FT_ERR_ARG;
    c->join = join;
    c->miter_limit = miter_limit;
    return FT_OK;
}

FT_API int ft_set_pen_width(ft_ctx* c, float w) {
    if (!c) return FT_ERR_ARG;
    c->s_width = w;
    c->sw_on_device = false;
    return FT_OK;
}

FT_API int ft_set_figure_cap(ft_ctx* c, uint32_t max_points) {
    if (!c) return FT_ERR_ARG;
    if (max_points > ftk::FIG_CAP_MAX) return fail(c, FT_ERR_ARG, "figure cap above FT_FIG_CAP_MAX");
    c->fig_cap = max_points <= (uint32_t)ftk::PT_CAP ? 0u : max_points;
    return FT_OK;
}

FT_API int ft_get_figure_cap(ft_ctx* c, uint32_t* max_points) {
    if (!c || !max_points) return FT_ERR_ARG;
    *max_points = c->fig_cap ? c->fig_cap : (uint32_t)ftk::PT_CAP;
    return FT_OK;
}

FT_API int ft_get_pen_width(ft_ctx* c, float* w) {
    if (!c || !w) return FT_ERR_ARG;
    if (c->sw_on_device && c->sw_chain.p) {
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
        FT_CU(cudaMemcpy(&c->s_width, static_cast<float*>(c->sw_chain.p) + c->sw_cur, sizeof(float),
                         cudaMemcpyDeviceToHost),
              "pen width");
    }
    *w = c->s_width;
    return FT_OK;
}

FT_API int ft_fill(ft_ctx* c, int32_t rule, const ft_op* ops, uint32_t n_ops, int32_t fmt, const uint8_t clr[4],
                   uint8_t* raster, uint32_t w, uint32_t h, uint32_t stride, int32_t where) {
    Stage stage_("ft_fill");
    return single(c, 0, rule, ops, n_ops, fmt, clr, raster, w, h, stride, where);
}

FT_API int ft_stroke(ft_ctx* c, const ft_op* ops, uint32_t n_ops, int32_t fmt, const uint8_t clr[4],
                     uint8_t* raster, uint32_t w, uint32_t h, uint32_t stride, int32_t where) {
    Stage stage_("ft_stroke");
    return single(c, 1, FT_NONZERO, ops, n_ops, fmt, clr, raster, w, h, stride, where);
}

// Host batches in chunks of paths whose ops and rasters are ascending, disjoint ranges of
// the host buffers: chunk k + 1 is copied in and chunk k - 1 copied out while chunk k is
// drawn (one copy stream each way, events between the stages, each chunk's plan kept).
// Returns -1 (nothing done) when the layout does not allow it.
static int run_pipelined(ft_ctx* c, int stroke, int rule, const ft_op* ops, uint32_t n_ops_total,
                         const ft_path_desc* paths, uint32_t n_paths, int fmt, uint8_t* rasters, uint64_t raster_bytes,
                         int n_chunks) {
    const uint32_t bpp = fmt == FT_RGBA8P ? 4 : 1;
    auto rend = [&](const ft_path_desc& d) {
        return d.height ? d.raster_offset + (uint64_t)(d.height - 1) * d.stride + (uint64_t)d.width * bpp
                        : d.raster_offset;
    };
    // chunks of about equal raster bytes, by the paths' raster offsets
    std::vector<uint32_t> pb(n_chunks + 1, n_paths);
    pb[0] = 0;
    for (int k = 1, i = 0; k < n_chunks; k++) {
        const uint64_t cut = raster_bytes / n_chunks * k;
        while (i < (int)n_paths && paths[i].raster_offset < cut) i++;
        pb[k] = (uint32_t)i;
    }
    struct Range {
        uint64_t o0, o1, r0, r1;
    };
    std::vector<Range> rg(n_chunks);
    for (int k = 0; k < n_chunks; k++) {
        if (pb[k + 1] <= pb[k]) return -1;
        Range r{UINT64_MAX, 0, UINT64_MAX, 0};
        for (uint32_t i = pb[k]; i < pb[k + 1]; i++) {
            const ft_path_desc& d = paths[i];
            r.o0 = std::min<uint64_t>(r.o0, d.op_begin);
            r.o1 = std::max<uint64_t>(r.o1, (uint64_t)d.op_begin + d.n_ops);
            r.r0 = std::min<uint64_t>(r.r0, d.raster_offset);
            r.r1 = std::max<uint64_t>(r.r1, rend(d));
        }
        if (k && (r.o0 < rg[k - 1].o1 || r.r0 < rg[k - 1].r1)) return -1;
        rg[k] = r;
    }
    if (!c->s_in) FT_CU(cudaStreamCreateWithFlags(&c->s_in, cudaStreamNonBlocking), "copy stream");
    if (!c->s_out) FT_CU(cudaStreamCreateWithFlags(&c->s_out, cudaStreamNonBlocking), "copy stream");
    while ((int)c->ev_chunk.size() < 2 * n_chunks + 2) {
        cudaEvent_t e;
        FT_CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
        c->ev_chunk.push_back(e);
    }
    while ((int)c->chunk_plans.size() < n_chunks) c->chunk_plans.emplace_back(new PlanSlot());
    FT_CU(c->ops.ensure(sizeof(ft_op) * std::max<uint64_t>(n_ops_total, 1)), "alloc ops");
    FT_CU(c->rasters.ensure(std::max<uint64_t>(raster_bytes, 1)), "alloc rasters");
    FT_CU(c->status.ensure(sizeof(int32_t) * std::max(n_paths, 1u)), "alloc status");
    cudaEvent_t* ev = c->ev_chunk.data();  // [0]: start, [1 + k]: copied in, [1 + K + k]: drawn, [1 + 2K]: out
    auto* ops_d = static_cast<ft_op*>(c->ops.p);
    auto* ras_d = static_cast<uint8_t*>(c->rasters.p);
    auto* st_d = static_cast<int32_t*>(c->status.p);
    FT_CU(cudaEventRecord(ev[0], c->stream), "event");  // after the context's earlier work
    FT_CU(cudaStreamWaitEvent(c->s_in, ev[0], 0), "wait");
    FT_CU(cudaStreamWaitEvent(c->s_out, ev[0], 0), "wait");
    for (int k = 0; k < n_chunks; k++) {
        const Range& r = rg[k];
        if (r.o1 > r.o0)
            FT_CU(cudaMemcpyAsync(ops_d + r.o0, ops + r.o0, sizeof(ft_op) * (r.o1 - r.o0), cudaMemcpyHostToDevice,
                                  c->s_in),
                  "upload ops");
        if (r.r1 > r.r0)
            FT_CU(cudaMemcpyAsync(ras_d + r.r0, rasters + r.r0, r.r1 - r.r0, cudaMemcpyHostToDevice, c->s_in),
                  "upload rasters");
        FT_CU(cudaEventRecord(ev[1 + k], c->s_in), "event");
    }
    for (int k = 0; k < n_chunks; k++) {
        FT_CU(cudaStreamWaitEvent(c->stream, ev[1 + k], 0), "wait");
        c->comp_timed = false;
        if (k == 0) FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
        int st = run_plan(c, *c->chunk_plans[k], stroke, rule, ops_d, paths + pb[k], pb[k + 1] - pb[k], fmt, ras_d,
                          nullptr, nullptr, st_d + pb[k], false);
        if (st != FT_OK) return st;
        FT_CU(cudaEventRecord(ev[1 + n_chunks + k], c->stream), "event");
        FT_CU(cudaStreamWaitEvent(c->s_out, ev[1 + n_chunks + k], 0), "wait");
        const Range& r = rg[k];
        if (r.r1 > r.r0)
            FT_CU(cudaMemcpyAsync(rasters + r.r0, ras_d + r.r0, r.r1 - r.r0, cudaMemcpyDeviceToHost, c->s_out),
                  "download rasters");
    }
    FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
    c->timed = true;
    c->last_n_paths = n_paths;
    FT_CU(cudaEventRecord(ev[1 + 2 * n_chunks], c->s_out), "event");
    FT_CU(cudaStreamWaitEvent(c->stream, ev[1 + 2 * n_chunks], 0), "wait");
    FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    return FT_OK;
}

// Chunks of a host batch: the tuning's host_chunks, else 2 from 64 MB of rasters.  More
// chunks lose: every chunk's persistent launch ends on its slowest paths (65,536 glyphs
// in 1 / 2 / 4 chunks: 16.3 / 15.7 / 21.6 ms end to end).
static int host_chunks(const ft_ctx* c, uint64_t raster_bytes, uint32_t n_paths) {
    int k = (c->tuned && c->tune.host_chunks > 0) ? c->tune.host_chunks : (raster_bytes >= (64ull << 20) ? 2 : 1);
    k = std::max(1, std::min(k, 16));
    return n_paths >= 4u * (uint32_t)k ? k : 1;
}

// Device address of a host raster buffer that the kernels can write in place: page-locked
// memory mapped into this device's address space (cudaHostAlloc, torch's pinned memory,
// cudaHostRegister), checked at both ends of the range; nullptr otherwise or when the
// tuning's host_mapped switches the mapping off for this buffer (1: rasters and ops are
// copied, 2: ops are copied).
static uint8_t* mapped_host(ft_ctx* c, const void* host, uint64_t n, bool ops) {
    uint8_t* p = static_cast<uint8_t*>(const_cast<void*>(host));
    const int mode = c->tuned ? c->tune.host_mapped : 0;
    if (mode == 1 || (ops && mode == 2) || !p || n == 0) return nullptr;
    cudaPointerAttributes a{}, b{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || cudaPointerGetAttributes(&b, p + (n - 1)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer || !b.devicePointer ||
        a.device != c->device || b.device != c->device)
        return nullptr;
    uint8_t* d = static_cast<uint8_t*>(a.devicePointer);
    return static_cast<uint8_t*>(b.devicePointer) == d + (n - 1) ? d : nullptr;
}

// The kernels load ops as 16-byte words: ops read in place must be 16-byte aligned.
static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

FT_API int ft_fill_batch(ft_ctx* c, int32_t stroke, int32_t rule, const ft_op* ops, uint32_t n_ops_total,
                         const ft_path_desc* paths, uint32_t n_paths, int32_t fmt, uint8_t* rasters,
                         uint64_t raster_bytes, int32_t where) {
    Stage stage_("ft_fill_batch");
    if (!c) return FT_ERR_ARG;
    if ((rule != FT_NONZERO && rule != FT_EVENODD) || (fmt != FT_MATTE8 && fmt != FT_RGBA8P) ||
        (where != FT_HOST && where != FT_DEVICE))
        return fail(c, FT_ERR_ARG, "bad rule, format or location");
    if (stroke) rule = FT_NONZERO;  // Plotter::stroke fills the outline NonZero (plotter.rs:364)
    if (n_paths && !paths) return fail(c, FT_ERR_ARG, "null path list");
    FT_CU(cudaSetDevice(c->device), "set device");
    for (uint32_t i = 0; i < n_paths; i++) {
        int st = check_path(c, paths[i], fmt, raster_bytes, n_ops_total);
        if (st != FT_OK) return st;
    }
    if (where == FT_HOST && fmt == FT_MATTE8) {
        // Matte8 rasters are only written (whole rows from the figure's first row down),
        // so a mapped host buffer takes the kernels' stores directly over the host link:
        // no raster copy in or out, the writes overlap the drawing
        uint8_t* mapped = mapped_host(c, rasters, raster_bytes, false);
        if (mapped) {
            // page-locked ops are read in place too (host_mapped 2: uploaded first)
            const ft_op* ops_d = reinterpret_cast<const ft_op*>(
                aligned16(ops) ? mapped_host(c, ops, sizeof(ft_op) * (uint64_t)n_ops_total, true) : nullptr);
            if (!ops_d) {
                FT_CU(c->ops.ensure(sizeof(ft_op) * std::max<uint64_t>(n_ops_total, 1)), "alloc ops");
                if (n_ops_total)
                    FT_CU(cudaMemcpyAsync(c->ops.p, ops, sizeof(ft_op) * n_ops_total, cudaMemcpyHostToDevice,
                                          c->stream),
                          "upload ops");
                ops_d = static_cast<const ft_op*>(c->ops.p);
            }
            const int st = run(c, stroke, rule, ops_d, paths, n_paths, fmt, mapped, nullptr, nullptr, true);
            if (st != FT_OK) return st;
            FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
            return FT_OK;
        }
    }
    if (where == FT_HOST) {
        const int k = host_chunks(c, raster_bytes, n_paths);
        if (k > 1) {
            const int st = run_pipelined(c, stroke, rule, ops, n_ops_total, paths, n_paths, fmt, rasters, raster_bytes, k);
            if (st != -1) return st;
        }
    }
    const ft_op* ops_d = ops;
    uint8_t* ras_d = rasters;
    if (where == FT_HOST) {  // unknown op kinds are reported per path (FT_ERR_ARG), as for device ops
        FT_CU(c->ops.ensure(sizeof(ft_op) * std::max<uint64_t>(n_ops_total, 1)), "alloc ops");
        FT_CU(c->rasters.ensure(std::max<uint64_t>(raster_bytes, 1)), "alloc rasters");
        if (n_ops_total)
            FT_CU(cudaMemcpyAsync(c->ops.p, ops, sizeof(ft_op) * n_ops_total, cudaMemcpyHostToDevice, c->stream),
                  "upload ops");
        if (raster_bytes)
            FT_CU(cudaMemcpyAsync(c->rasters.p, rasters, raster_bytes, cudaMemcpyHostToDevice, c->stream),
                  "upload rasters");
        ops_d = static_cast<const ft_op*>(c->ops.p);
        ras_d = static_cast<uint8_t*>(c->rasters.p);
    } else if ((reinterpret_cast<uintptr_t>(ops) & 15) || (fmt == FT_RGBA8P && (reinterpret_cast<uintptr_t>(rasters) & 3))) {
        return fail(c, FT_ERR_ARG, "device ops need 16-byte alignment, Rgba8p rasters 4-byte alignment");
    }
    int st = run(c, stroke, rule, ops_d, paths, n_paths, fmt, ras_d, nullptr, nullptr);
    if (st != FT_OK) return st;
    if (where == FT_HOST) {
        if (raster_bytes)
            FT_CU(cudaMemcpyAsync(rasters, c->rasters.p, raster_bytes, cudaMemcpyDeviceToHost, c->stream),
                  "download rasters");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    }
    return FT_OK;
}

// Rows per band of the ordered composite = warps of a compositor CTA (one row each):
// at most eight (built-in: 4 for Rgba8p tiles, measured fastest on 16,384 strokes on
// 2048x2048; 8 for Matte8, whose compositor keeps whole rows: as many as its shared
// memory holds).
static int composite_band_rows(ft_ctx* c, uint32_t w, int fmt) {
    int R = (c->tuned && c->tune.band_rows > 0) ? std::min((int)c->tune.band_rows, ftk::NWARP)
                                                : (fmt == FT_MATTE8 ? ftk::NWARP : 4);
    if (fmt == FT_MATTE8)
        while (R > 1 && ftk::composite_bands_smem(R, (int)w) > c->max_smem) R--;
    return R;
}

// Width of an Rgba8p compositor tile (pixels): built-in the narrowest of 1024, 512, 256
// and 128 that covers the canvas in as few tiles (every tile re-reads its band's edges).
static int composite_tile_w(const ft_ctx* c, uint32_t w) {
    if (c->tuned && c->tune.tile_w > 0) return c->tune.tile_w;
    int tw = 1024;
    while (tw > 128 && (w + tw / 2 - 1) / (tw / 2) == (w + tw - 1) / tw) tw /= 2;
    return tw;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// A 2-D tensor map of an Rgba8p canvas (u32 pixels, rows `stride` bytes apart) with boxes
// of box_w x box_h pixels, through the runtime's driver entry point; false when the
// canvas does not allow one (TMA wants a 16-byte aligned base and row stride).
static bool canvas_tensor_map(CUtensorMap* tm, void* base, uint32_t w, uint32_t h, uint32_t stride, int box_w,
                              int box_h, bool bytes = false) {
    static EncodeTiledFn encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<EncodeTiledFn>(f);
    });
    if (!encode || !base || !w || !h || (reinterpret_cast<uintptr_t>(base) & 15) || (stride & 15) ||
        (uint64_t)stride >= (1ull << 40))
        return false;
    const cuuint64_t dims[2] = {w, h};
    const cuuint64_t strides[1] = {stride};
    const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    const cuuint32_t elem[2] = {1, 1};
    return encode(tm, bytes ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, base, dims, strides,
                  box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

FT_API int ft_composite_batch(ft_ctx* c, int32_t stroke, int32_t rule, const ft_op* ops, uint32_t n_ops_total,
                              const ft_path_desc* paths, uint32_t n_paths, int32_t fmt, uint8_t* raster, uint32_t w,
                              uint32_t h, uint32_t stride, int32_t where) {
    Stage stage_("ft_composite_batch");
    return composite_impl(c, stroke, rule, ops, n_ops_total, paths, n_paths, fmt, raster, w, h, stride, where,
                          nullptr);
}

}  // extern "C"

static int composite_impl(ft_ctx* c, int32_t stroke, int32_t rule, const ft_op* ops, uint32_t n_ops_total,
                          const ft_path_desc* paths, uint32_t n_paths, int32_t fmt, uint8_t* raster, uint32_t w,
                          uint32_t h, uint32_t stride, int32_t where, float* sw_out) {
    if (!c) return FT_ERR_ARG;
    if ((rule != FT_NONZERO && rule != FT_EVENODD) || (fmt != FT_MATTE8 && fmt != FT_RGBA8P) ||
        (where != FT_HOST && where != FT_DEVICE))
        return fail(c, FT_ERR_ARG, "bad rule, format or location");
    if (stroke) rule = FT_NONZERO;
    if ((n_paths && !paths) || (n_ops_total && !ops) || (w && h && !raster)) return fail(c, FT_ERR_ARG, "null buffer");
    if (w > FT_MAX_WIDTH) return fail(c, FT_ERR_CAP, "raster wider than FT_MAX_WIDTH");
    const uint32_t bpp = fmt == FT_RGBA8P ? 4 : 1;
    if (h && stride < (uint64_t)w * bpp) return fail(c, FT_ERR_ARG, "stride smaller than a row");
    if (fmt == FT_RGBA8P && (stride & 3)) return fail(c, FT_ERR_ARG, "Rgba8p rasters need 4-byte aligned rows");
    for (uint32_t i = 0; i < n_paths; i++)
        if ((uint64_t)paths[i].op_begin + paths[i].n_ops > n_ops_total)
            return fail(c, FT_ERR_ARG, "path ops out of range");
    FT_CU(cudaSetDevice(c->device), "set device");
    const uint64_t raster_bytes = h ? (uint64_t)(h - 1) * stride + (uint64_t)w * bpp : 0;
    const ft_op* ops_d = ops;
    uint8_t* ras_d = raster;
    if (where == FT_HOST) {
        if (!valid_ops_host(ops, n_ops_total)) return fail(c, FT_ERR_ARG, "unknown path op kind");
        FT_CU(c->ops.ensure(sizeof(ft_op) * std::max<uint64_t>(n_ops_total, 1)), "alloc ops");
        FT_CU(c->rasters.ensure(std::max<uint64_t>(raster_bytes, 1)), "alloc raster");
        if (n_ops_total)
            FT_CU(cudaMemcpyAsync(c->ops.p, ops, sizeof(ft_op) * n_ops_total, cudaMemcpyHostToDevice, c->stream),
                  "upload ops");
        if (raster_bytes)
            FT_CU(cudaMemcpyAsync(c->rasters.p, raster, raster_bytes, cudaMemcpyHostToDevice, c->stream),
                  "upload raster");
        ops_d = static_cast<const ft_op*>(c->ops.p);
        ras_d = static_cast<uint8_t*>(c->rasters.p);
    } else if ((reinterpret_cast<uintptr_t>(ops) & 15) || (fmt == FT_RGBA8P && (reinterpret_cast<uintptr_t>(raster) & 3))) {
        return fail(c, FT_ERR_ARG, "device ops need 16-byte alignment, Rgba8p rasters 4-byte alignment");
    }
    // a single Rgba8p call is composited from its Matte8 coverage (the mask route below):
    // its bands are the Matte8 compositor's
    const bool mask_route = fmt == FT_RGBA8P && n_paths == 1 && !(c->tuned && c->tune.tile_stage > 0) &&
                            ftk::composite_bands_smem(composite_band_rows(c, w, FT_MATTE8), (int)w) <= c->max_smem;
    const int R = composite_band_rows(c, w, mask_route ? FT_MATTE8 : fmt);
    const int n_bands = (int)((h + R - 1) / R);
    const int tile_w = composite_tile_w(c, w);
    const int stage = (c->tuned && c->tune.tile_stage > 0) ? c->tune.tile_stage : 1;
    const int smem_b = fmt == FT_MATTE8 ? ftk::composite_bands_smem(R, (int)w)
                                        : ftk::composite_tile_smem(R, tile_w, stage == 1);
    if (smem_b > c->max_smem) return fail(c, FT_ERR_CAP, "raster too wide for the band compositor");
    const int smem_a = build_smem(c, n_bands);
    if ((size_t)(n_bands + 1) * sizeof(int) > (size_t)smem_a)
        return fail(c, FT_ERR_CAP, "raster too tall for the band compositor");
    FT_CU(c->paths.ensure(sizeof(ft_path_desc) * std::max(n_paths, 1u)), "alloc paths");
    FT_CU(c->status.ensure(sizeof(int32_t) * std::max(n_paths, 1u)), "alloc status");
    FT_CU(c->queue.ensure(256), "alloc queue");
    FT_CU(c->crec.ensure(sizeof(int4) * std::max(n_paths, 1u)), "alloc path records");
    FT_CU(c->bandoff.ensure(sizeof(int) * (size_t)std::max(n_paths, 1u) * (n_bands + 1)), "alloc band offsets");
    FT_CU(c->pool_used.ensure(sizeof(unsigned long long)), "alloc pool counter");
    // un-capped fills: every CTA's scratch holds a figure of fig_cap vertices (8 GB in all at most)
    const bool uncapped = !stroke && c->fig_cap > (uint32_t)ftk::PT_CAP;
    const ftk::ScrLayout L = ftk::scr_layout(uncapped ? c->fig_cap : ftk::PT_CAP);
    int grid = std::max(1, std::min((int)std::max(n_paths, 1u),
                                    c->sm_count * ftk::composite_build_blocks_per_sm(smem_a, stroke != 0)));
    if (uncapped) grid = (int)std::max<size_t>(1, std::min<size_t>((size_t)grid, (8ull << 30) / L.bytes));
    FT_CU(c->scratch.ensure(L.bytes * (size_t)grid), "alloc scratch");
    if (n_paths)
        FT_CU(cudaMemcpyAsync(c->paths.p, paths, sizeof(ft_path_desc) * n_paths, cudaMemcpyHostToDevice, c->stream),
              "upload paths");
    // one fill path: its figure is built over the whole GPU (the grid build, whose raw
    // vertex arrays grow until the path's raw vertices fit) or by one CTA of k_cbuild
    const int fig_build = c->tuned ? c->tune.fig_build : 0;
    bool grid_build = n_paths == 1 && paths[0].n_ops > 0 &&
                      (fig_build == 2 || (fig_build == 0 && paths[0].n_ops >= FT_GRID_BUILD_OPS));
    auto first_cap = [&](size_t& cap) {
        if (cap) return;
        const uint64_t est = std::max<uint64_t>((uint64_t)paths[0].n_ops * 64, 1u << 20);
        cap = (size_t)std::min<uint64_t>((est + ftk::GB_TILE - 1) / ftk::GB_TILE * ftk::GB_TILE,
                                         (uint64_t)ftk::GB_RAW_MAX);
    };
    if (grid_build) first_cap(c->gb_raw_cap);
    if (grid_build && stroke) first_cap(c->gs_sraw_cap);
    // edge pool: grows until every path's binned edges fit
    // first pool size in edges (it grows on demand)
    const bool penv = c->tuned && c->tune.pool_edges > 0;
    uint64_t want = penv ? (uint64_t)c->tune.pool_edges : std::max<uint64_t>((uint64_t)n_ops_total * 64, 1u << 20);
    for (int attempt = 0; attempt < 4; attempt++) {
        if (!penv || attempt > 0) want = std::max<uint64_t>(want, c->pool.cap / sizeof(ftk::EdgeRec));
        if (penv && attempt == 0 && c->pool.cap > want * sizeof(ftk::EdgeRec)) c->pool.release();
        FT_CU(c->pool.ensure(want * sizeof(ftk::EdgeRec)), "alloc edge pool");
        FT_CU(cudaMemsetAsync(c->queue.p, 0, 256, c->stream), "reset queue");
        FT_CU(cudaMemsetAsync(c->status.p, 0, sizeof(int32_t) * std::max(n_paths, 1u), c->stream), "reset status");
        FT_CU(cudaMemsetAsync(c->pool_used.p, 0, sizeof(unsigned long long), c->stream), "reset pool");
        // one path: its edges are built and binned over the whole GPU after the figure
        const bool split = n_paths == 1;
        if (split) {
            FT_CU(c->figbins.ensure(16 + sizeof(int) * 2 * (size_t)std::max(n_bands, 1)), "alloc figure bins");
            FT_CU(cudaMemsetAsync(c->figbins.p, 0, 16 + sizeof(int) * (size_t)n_bands, c->stream), "reset bins");
        }
        ftk::KParams p;
        fill_params(c, p, stroke, rule, fmt, smem_a);
        p.ops = ops_d;
        p.paths = static_cast<const ft_path_desc*>(c->paths.p);
        p.n_items = n_paths;
        p.queue = static_cast<uint32_t*>(c->queue.p);
        p.status = static_cast<int32_t*>(c->status.p);
        p.scratch = static_cast<unsigned char*>(c->scratch.p);
        p.rasters = ras_d;
        p.canvas_w = w;
        p.canvas_h = h;
        p.canvas_stride = stride;
        p.band_rows = R;
        p.n_bands = n_bands;
        p.pool = static_cast<ftk::EdgeRec*>(c->pool.p);
        p.pool_used = static_cast<unsigned long long*>(c->pool_used.p);
        p.pool_cap = c->pool.cap / sizeof(ftk::EdgeRec);
        p.bandoff = static_cast<int*>(c->bandoff.p);
        p.crec = static_cast<int4*>(c->crec.p);
        p.sw_out = sw_out;
        p.pt_cap = uncapped ? (int)c->fig_cap : ftk::PT_CAP;
        p.L = L;
        if (split) {
            p.split_bin = 1;
            p.fig_state = static_cast<int4*>(c->figbins.p);
            p.bin_hist = reinterpret_cast<int*>(static_cast<char*>(c->figbins.p) + 16);
        }
        const size_t raw_cap = c->gb_raw_cap, sraw_cap = stroke ? c->gs_sraw_cap : 0;
        bool use_probe = false;
        ftk::KParams pp;  // the probe's parameters
        if (grid_build) {
            const ftk::GbLayout G = ftk::gb_layout(paths[0].n_ops, raw_cap, sraw_cap);
            FT_CU(c->gbuf.ensure(G.bytes), "alloc grid build");
            unsigned char* gb = static_cast<unsigned char*>(c->gbuf.p);
            FT_CU(cudaMemsetAsync(gb, 0, 512, c->stream), "reset grid build");
            FT_CU(cudaMemsetAsync(gb + G.tr, 0xFF, G.tp - G.tr, c->stream), "reset grid build");  // tr, tr2
            ftk::GridBuildBufs& g = p.gb;
            g.ops = ops_d + paths[0].op_begin;
            g.n_ops = (int)paths[0].n_ops;
            g.s_width = paths[0].s_width;
            g.raw_cap = (int)raw_cap;
            g.done = reinterpret_cast<unsigned*>(gb);
            g.n_raw = reinterpret_cast<long long*>(gb + 32);
            g.count = reinterpret_cast<int*>(gb + 40);
            g.opa = reinterpret_cast<int4*>(gb + G.opa);
            g.opw = reinterpret_cast<int*>(gb + G.opw);
            g.opn = reinterpret_cast<long long*>(gb + G.opn);
            g.opi = reinterpret_cast<int2*>(gb + G.opi);
            g.opl = reinterpret_cast<int*>(gb + G.opl);
            g.raw = reinterpret_cast<int2*>(gb + G.raw);
            g.fl = gb + G.fl;
            g.kp = gb + G.kp;
            g.rk = reinterpret_cast<int*>(gb + G.rk);
            g.tr = reinterpret_cast<int*>(gb + G.tr);
            g.tp = reinterpret_cast<int4*>(gb + G.tp);
            g.top = reinterpret_cast<int4*>(gb + G.top);
            g.final_flag = nullptr;
            g.skip = nullptr;
            if (stroke) {
                ftk::GridStrokeBufs& q = p.gs;
                q.sraw_cap = (int)sraw_cap;
                q.st = reinterpret_cast<int*>(gb + 128);
                q.n_sraw = reinterpret_cast<long long*>(gb + 160);
                q.done = reinterpret_cast<unsigned*>(gb + 192);
                q.raw4 = reinterpret_cast<float4*>(gb + G.raw4);
                q.sfl = gb + G.sfl;
                q.sopi = reinterpret_cast<int*>(gb + G.sopi);
                q.stile = reinterpret_cast<int2*>(gb + G.stile);
                q.subt = reinterpret_cast<int*>(gb + G.subt);
                q.itoff = reinterpret_cast<int*>(gb + G.itoff);
                q.itc = reinterpret_cast<int*>(gb + G.itc);
                q.final_flag = nullptr;
                q.skip = nullptr;
            }
            // a probe over the first ops: a capped figure usually reaches its cap there, and
            // the build over all ops is then skipped
            const int probe_ops = std::max(2048, p.pt_cap / 32);
            use_probe = (int)paths[0].n_ops > 8 * probe_ops;
            if (use_probe && stroke) {
                // the stroke points over the first ops: the 65,535-point cap is usually reached there
                pp = p;
                pp.gb.n_ops = probe_ops;
                ftk::GridStrokeBufs& q = pp.gs;
                q.n_sraw = reinterpret_cast<long long*>(gb + 256);
                q.done = reinterpret_cast<unsigned*>(gb + 288);
                q.final_flag = reinterpret_cast<int*>(gb + 320);
                p.gs.skip = q.final_flag;
            } else if (use_probe) {
                pp = p;
                ftk::GridBuildBufs& q = pp.gb;
                q.n_ops = probe_ops;
                q.done = reinterpret_cast<unsigned*>(gb + 128);
                q.n_raw = reinterpret_cast<long long*>(gb + 160);
                q.count = reinterpret_cast<int*>(gb + 168);
                q.final_flag = reinterpret_cast<int*>(gb + 172);
                q.tr = reinterpret_cast<int*>(gb + G.tr2);
                g.skip = q.final_flag;
            }
        }
        c->comp_timed = false;
        FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
        if (n_paths) {
            Stage st_build("figure build and edge binning");
            if (grid_build && stroke) {
                FT_CU(ftk::launch_grid_stroke(p, c->sm_count, c->stream, use_probe ? &pp : nullptr),
                      "launch grid stroke build");
                c->launches += use_probe ? 15 : 11;
            } else if (grid_build) {
                FT_CU(ftk::launch_grid_build(p, c->sm_count, c->stream, use_probe ? &pp : nullptr),
                      "launch grid figure build");
                c->launches += use_probe ? 11 : 6;
            } else {
                FT_CU(ftk::launch_composite_build(p, grid, smem_a, c->stream, grid <= c->sm_count),
                      "launch composite build");
                c->launches++;
            }
            if (split) {
                FT_CU(ftk::launch_figure_bins(p, 4 * c->sm_count, c->stream), "launch figure bins");
                c->launches += 3;
            }
        }
        unsigned long long used = 0;
        int4 cr0 = make_int4(0, 0, 0, 0);  // a single call's first raster row, binned edges
        FT_CU(cudaMemcpyAsync(&used, c->pool_used.p, sizeof(used), cudaMemcpyDeviceToHost, c->stream), "pool size");
        if (n_paths == 1)
            FT_CU(cudaMemcpyAsync(&cr0, c->crec.p, sizeof(int4), cudaMemcpyDeviceToHost, c->stream), "path record");
        long long n_raw = 0, n_raw_probe = 0, n_sraw = 0;
        if (grid_build)
            FT_CU(cudaMemcpyAsync(&n_raw, p.gb.n_raw, sizeof(n_raw), cudaMemcpyDeviceToHost, c->stream), "raw count");
        long long n_sraw_probe = 0;
        if (grid_build && stroke)
            FT_CU(cudaMemcpyAsync(&n_sraw, p.gs.n_sraw, sizeof(n_sraw), cudaMemcpyDeviceToHost, c->stream),
                  "stroke point count");
        if (grid_build && stroke && use_probe)
            FT_CU(cudaMemcpyAsync(&n_sraw_probe, pp.gs.n_sraw, sizeof(n_sraw_probe), cudaMemcpyDeviceToHost,
                                  c->stream),
                  "stroke point count");
        if (use_probe)
            FT_CU(cudaMemcpyAsync(&n_raw_probe, pp.gb.n_raw, sizeof(n_raw_probe), cudaMemcpyDeviceToHost, c->stream),
                  "raw count");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
        n_raw = std::max(n_raw, n_raw_probe);  // the full build is skipped after a complete probe
        n_sraw = std::max(n_sraw, n_sraw_probe);
        if (grid_build && stroke && n_sraw > (long long)sraw_cap) {
            // more raw stroke points than the arrays hold: grow them, or build on one CTA
            if (n_sraw > ftk::GB_RAW_MAX) {
                grid_build = false;
            } else {
                const long long want_raw = std::min<long long>(n_sraw + n_sraw / 8, ftk::GB_RAW_MAX);
                c->gs_sraw_cap = (size_t)((want_raw + ftk::GB_TILE - 1) / ftk::GB_TILE * ftk::GB_TILE);
            }
            attempt--;
            continue;
        }
        if (grid_build && n_raw > (long long)raw_cap) {
            // more raw vertices than the arrays hold: grow them, or build on one CTA
            if (n_raw > ftk::GB_RAW_MAX) {
                grid_build = false;
            } else {
                const long long want_raw = std::min<long long>(n_raw + n_raw / 8, ftk::GB_RAW_MAX);
                c->gb_raw_cap = (size_t)((want_raw + ftk::GB_TILE - 1) / ftk::GB_TILE * ftk::GB_TILE);
            }
            attempt--;  // a raw-vertex retry does not count against the edge pool's
            continue;
        }
        if (used > p.pool_cap) {
            want = used + used / 4;
            continue;
        }
        if (n_paths && n_bands) {
            Stage st_comp("compositing");
            // a single Rgba8p call: its Matte8 coverage into a mask (the band compositor), then
            // SrcOver from the mask, canvas and mask streamed through shared memory by TMA
            const uint32_t mstride = (w + 15) & ~15u;
            const int smem_m = ftk::composite_bands_smem(R, (int)w);
            bool streamed = false;
            if (mask_route && smem_m <= c->max_smem) {
                FT_CU(c->mask.ensure((size_t)mstride * h), "alloc mask");
                CUtensorMap tc, tmk;
                if (canvas_tensor_map(&tc, ras_d, w, h, stride, ftk::SO_COLS, ftk::SO_ROWS) &&
                    canvas_tensor_map(&tmk, c->mask.p, w, h, mstride, ftk::SO_COLS, ftk::SO_ROWS, true)) {
                    ftk::KParams pm = p;
                    pm.rasters = static_cast<uint8_t*>(c->mask.p);
                    pm.canvas_stride = mstride;
                    pm.fmt = FT_MATTE8;
                    FT_CU(ftk::launch_composite_bands(pm, smem_m, c->stream), "launch band compositor");
                    const uint8_t* k = paths[0].clr;
                    const unsigned clr = (unsigned)k[0] | ((unsigned)k[1] << 8) | ((unsigned)k[2] << 16) |
                                         ((unsigned)k[3] << 24);
                    FT_CU(cudaEventRecord(c->ev_comp, c->stream), "event");
                    FT_CU(ftk::launch_srcover_mask(tc, tmk, (int)w, (int)h, std::min(cr0.x, (int)h), clr, p.status,
                                                   c->sm_count, c->stream),
                          "launch mask compositor");
                    c->comp_timed = true;
                    c->launches++;
                    streamed = true;
                }
            }
            if (streamed) {
            } else if (fmt == FT_MATTE8) {
                FT_CU(ftk::launch_composite_bands(p, smem_b, c->stream), "launch band compositor");
            } else {
                CUtensorMap tm;
                memset(&tm, 0, sizeof(tm));
                p.seg_w = tile_w;
                p.use_tma = stage == 1 && canvas_tensor_map(&tm, ras_d, w, h, stride, std::min(tile_w, 256), R) ? 1 : 0;
                FT_CU(cudaEventRecord(c->ev_comp, c->stream), "event");
                FT_CU(ftk::launch_composite_tiles(p, tm, c->stream), "launch tile compositor");
                c->comp_timed = true;
            }
            c->launches++;
        }
        FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
        c->timed = true;
        c->last_n_paths = n_paths;
        if (where == FT_HOST) {
            if (raster_bytes)
                FT_CU(cudaMemcpyAsync(raster, c->rasters.p, raster_bytes, cudaMemcpyDeviceToHost, c->stream),
                      "download raster");
            FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
        }
        return FT_OK;
    }
    return fail(c, FT_ERR_NOMEM, "edge pool did not converge");
}

// ---------------------------------------------------------------- conversion
namespace ftc {
cudaError_t launch_convert(int src_fmt, const uint8_t* src, uint32_t src_stride, uint8_t* dst, uint32_t dst_stride,
                           uint32_t w, uint32_t h, const uint8_t* lut, int grid, cudaStream_t s);
int convert_blocks_per_sm();
cudaError_t launch_srcover(bool backward, const float* cov, uint32_t n_layers, uint64_t plane, const float4* clr,
                           const float4* init, float4* out, const float4* grad_out, float* grad_cov,
                           float4* grad_init, uint32_t n_px, int grid, cudaStream_t s, bool partial = false);
}

// lut[a * 256 + c]: the straight channel c / a (clamped to 1; 0 when a = 0) through
// the sRGB transfer function (IEC 61966-2-1), rounded to the nearest byte.
static void srgb_table(std::vector<uint8_t>& lut) {
    lut.assign(256 * 256, 0);
    for (int a = 1; a < 256; a++)
        for (int ch = 0; ch < 256; ch++) {
            const double v = std::min(1.0, (double)ch / (double)a);
            const double e = v <= 0.0031308 ? 12.92 * v : 1.055 * std::pow(v, 1.0 / 2.4) - 0.055;
            lut[a * 256 + ch] = (uint8_t)std::min(255.0, std::floor(e * 255.0 + 0.5));
        }
}

// ------------------------------------------------------------------ autotuner
// Signature of a batch for the tuning cache: GPU, call kind and powers of two of the
// path count, mean / largest canvas side and mean op count.
static std::string tune_key(ft_ctx* c, int stroke, int rule, int fmt, const ft_path_desc* paths, uint32_t n_paths) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess) prop.name[0] = 0;
    double side = 0.0, ops = 0.0;
    uint32_t max_side = 0;
    for (uint32_t i = 0; i < n_paths; i++) {
        side += 0.5 * ((double)paths[i].width + paths[i].height);
        ops += paths[i].n_ops;
        max_side = std::max(max_side, std::max(paths[i].width, paths[i].height));
    }
    auto lg = [](double v) { return v >= 1.0 ? (int)std::floor(std::log2(v)) : -1; };
    const double n = std::max(n_paths, 1u);
    std::string name(prop.name);
    for (char& ch : name)
        if (ch == ' ') ch = '_';
    char buf[512];
    snprintf(buf, sizeof(buf), "%s/sm%d/k%d.r%d.f%d/n%d.s%d.m%d.o%d", name.c_str(), c->sm_count, stroke, rule, fmt,
             lg(n_paths), lg(side / n), lg(max_side), lg(ops / n));
    return std::string(buf);
}

static bool tune_lookup(const char* path, const std::string& key, ft_tuning* t) {
    if (!path) return false;
    FILE* f = fopen(path, "r");
    if (!f) return false;
    char line[1024];
    bool found = false;
    while (fgets(line, sizeof(line), f)) {
        char k[600];
        ft_tuning v;
        float ms;
        v = ft_tuning{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (sscanf(line, "%599s %d %d %d %d %d %d %d %d %d %d %f", k, &v.warp_max_side, &v.cta_smem_bytes,
                   &v.split_px, &v.grid_per_sm, &v.band_rows, &v.pool_edges, &v.host_chunks, &v.host_mapped,
                   &v.tile_w, &v.tile_stage, &ms) == 12 &&
            key == k) {
            *t = v;  // the last entry for a key wins
            found = true;
        }
    }
    fclose(f);
    return found;
}

// ------------------------------------------------------------ coverage adjoint
// Saved state between ft_adjoint_forward and ft_adjoint_backward.
struct ft_adjoint {
    ft_ctx* ctx = nullptr;
    DevBuf ops, paths, area, status, scratch, cov, gcov, gops, gwidth;
    const ft_op* ops_d = nullptr;  // device ops the kernels read (`ops` or a caller's copy)
    float* cov_d = nullptr;        // device coverage of the last forward
    int no_area = 0;               // no winding area kept: the backward reads cov_d (NonZero)
    std::vector<ft_path_desc> h_paths;
    uint32_t n_ops = 0, n_paths = 0;
    uint64_t cov_bytes = 0;
    int rule = FT_NONZERO;
    int stroke = 0, join = FT_JOIN_MITER;
    float miter_limit = 4.0f;
    float xf[6] = {1, 0, 0, 0, 1, 0};
    float tol_sq = 0.09f;
    int grid_f = 1, grid_b = 1;
    bool ready = false;
};

static int adjoint_check_path(ft_ctx* c, const ft_path_desc& d, uint64_t cov_bytes, uint64_t n_ops_total) {
    if ((uint64_t)d.op_begin + d.n_ops > n_ops_total) return fail(c, FT_ERR_ARG, "path ops out of range");
    if (d.width > FT_MAX_WIDTH) return fail(c, FT_ERR_CAP, "coverage wider than FT_MAX_WIDTH");
    if (d.width == 0 || d.height == 0) return FT_OK;
    if ((d.raster_offset & 3) || (d.stride & 3)) return fail(c, FT_ERR_ARG, "coverage offset and stride need 4-byte alignment");
    if ((uint64_t)d.stride < 4ull * d.width) return fail(c, FT_ERR_ARG, "coverage stride below 4 * width");
    const uint64_t end = d.raster_offset + (uint64_t)d.stride * (d.height - 1) + 4ull * d.width;
    if (end > cov_bytes) return fail(c, FT_ERR_ARG, "coverage outside the buffer");
    return FT_OK;
}

// Plotter settings a coverage pass runs with (the context's at the caller's forward).
struct AdjSettings {
    int join = FT_JOIN_MITER;
    float miter_limit = 4.0f;
    float xf[6] = {1, 0, 0, 0, 1, 0};
    float tol_sq = 0.09f;
};

static AdjSettings ctx_settings(const ft_ctx* c) {
    AdjSettings s;
    s.join = c->join;
    s.miter_limit = c->miter_limit;
    for (int k = 0; k < 6; k++) s.xf[k] = c->xf[k];
    const float t = std::max(c->tolerance, 0.01f);
    s.tol_sq = t * t;
    return s;
}

static fta::AParams adjoint_params(const ft_adjoint* a) {
    fta::AParams p{};
    p.ops = a->ops_d;
    p.paths = static_cast<const ft_path_desc*>(a->paths.p);
    p.n_paths = a->n_paths;
    p.area = static_cast<float*>(a->area.p);
    p.status = static_cast<int*>(a->status.p);
    p.scratch = static_cast<unsigned char*>(a->scratch.p);
    for (int k = 0; k < 6; k++) p.xf[k] = a->xf[k];
    p.tol_sq = a->tol_sq;
    p.rule = a->rule;
    p.stroke = a->stroke;
    p.join = a->join;
    p.miter_limit = a->miter_limit;
    p.miter_g = ft_miter_angle(a->miter_limit);
    p.cov = a->cov_d;
    p.no_area = a->no_area;
    return p;
}

// Coverage forward of checked paths (host descriptors) over device ops `ops_d` into
// device coverage `cov_d`: sizes the saved state, uploads the descriptors, resets the
// status and launches; `events` brackets the launch with the context's timing events.
static int adjoint_forward_dev(ft_ctx* c, ft_adjoint* a, int stroke, int rule, const ft_op* ops_d,
                               uint32_t n_ops_total, const ft_path_desc* paths, uint32_t n_paths, float* cov_d,
                               uint64_t cov_bytes, const AdjSettings& set, bool events, bool no_area = false) {
    a->ready = false;
    a->cov_d = cov_d;
    a->no_area = no_area && rule == FT_NONZERO ? 1 : 0;
    a->rule = rule;
    a->stroke = stroke ? 1 : 0;
    a->join = set.join;
    a->miter_limit = set.miter_limit;
    a->n_ops = n_ops_total;
    a->n_paths = n_paths;
    a->cov_bytes = cov_bytes;
    a->ops_d = ops_d;
    a->h_paths.assign(paths, paths + n_paths);
    for (int k = 0; k < 6; k++) a->xf[k] = set.xf[k];
    a->tol_sq = set.tol_sq;
    FT_CU(a->paths.ensure(sizeof(ft_path_desc) * std::max(n_paths, 1u)), "alloc paths");
    FT_CU(a->status.ensure(sizeof(int32_t) * std::max(n_paths, 1u)), "alloc status");
    FT_CU(a->area.ensure(a->no_area ? 4 : std::max<uint64_t>(cov_bytes, 4)), "alloc winding area");
    // as many CTAs per SM as fit (strokes: at most 3, each with a 16 MB scratch)
    const int bps_f = std::min(a->stroke ? 3 : 64, fta::adjoint_blocks_per_sm(false));
    const int bps_b = std::min(a->stroke ? 3 : 64, fta::adjoint_blocks_per_sm(true));
    a->grid_f = (int)std::max(1u, std::min<uint32_t>(n_paths, (uint32_t)(bps_f * c->sm_count)));
    a->grid_b = (int)std::max(1u, std::min<uint32_t>(n_paths, (uint32_t)(bps_b * c->sm_count)));
    const size_t per_cta = a->stroke ? fta::A_SCRATCH_STROKE : fta::A_SCRATCH_PER_CTA;
    FT_CU(a->scratch.ensure(per_cta * (size_t)std::max(a->grid_f, a->grid_b)), "alloc scratch");
    if (n_paths)
        FT_CU(cudaMemcpyAsync(a->paths.p, paths, sizeof(ft_path_desc) * n_paths, cudaMemcpyHostToDevice, c->stream),
              "upload paths");
    FT_CU(cudaMemsetAsync(a->status.p, 0, sizeof(int32_t) * std::max(n_paths, 1u), c->stream), "reset status");
    fta::AParams p = adjoint_params(a);
    c->comp_timed = false;
    if (events) FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
    if (n_paths) {
        FT_CU(fta::launch_adjoint(false, p, a->grid_f, c->stream), "launch adjoint forward");
        c->launches++;
    }
    if (events) {
        FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
        c->timed = true;
    }
    a->ready = true;
    return FT_OK;
}

// Coverage backward into device gradients; grad_ops and grad_width accumulate (the
// caller zeroes them).
static int adjoint_backward_dev(ft_ctx* c, ft_adjoint* a, const float* gcov_d, float* gops_d, float* gw_d,
                                bool events) {
    fta::AParams p = adjoint_params(a);
    p.grad_cov = gcov_d;
    p.grad_ops = gops_d;
    p.grad_width = gw_d;
    c->comp_timed = false;
    if (events) FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
    if (a->n_paths) {
        FT_CU(fta::launch_adjoint(true, p, a->grid_b, c->stream), "launch adjoint backward");
        c->launches++;
    }
    if (events) {
        FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
        c->timed = true;
    }
    return FT_OK;
}

extern "C" {

FT_API int ft_adjoint_forward(ft_ctx* c, int32_t stroke, int32_t rule, const ft_op* ops, uint32_t n_ops_total,
                              const ft_path_desc* paths, uint32_t n_paths, float* cov, uint64_t cov_bytes,
                              int32_t where, ft_adjoint** saved) {
    Stage stage_("ft_adjoint_forward");
    if (!c || !saved) return FT_ERR_ARG;
    if (stroke) rule = FT_NONZERO;  // Plotter::stroke fills the outline NonZero (plotter.rs:364)
    if ((rule != FT_NONZERO && rule != FT_EVENODD) || (where != FT_HOST && where != FT_DEVICE))
        return fail(c, FT_ERR_ARG, "bad rule or location");
    if ((n_paths && !paths) || (n_ops_total && !ops) || (cov_bytes && !cov))
        return fail(c, FT_ERR_ARG, "null pointer");
    for (uint32_t i = 0; i < n_paths; i++) {
        int st = adjoint_check_path(c, paths[i], cov_bytes, n_ops_total);
        if (st != FT_OK) return st;
    }
    if (where == FT_DEVICE && ((reinterpret_cast<uintptr_t>(ops) & 15) || (reinterpret_cast<uintptr_t>(cov) & 3)))
        return fail(c, FT_ERR_ARG, "device ops need 16-byte alignment, coverage 4-byte alignment");
    if (where == FT_HOST && !valid_ops_host(ops, n_ops_total)) return fail(c, FT_ERR_ARG, "unknown path op kind");
    FT_CU(cudaSetDevice(c->device), "set device");
    ft_adjoint* a = *saved;
    if (!a) {
        a = new ft_adjoint();
        a->ctx = c;
        *saved = a;
    }
    a->ready = false;
    FT_CU(a->ops.ensure(sizeof(ft_op) * std::max(n_ops_total, 1u)), "alloc ops");
    if (n_ops_total)
        FT_CU(cudaMemcpyAsync(a->ops.p, ops, sizeof(ft_op) * n_ops_total,
                              where == FT_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, c->stream),
              "copy ops");
    float* cov_d = cov;
    if (where == FT_HOST) {
        FT_CU(a->cov.ensure(std::max<uint64_t>(cov_bytes, 4)), "alloc coverage");
        cov_d = static_cast<float*>(a->cov.p);
    }
    int st = adjoint_forward_dev(c, a, stroke, rule, static_cast<const ft_op*>(a->ops.p), n_ops_total, paths,
                                 n_paths, cov_d, cov_bytes, ctx_settings(c), true);
    if (st != FT_OK) return st;
    if (where == FT_HOST) {
        if (cov_bytes) FT_CU(cudaMemcpyAsync(cov, cov_d, cov_bytes, cudaMemcpyDeviceToHost, c->stream), "download coverage");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    }
    return FT_OK;
}

FT_API int ft_adjoint_backward(ft_ctx* c, ft_adjoint* a, const float* grad_cov, float* grad_ops, float* grad_width,
                               int32_t where) {
    Stage stage_("ft_adjoint_backward");
    if (!c || !a) return FT_ERR_ARG;
    if (!a->ready) return fail(c, FT_ERR_ARG, "backward without a forward");
    if (a->ctx != c) return fail(c, FT_ERR_ARG, "saved state belongs to another context");
    if (where != FT_HOST && where != FT_DEVICE) return fail(c, FT_ERR_ARG, "bad location");
    if ((a->cov_bytes && !grad_cov) || (a->n_ops && !grad_ops)) return fail(c, FT_ERR_ARG, "null pointer");
    if (where == FT_DEVICE && (reinterpret_cast<uintptr_t>(grad_cov) & 3))
        return fail(c, FT_ERR_ARG, "grad_cov needs 4-byte alignment");
    FT_CU(cudaSetDevice(c->device), "set device");
    const size_t gops_bytes = sizeof(float) * 6 * (size_t)a->n_ops;
    const float* gcov_d = grad_cov;
    float* gops_d = grad_ops;
    if (where == FT_HOST) {
        FT_CU(a->gcov.ensure(std::max<uint64_t>(a->cov_bytes, 4)), "alloc coverage gradient");
        FT_CU(a->gops.ensure(std::max<size_t>(gops_bytes, 4)), "alloc op gradient");
        if (a->cov_bytes)
            FT_CU(cudaMemcpyAsync(a->gcov.p, grad_cov, a->cov_bytes, cudaMemcpyHostToDevice, c->stream),
                  "upload coverage gradient");
        gcov_d = static_cast<const float*>(a->gcov.p);
        gops_d = static_cast<float*>(a->gops.p);
    }
    if (gops_bytes) FT_CU(cudaMemsetAsync(gops_d, 0, gops_bytes, c->stream), "reset op gradient");
    float* gw_d = nullptr;  // the kernel accumulates starting-width gradients of strokes here
    if (a->n_paths) {
        if (where == FT_DEVICE && grad_width) {
            gw_d = grad_width;
        } else {
            FT_CU(a->gwidth.ensure(sizeof(float) * a->n_paths), "alloc width gradient");
            gw_d = static_cast<float*>(a->gwidth.p);
        }
        FT_CU(cudaMemsetAsync(gw_d, 0, sizeof(float) * a->n_paths, c->stream), "reset width gradient");
    }
    int st = adjoint_backward_dev(c, a, gcov_d, gops_d, gw_d, true);
    if (st != FT_OK) return st;
    if (where == FT_HOST) {
        if (grad_width && a->n_paths)
            FT_CU(cudaMemcpyAsync(grad_width, gw_d, sizeof(float) * a->n_paths, cudaMemcpyDeviceToHost, c->stream),
                  "download width gradient");
        if (gops_bytes)
            FT_CU(cudaMemcpyAsync(grad_ops, gops_d, gops_bytes, cudaMemcpyDeviceToHost, c->stream),
                  "download op gradient");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    }
    return FT_OK;
}

FT_API int ft_adjoint_status(ft_ctx* c, ft_adjoint* a, int32_t* status, uint32_t n) {
    if (!c || !a || (n && !status)) return FT_ERR_ARG;
    FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    const uint32_t k = std::min(n, a->ready ? a->n_paths : 0u);
    if (k) FT_CU(cudaMemcpy(status, a->status.p, sizeof(int32_t) * k, cudaMemcpyDeviceToHost), "status");
    for (uint32_t i = k; i < n; i++) status[i] = FT_OK;
    return FT_OK;
}

FT_API void ft_adjoint_destroy(ft_adjoint* a) {
    if (!a) return;
    if (a->ctx) {
        cudaSetDevice(a->ctx->device);
        if (a->ctx->stream) cudaStreamSynchronize(a->ctx->stream);
    }
    DevBuf* bufs[] = {&a->ops, &a->paths, &a->area, &a->status, &a->scratch, &a->cov, &a->gcov, &a->gops, &a->gwidth};
    for (DevBuf* b : bufs) b->release();
    delete a;
}

FT_API int ft_convert(ft_ctx* c, int32_t src_fmt, const uint8_t* src, uint32_t src_stride, int32_t dst_fmt,
                      uint8_t* dst, uint32_t dst_stride, uint32_t w, uint32_t h, int32_t where) {
    Stage stage_("ft_convert");
    if (!c) return FT_ERR_ARG;
    if (!((src_fmt == FT_RGBA8P && dst_fmt == FT_SRGBA8) || (src_fmt == FT_MATTE8 && dst_fmt == FT_SGRAY8)) ||
        (where != FT_HOST && where != FT_DEVICE))
        return fail(c, FT_ERR_ARG, "conversions: Rgba8p -> SRgba8, Matte8 -> SGray8");
    const uint64_t row = (uint64_t)w * (src_fmt == FT_RGBA8P ? 4 : 1);
    if (w == 0 || h == 0) return FT_OK;
    if (!src || !dst || src_stride < row || dst_stride < row) return fail(c, FT_ERR_ARG, "bad buffer or stride");
    FT_CU(cudaSetDevice(c->device), "set device");
    if (!c->srgb_lut.p) {
        std::vector<uint8_t> lut;
        srgb_table(lut);
        FT_CU(c->srgb_lut.ensure(lut.size()), "alloc sRGB table");
        FT_CU(cudaMemcpyAsync(c->srgb_lut.p, lut.data(), lut.size(), cudaMemcpyHostToDevice, c->stream),
              "upload sRGB table");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");  // the host table goes out of scope
    }
    const uint64_t src_bytes = (uint64_t)src_stride * (h - 1) + row, dst_bytes = (uint64_t)dst_stride * (h - 1) + row;
    const uint8_t* s_d = src;
    uint8_t* d_d = dst;
    if (where == FT_HOST) {
        FT_CU(c->conv_src.ensure(src_bytes), "alloc conversion source");
        FT_CU(c->conv_dst.ensure(dst_bytes), "alloc conversion output");
        FT_CU(cudaMemcpyAsync(c->conv_src.p, src, src_bytes, cudaMemcpyHostToDevice, c->stream), "upload raster");
        s_d = static_cast<const uint8_t*>(c->conv_src.p);
        d_d = static_cast<uint8_t*>(c->conv_dst.p);
    }
    const uint64_t work = (row / 16 + row % 16) * h;
    const int grid = (int)std::max<uint64_t>(
        1, std::min<uint64_t>((work + 255) / 256, (uint64_t)c->sm_count * ftc::convert_blocks_per_sm()));
    c->comp_timed = false;
    FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
    FT_CU(ftc::launch_convert(src_fmt, s_d, src_stride, d_d, dst_stride, w, h,
                              static_cast<const uint8_t*>(c->srgb_lut.p), grid, c->stream),
          "launch conversion");
    FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
    c->timed = true;
    c->launches++;
    if (where == FT_HOST) {
        FT_CU(cudaMemcpyAsync(dst, d_d, dst_bytes, cudaMemcpyDeviceToHost, c->stream), "download raster");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    }
    return FT_OK;
}

static int srcover_call(ft_ctx* c, bool backward, const float* cov, uint32_t n_layers, uint64_t plane,
                        const float* clr, const float* init, float* out, const float* grad_out, float* grad_cov,
                        float* grad_init, uint32_t n_px) {
    if (!c) return FT_ERR_ARG;
    if (n_px == 0) return FT_OK;
    if ((n_layers && (!cov || !clr)) || (!backward && !out) || (backward && (!grad_out || (n_layers && !grad_cov))) ||
        (n_layers > 1 && plane < n_px))
        return fail(c, FT_ERR_ARG, "bad SrcOver arguments");
    const uintptr_t v4 = reinterpret_cast<uintptr_t>(clr) | reinterpret_cast<uintptr_t>(init) |
                         reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(grad_out) |
                         reinterpret_cast<uintptr_t>(grad_init);
    if (v4 & 15) return fail(c, FT_ERR_ARG, "colour and canvas buffers need 16-byte alignment");
    FT_CU(cudaSetDevice(c->device), "set device");
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((n_px + 255) / 256, (uint64_t)c->sm_count * 16));
    c->comp_timed = false;
    FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
    FT_CU(ftc::launch_srcover(backward, cov, n_layers, plane, reinterpret_cast<const float4*>(clr),
                              reinterpret_cast<const float4*>(init), reinterpret_cast<float4*>(out),
                              reinterpret_cast<const float4*>(grad_out), grad_cov, reinterpret_cast<float4*>(grad_init),
                              n_px, grid, c->stream),
          "launch SrcOver");
    FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
    c->timed = true;
    c->launches++;
    return FT_OK;
}

FT_API int ft_srcover_forward(ft_ctx* c, const float* cov, uint32_t n_layers, uint64_t plane_floats, const float* clr,
                              const float* init, float* out, uint32_t n_px) {
    return srcover_call(c, false, cov, n_layers, plane_floats, clr, init, out, nullptr, nullptr, nullptr, n_px);
}

FT_API int ft_srcover_backward(ft_ctx* c, const float* cov, uint32_t n_layers, uint64_t plane_floats,
                               const float* clr, const float* init, const float* grad_out, float* grad_cov,
                               float* grad_init, uint32_t n_px) {
    return srcover_call(c, true, cov, n_layers, plane_floats, clr, init, nullptr, grad_out, grad_cov, grad_init,
                        n_px);
}

// ------------------------------------------------ differentiable ordered composite
}  // extern "C"

// Saved state between ft_stroke_composite_forward and ft_stroke_composite_backward:
// copies of the ops and colours, the canvas before each chunk of strokes, and the
// coverage of the chunk last covered.
struct ft_composite_adjoint {
    ft_ctx* ctx = nullptr;
    ft_adjoint* adj = nullptr;  // winding area and scratch of the chunk in `cov`
    DevBuf ops, clr, prefix, cov, gcov, gbuf, status, gops, gwidth;
    std::vector<ft_path_desc> h_paths, descs;
    AdjSettings set;
    uint32_t n_ops = 0, n_paths = 0, width = 0, height = 0, chunk = 1, n_chunks = 0;
    int fresh = -1;  // chunk whose coverage `cov` and `adj` hold
    bool ready = false;
    uint64_t plane_bytes() const { return 4ull * width * height; }
    uint32_t chunk_begin(uint32_t ch) const { return ch * chunk; }
    uint32_t chunk_size(uint32_t ch) const { return std::min(chunk, n_paths - ch * chunk); }
    float4* prefix_at(uint32_t ch) const {
        return static_cast<float4*>(prefix.p) + (size_t)ch * width * height;
    }
};

// Coverage of chunk `ch` into `cov` (and the winding area into the inner saved state).
static int composite_cover(ft_ctx* c, ft_composite_adjoint* s, uint32_t ch) {
    const uint32_t b = s->chunk_begin(ch), k = s->chunk_size(ch);
    s->descs.resize(k);
    for (uint32_t j = 0; j < k; j++) {
        ft_path_desc d = s->h_paths[b + j];
        d.width = s->width;
        d.height = s->height;
        d.raster_offset = (uint64_t)j * s->plane_bytes();
        d.stride = 4 * s->width;
        s->descs[j] = d;
    }
    s->fresh = -1;
    int st = adjoint_forward_dev(c, s->adj, 1, FT_NONZERO, static_cast<const ft_op*>(s->ops.p), s->n_ops,
                                 s->descs.data(), k, static_cast<float*>(s->cov.p), (uint64_t)k * s->plane_bytes(),
                                 s->set, false, true);
    if (st == FT_OK) s->fresh = (int)ch;
    return st;
}

extern "C" {

FT_API int ft_stroke_composite_forward(ft_ctx* c, const ft_op* ops, uint32_t n_ops_total, const ft_path_desc* paths,
                                       uint32_t n_paths, const float* clr, uint32_t width, uint32_t height,
                                       const float* init, float* out, uint32_t chunk, int32_t where,
                                       ft_composite_adjoint** saved) {
    Stage stage_("ft_stroke_composite_forward");
    if (!c || !saved) return FT_ERR_ARG;
    if (where != FT_HOST && where != FT_DEVICE) return fail(c, FT_ERR_ARG, "bad location");
    if (width == 0 || height == 0) return fail(c, FT_ERR_ARG, "empty canvas");
    if (width > FT_MAX_WIDTH) return fail(c, FT_ERR_CAP, "canvas wider than FT_MAX_WIDTH");
    const uint64_t n_px = (uint64_t)width * height;
    if (n_px > 0xFFFFFFFFull) return fail(c, FT_ERR_CAP, "canvas of more than 2^32 pixels");
    if ((n_paths && (!paths || !clr)) || (n_ops_total && !ops) || !out) return fail(c, FT_ERR_ARG, "null pointer");
    for (uint32_t i = 0; i < n_paths; i++)
        if ((uint64_t)paths[i].op_begin + paths[i].n_ops > n_ops_total)
            return fail(c, FT_ERR_ARG, "path ops out of range");
    if (where == FT_DEVICE) {
        const uintptr_t a16 = reinterpret_cast<uintptr_t>(ops) | reinterpret_cast<uintptr_t>(clr) |
                              reinterpret_cast<uintptr_t>(init) | reinterpret_cast<uintptr_t>(out);
        if (a16 & 15) return fail(c, FT_ERR_ARG, "device ops, colours and canvases need 16-byte alignment");
    } else if (!valid_ops_host(ops, n_ops_total)) {
        return fail(c, FT_ERR_ARG, "unknown path op kind");
    }
    FT_CU(cudaSetDevice(c->device), "set device");
    ft_composite_adjoint* s = *saved;
    if (!s) {
        s = new ft_composite_adjoint();
        s->ctx = c;
        *saved = s;
    }
    if (s->ctx != c) return fail(c, FT_ERR_ARG, "saved state belongs to another context");
    s->ready = false;
    s->fresh = -1;
    s->set = ctx_settings(c);
    s->n_ops = n_ops_total;
    s->n_paths = n_paths;
    s->width = width;
    s->height = height;
    s->h_paths.assign(paths, paths + n_paths);
    const uint64_t plane = s->plane_bytes();
    if (chunk == 0) {
        // coverage and coverage gradient of a chunk in at most 60 % of the free memory
        // (160 GB at most), equal chunks.  Fewer chunks recompute less in the backward:
        // 16,384 strokes on 2048x2048 in 4 / 6 / 8 chunks measured bwd / fwd 1.98 / 2.05 / 2.05
        size_t free_b = 0, total_b = 0;
        FT_CU(cudaMemGetInfo(&free_b, &total_b), "memory info");
        // the saved state's own coverage buffers from an earlier call count as free
        const uint64_t avail = (uint64_t)free_b + s->cov.cap + s->gcov.cap;
        const uint64_t budget = std::min<uint64_t>(avail / 5 * 3, 160ull << 30);
        const uint64_t kmax = std::max<uint64_t>(1, budget / (2 * plane));
        const uint64_t nch = (std::max(n_paths, 1u) + kmax - 1) / kmax;
        chunk = (uint32_t)((std::max(n_paths, 1u) + nch - 1) / nch);
    }
    s->chunk = std::max(1u, std::min(chunk, std::max(n_paths, 1u)));
    s->n_chunks = (n_paths + s->chunk - 1) / s->chunk;
    if (!s->adj) {
        s->adj = new ft_adjoint();
        s->adj->ctx = c;
    }
    FT_CU(s->ops.ensure(sizeof(ft_op) * std::max(n_ops_total, 1u)), "alloc ops");
    FT_CU(s->clr.ensure(16ull * std::max(n_paths, 1u)), "alloc colours");
    FT_CU(s->status.ensure(4ull * std::max(n_paths, 1u)), "alloc status");
    FT_CU(s->prefix.ensure(16ull * n_px * (s->n_chunks + 1)), "alloc canvas before each chunk");
    FT_CU(s->cov.ensure(std::max<uint64_t>(plane * s->chunk, 4)), "alloc chunk coverage");
    const cudaMemcpyKind in = where == FT_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (n_ops_total) FT_CU(cudaMemcpyAsync(s->ops.p, ops, sizeof(ft_op) * n_ops_total, in, c->stream), "copy ops");
    if (n_paths) FT_CU(cudaMemcpyAsync(s->clr.p, clr, 16ull * n_paths, in, c->stream), "copy colours");
    if (init)
        FT_CU(cudaMemcpyAsync(s->prefix.p, init, 16ull * n_px, in, c->stream), "copy initial canvas");
    else
        FT_CU(cudaMemsetAsync(s->prefix.p, 0, 16ull * n_px, c->stream), "clear initial canvas");
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((n_px + 255) / 256, (uint64_t)c->sm_count * 16));
    c->comp_timed = false;
    FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
    for (uint32_t ch = 0; ch < s->n_chunks; ch++) {
        int st = composite_cover(c, s, ch);
        if (st != FT_OK) return st;
        const uint32_t b = s->chunk_begin(ch), k = s->chunk_size(ch);
        FT_CU(cudaMemcpyAsync(static_cast<int32_t*>(s->status.p) + b, s->adj->status.p, 4ull * k,
                              cudaMemcpyDeviceToDevice, c->stream),
              "copy status");
        FT_CU(ftc::launch_srcover(false, static_cast<const float*>(s->cov.p), k, plane / 4,
                                  static_cast<const float4*>(s->clr.p) + b, s->prefix_at(ch), s->prefix_at(ch + 1),
                                  nullptr, nullptr, nullptr, (uint32_t)n_px, grid, c->stream),
              "launch SrcOver");
        c->launches++;
    }
    FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
    c->timed = true;
    FT_CU(cudaMemcpyAsync(out, s->prefix_at(s->n_chunks), 16ull * n_px,
                          where == FT_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, c->stream),
          "copy canvas");
    if (where == FT_HOST) FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    s->ready = true;
    return FT_OK;
}

FT_API int ft_stroke_composite_backward(ft_ctx* c, ft_composite_adjoint* s, const float* grad_out, float* grad_ops,
                                        float* grad_width, float* grad_init, int32_t where) {
    Stage stage_("ft_stroke_composite_backward");
    if (!c || !s) return FT_ERR_ARG;
    if (!s->ready) return fail(c, FT_ERR_ARG, "backward without a forward");
    if (s->ctx != c) return fail(c, FT_ERR_ARG, "saved state belongs to another context");
    if (where != FT_HOST && where != FT_DEVICE) return fail(c, FT_ERR_ARG, "bad location");
    if (!grad_out || (s->n_ops && !grad_ops)) return fail(c, FT_ERR_ARG, "null pointer");
    if (where == FT_DEVICE) {
        const uintptr_t a16 = reinterpret_cast<uintptr_t>(grad_out) | reinterpret_cast<uintptr_t>(grad_init);
        if ((a16 & 15) || (reinterpret_cast<uintptr_t>(grad_ops) & 3) || (reinterpret_cast<uintptr_t>(grad_width) & 3))
            return fail(c, FT_ERR_ARG, "device canvases need 16-byte alignment, gradients 4-byte alignment");
    }
    FT_CU(cudaSetDevice(c->device), "set device");
    const uint64_t n_px = (uint64_t)s->width * s->height, plane = s->plane_bytes();
    const size_t gops_bytes = 24ull * s->n_ops;
    FT_CU(s->gcov.ensure(std::max<uint64_t>(plane * s->chunk, 4)), "alloc chunk coverage gradient");
    FT_CU(s->gbuf.ensure(32ull * n_px), "alloc canvas gradients");
    float* gops_d = grad_ops;
    float* gw_d = grad_width;
    if (where == FT_HOST || !grad_ops) {
        FT_CU(s->gops.ensure(std::max<size_t>(gops_bytes, 4)), "alloc op gradient");
        gops_d = static_cast<float*>(s->gops.p);
    }
    if (where == FT_HOST || !grad_width) {
        FT_CU(s->gwidth.ensure(4ull * std::max(s->n_paths, 1u)), "alloc width gradient");
        gw_d = static_cast<float*>(s->gwidth.p);
    }
    float4* g_cur = static_cast<float4*>(s->gbuf.p);
    float4* g_next = g_cur + n_px;
    FT_CU(cudaMemcpyAsync(g_cur, grad_out, 16ull * n_px,
                          where == FT_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, c->stream),
          "copy canvas gradient");
    if (gops_bytes) FT_CU(cudaMemsetAsync(gops_d, 0, gops_bytes, c->stream), "reset op gradient");
    if (s->n_paths) FT_CU(cudaMemsetAsync(gw_d, 0, 4ull * s->n_paths, c->stream), "reset width gradient");
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((n_px + 255) / 256, (uint64_t)c->sm_count * 16));
    c->comp_timed = false;
    FT_CU(cudaEventRecord(c->ev0, c->stream), "event");
    for (uint32_t ch = s->n_chunks; ch-- > 0;) {
        if (s->fresh != (int)ch) {  // recompute this chunk's coverage
            int st = composite_cover(c, s, ch);
            if (st != FT_OK) return st;
        }
        const uint32_t b = s->chunk_begin(ch), k = s->chunk_size(ch);
        FT_CU(ftc::launch_srcover(true, static_cast<const float*>(s->cov.p), k, plane / 4,
                                  static_cast<const float4*>(s->clr.p) + b, s->prefix_at(ch), nullptr, g_cur,
                                  static_cast<float*>(s->gcov.p), g_next, (uint32_t)n_px, grid, c->stream, true),
              "launch SrcOver adjoint");
        c->launches++;
        int st = adjoint_backward_dev(c, s->adj, static_cast<const float*>(s->gcov.p), gops_d, gw_d + b, false);
        if (st != FT_OK) return st;
        std::swap(g_cur, g_next);
    }
    FT_CU(cudaEventRecord(c->ev1, c->stream), "event");
    c->timed = true;
    const cudaMemcpyKind outk = where == FT_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (grad_init) FT_CU(cudaMemcpyAsync(grad_init, g_cur, 16ull * n_px, outk, c->stream), "copy initial gradient");
    if (where == FT_HOST) {
        if (gops_bytes) FT_CU(cudaMemcpyAsync(grad_ops, gops_d, gops_bytes, outk, c->stream), "download op gradient");
        if (grad_width && s->n_paths)
            FT_CU(cudaMemcpyAsync(grad_width, gw_d, 4ull * s->n_paths, outk, c->stream), "download width gradient");
        FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    }
    return FT_OK;
}

FT_API int ft_stroke_composite_status(ft_ctx* c, ft_composite_adjoint* s, int32_t* status, uint32_t n) {
    if (!c || !s || (n && !status)) return FT_ERR_ARG;
    FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    const uint32_t k = std::min(n, s->ready ? s->n_paths : 0u);
    if (k) FT_CU(cudaMemcpy(status, s->status.p, sizeof(int32_t) * k, cudaMemcpyDeviceToHost), "status");
    for (uint32_t i = k; i < n; i++) status[i] = FT_OK;
    return FT_OK;
}

FT_API uint32_t ft_stroke_composite_chunk(ft_composite_adjoint* s) { return s ? s->chunk : 0; }

FT_API void ft_stroke_composite_destroy(ft_composite_adjoint* s) {
    if (!s) return;
    if (s->ctx) {
        cudaSetDevice(s->ctx->device);
        if (s->ctx->stream) cudaStreamSynchronize(s->ctx->stream);
    }
    ft_adjoint_destroy(s->adj);
    DevBuf* bufs[] = {&s->ops, &s->clr, &s->prefix, &s->cov, &s->gcov, &s->gbuf, &s->status, &s->gops, &s->gwidth};
    for (DevBuf* b : bufs) b->release();
    delete s;
}

FT_API int ft_autotune_batch(ft_ctx* c, int32_t stroke, int32_t rule, const ft_op* ops, uint32_t n_ops_total,
                             const ft_path_desc* paths, uint32_t n_paths, int32_t fmt, uint8_t* rasters,
                             uint64_t raster_bytes, const char* cache_path, ft_tuning* chosen, float* ms_out) {
    Stage stage_("ft_autotune_batch");
    if (!c) return FT_ERR_ARG;
    if (n_paths && !paths) return fail(c, FT_ERR_ARG, "null path list");
    for (uint32_t i = 0; i < n_paths; i++) {
        int st = check_path(c, paths[i], fmt, raster_bytes, n_ops_total);
        if (st != FT_OK) return st;
    }
    if (ms_out) *ms_out = 0.0f;
    const std::string key = tune_key(c, stroke, rule, fmt, paths, n_paths);
    ft_tuning best{0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (tune_lookup(cache_path, key, &best) && ft_set_tuning(c, &best) == FT_OK) {
        if (chosen) *chosen = best;
        return FT_OK;
    }
    const ft_tuning saved = c->tune;
    const bool saved_tuned = c->tuned;
    // candidate plans: the built-in plan first, then canvas side of the warp/CTA split x
    // CTA tile height (shared memory) x resident CTAs per SM.  A candidate replaces the
    // plan in hand only when it is faster by more than the timing noise (1 %): a knob the
    // batch never exercises (the CTA tile of a batch that only the warp rasteriser draws)
    // keeps its built-in value.
    const int sides[] = {ftk::WARP_MAX_SIDE, 0, 64, 128, 256, 512};
    const int smems[] = {0, 40 * 1024, 48 * 1024, 64 * 1024, 96 * 1024};
    const int grids[] = {0, 2};
    float best_ms = 0.0f;
    bool have = false;
    cudaEvent_t e0, e1;
    FT_CU(cudaEventCreate(&e0), "event");
    FT_CU(cudaEventCreate(&e1), "event");
    for (int si = 0; si < (int)(sizeof(sides) / sizeof(sides[0])); si++)
        for (int mi = 0; mi < (int)(sizeof(smems) / sizeof(smems[0])); mi++)
            for (int gp : grids) {
                const int ws = sides[si], sm = smems[mi];
                const bool builtin = si == 0 && mi == 0 && gp == 0;
                // the built-in side and shared memory appear once, in the built-in plan
                if (!builtin && (si == 0 || mi == 0)) continue;
                if (sm > c->max_smem) continue;
                // the batch plan's knobs; the composite and host-transfer knobs stay as set
                c->tune = ft_tuning{ws, sm, builtin ? 0 : 1 << 20, gp, saved.band_rows, saved.pool_edges,
                                    saved.host_chunks, saved.host_mapped, saved.tile_w, saved.tile_stage,
                                    saved.fig_build};
                c->tuned = true;
                ft_batch* b = nullptr;
                if (ft_batch_create(c, stroke, rule, paths, n_paths, fmt, &b) != FT_OK) continue;
                bool ok = ft_batch_launch(c, b, ops, n_ops_total, rasters, raster_bytes) == FT_OK;  // warm-up
                float total = 0.0f;
                const int reps = 3;
                if (ok) ok = cudaEventRecord(e0, c->stream) == cudaSuccess;
                for (int r = 0; ok && r < reps; r++)
                    ok = ft_batch_launch(c, b, ops, n_ops_total, rasters, raster_bytes) == FT_OK;
                if (ok)
                    ok = cudaEventRecord(e1, c->stream) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
                         cudaEventElapsedTime(&total, e0, e1) == cudaSuccess;
                ft_batch_destroy(b);
                if (!ok) continue;
                const float ms = total / reps;
                if (!have || ms < 0.99f * best_ms) {
                    best_ms = ms;
                    best = c->tune;
                    have = true;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!have) {
        c->tune = saved;
        c->tuned = saved_tuned;
        return fail(c, FT_ERR_CUDA, "no candidate plan ran");
    }
    c->tune = best;
    c->tuned = true;
    if (cache_path) {
        FILE* f = fopen(cache_path, "a");
        if (f) {
            fprintf(f, "%s %d %d %d %d %d %d %d %d %d %d %.4f\n", key.c_str(), best.warp_max_side,
                    best.cta_smem_bytes, best.split_px, best.grid_per_sm, best.band_rows, best.pool_edges,
                    best.host_chunks, best.host_mapped, best.tile_w, best.tile_stage, best_ms);
            fclose(f);
        }
    }
    if (chosen) *chosen = best;
    if (ms_out) *ms_out = best_ms;
    return FT_OK;
}

FT_API int ft_batch_status(ft_ctx* c, int32_t* status, uint32_t n) {
    if (!c || (n && !status)) return FT_ERR_ARG;
    FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    const uint32_t k = std::min(n, c->last_n_paths);
    if (k) FT_CU(cudaMemcpy(status, c->status.p, sizeof(int32_t) * k, cudaMemcpyDeviceToHost), "status");
    for (uint32_t i = k; i < n; i++) status[i] = FT_OK;
    return FT_OK;
}

FT_API int ft_sync(ft_ctx* c) {
    if (!c) return FT_ERR_ARG;
    FT_CU(cudaStreamSynchronize(c->stream), "synchronize");
    return FT_OK;
}

FT_API const char* ft_last_error(ft_ctx* c) {
    if (!c) return "null context";
    return c->err.c_str();
}

FT_API int ft_last_timings(ft_ctx* c, float* kernel_ms) {
    if (!c || !kernel_ms) return FT_ERR_ARG;
    *kernel_ms = 0.f;
    if (!c->timed) return FT_OK;
    FT_CU(cudaEventSynchronize(c->ev1), "event sync");
    FT_CU(cudaEventElapsedTime(kernel_ms, c->ev0, c->ev1), "event time");
    return FT_OK;
}

FT_API int ft_last_composite_ms(ft_ctx* c, float* ms) {
    if (!c || !ms) return FT_ERR_ARG;
    *ms = 0.f;
    if (!c->timed || !c->comp_timed) return FT_OK;
    FT_CU(cudaEventSynchronize(c->ev1), "event sync");
    FT_CU(cudaEventElapsedTime(ms, c->ev_comp, c->ev1), "event time");
    return FT_OK;
}

FT_API uint64_t ft_launch_count(ft_ctx* c) { return c ? c->launches : 0; }

}  // extern "C"
