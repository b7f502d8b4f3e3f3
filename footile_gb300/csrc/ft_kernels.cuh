// ft_kernels.cuh — launch interface between the C ABI (ft_capi.cu) and the kernels.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/footile_gpu.h"

namespace ftk {

constexpr int BLOCK = 256;                 // threads per CTA
constexpr int NWARP = BLOCK / 32;
constexpr int RAW_CAP = 2048;              // raw (pre-dedupe) vertices per compaction window
constexpr int PT_CAP = FT_MAX_POINTS;      // vertices kept per figure (u16 vertex ids)
constexpr int OUT_CAP = 2 * RAW_CAP;       // stroke outline points staged per window

// One unit of the device work queue: rows [row_begin, row_end) of one path's
// raster, rasterised `band_rows` rows at a time.
struct WorkItem {
    uint32_t path;
    uint32_t row_begin;
    uint32_t row_end;
    uint32_t band_rows;
};

// One non-horizontal edge of a figure (footile fig.rs:47-66), 32 bytes.  `ed` is
// +1 when the edge direction equals the figure direction, -1 otherwise, 0 for
// "no edge" (horizontal or degenerate segment).
struct __align__(16) EdgeRec {
    int y_upper, y_lower, x_bot0, inv_slope;
    int step_pix, ed, start_row, end_row;
};

// One stroke sub-path (stroker.rs:31-40).
struct SubRec {
    int start;     // first stroke point
    int n;         // points
    int joined;    // joined ends
    int len;       // SubStroke::len() (u16 arithmetic)
    int item_off;  // first outline item of this sub-stroke
    int pad[3];
};

// Per-CTA scratch in global memory, private to one resident CTA and reused for
// every work item it takes (stays L2-resident for small figures).  Every array
// starts on a 256-byte boundary.
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t SCR_PTS = 0;                                                   // int2[PT_CAP] vertices
constexpr size_t SCR_SS = align256(SCR_PTS + (size_t)PT_CAP * sizeof(int2));    // int[PT_CAP] sub-figure starts
constexpr size_t SCR_EDGES = align256(SCR_SS + (size_t)PT_CAP * sizeof(int));   // EdgeRec[PT_CAP]
constexpr size_t SCR_SPTS = align256(SCR_EDGES + (size_t)PT_CAP * sizeof(EdgeRec));  // float4[PT_CAP] stroke points
constexpr size_t SCR_SUBS = align256(SCR_SPTS + (size_t)PT_CAP * sizeof(float4));    // SubRec[PT_CAP] sub-strokes
constexpr size_t SCR_SOFF = align256(SCR_SUBS + (size_t)PT_CAP * sizeof(SubRec));    // int[2*PT_CAP+8] offsets
// Raw (pre-dedupe) vertices of one chunk of ops, emitted once by all threads and
// compacted window by window (CTA figure builds): positions as int2 (fills) or float4
// with the width (strokes), sub-figure start flags, stroke join flags, source ops.
constexpr int RAWG = 32768;
constexpr size_t SCR_RAWG = align256(SCR_SOFF + (size_t)(2 * PT_CAP + 8) * sizeof(int));  // float4[RAWG]
constexpr size_t SCR_RSG = align256(SCR_RAWG + (size_t)RAWG * 16);                         // u8[RAWG]
constexpr size_t SCR_JPG = align256(SCR_RSG + (size_t)RAWG);                               // u8[RAWG]
constexpr size_t SCR_OPIG = align256(SCR_JPG + (size_t)RAWG);                              // int[RAWG]
constexpr size_t SCRATCH_BYTES_PER_CTA = align256(SCR_OPIG + (size_t)RAWG * sizeof(int));

// Scratch layout of one CTA figure build for figures of up to `cap` vertices: the
// SCR_* layout above for footile's cap, larger for the un-capped extension (fills).
struct ScrLayout {
    size_t pts, ss, edges, spts, subs, soff, rawg, rsg, jpg, opig, bytes;
};
constexpr ScrLayout scr_layout(size_t cap) {
    ScrLayout L{};
    L.pts = 0;
    L.ss = align256(L.pts + cap * sizeof(int2));
    L.edges = align256(L.ss + cap * sizeof(int));
    L.spts = align256(L.edges + cap * sizeof(EdgeRec));
    L.subs = align256(L.spts + (size_t)PT_CAP * sizeof(float4));
    L.soff = align256(L.subs + (size_t)PT_CAP * sizeof(SubRec));
    L.rawg = align256(L.soff + (size_t)(2 * PT_CAP + 8) * sizeof(int));
    L.rsg = align256(L.rawg + (size_t)RAWG * 16);
    L.jpg = align256(L.rsg + (size_t)RAWG);
    L.opig = align256(L.jpg + (size_t)RAWG);
    L.bytes = align256(L.opig + (size_t)RAWG * sizeof(int));
    return L;
}
static_assert(scr_layout(PT_CAP).bytes == SCRATCH_BYTES_PER_CTA && scr_layout(PT_CAP).rawg == SCR_RAWG &&
                  scr_layout(PT_CAP).edges == SCR_EDGES && scr_layout(PT_CAP).subs == SCR_SUBS,
              "scratch layouts agree");
// Largest figure of the un-capped extension (ft_set_figure_cap).
constexpr uint32_t FIG_CAP_MAX = 1u << 26;

// Warp rasteriser (one warp per small path): per-warp share of the CTA scratch.
constexpr int WARP_CAP = 8191;        // vertices a warp holds; larger figures go to a CTA
constexpr int WARP_MAX_SIDE = 512;    // canvases up to this width and height use the warp rasteriser
static_assert(WARP_MAX_SIDE <= 1023, "sweep records hold rows below 1023");
constexpr size_t WS_PTS = 0;
constexpr size_t WS_SS = align256(WS_PTS + (size_t)WARP_CAP * sizeof(int2));
constexpr size_t WS_SORT = align256(WS_SS + (size_t)WARP_CAP * sizeof(int));     // sweep records by start row
constexpr size_t WS_ACT = align256(WS_SORT + (size_t)WARP_CAP * sizeof(int4));
constexpr size_t WS_BYTES = align256(WS_ACT + (size_t)WARP_CAP * sizeof(int4));  // active sweep records
constexpr int SWEEP_END_FAR = 1023;  // sweep record end row: beyond the warp's last row
static_assert(NWARP * WS_BYTES <= SCRATCH_BYTES_PER_CTA, "warp scratch layout");

// Grid-wide figure build of one fill path (launch_grid_build): per-op and per-raw-vertex
// arrays in one device buffer laid out by gb_layout.
constexpr int GB_PER = 4;                      // raw vertices per thread of the tile kernels
constexpr int GB_TILE = GB_PER * BLOCK;        // raw vertices per tile
constexpr int GB_TOP_BLOCKS = 512;             // CTAs of the top-vertex search
constexpr int GB_D0 = 3;                       // an op's curve walk is split at this depth
constexpr int GB_LANES = 1 << GB_D0;           // threads per op of the count and emit walks
constexpr int GB_OPB = BLOCK / GB_LANES;       // ops per CTA of the count and emit walks
constexpr long long GB_RAW_MAX = 1ll << 29;    // raw vertices the grid build takes at most
struct GridBuildBufs {
    const ft_op* ops;   // the path's ops
    int n_ops;
    float s_width;      // pen width before the path
    int raw_cap;        // raw vertices the arrays hold (a multiple of GB_TILE)
    unsigned* done;     // [8] tickets: the last CTA of a kernel to finish runs its scan
    long long* n_raw;   // raw vertices of the path
    int* count;         // vertices kept
    int4* opa;          // per 256 ops: last Move/Line/Quad/Cubic/Close op, last PenWidth op, last Close/Move op
    int* opw;           // per op: last PenWidth op at or before it in its 256 (strokes)
    long long* opn;     // per GB_OPB ops: raw vertices
    int2* opi;          // per op: last Move/Line/Quad/Cubic/Close op before it in its 256, raw offset in its GB_OPB
    int* opl;           // per op and lane: the lane's raw offset in the op
    int2* raw;          // raw vertices, 16.16
    unsigned char* fl;  // per raw vertex: 1 = starts a sub-figure
    unsigned char* kp;  // per raw vertex: 1 = kept, 2 = pops its sub-figure's first vertex
    int* rk;            // per raw vertex: the first raw vertex of its sub-figure
    int* tr;            // per tile: last sub-figure start
    int4* tp;           // per tile: position aggregate (kept - popped, runs, max prefix)
    int4* top;          // per CTA of the top-vertex search: min (y, x, id)
    int* final_flag;    // nullable: set when the cap is reached (the figure is complete)
    const int* skip;    // nullable: the kernels after k_gb_ops do nothing when *skip is set
};
// Grid-wide build of one stroke path (the stroker's points, sub-strokes and outline, then
// the outline's figure through the fill build's k_gb_keep / k_gb_write / k_gb_top).
constexpr int GS_ITEMS_CAP = 6 * PT_CAP + 256;  // outline items of 65,535 stroke points at most
struct GridStrokeBufs {
    int sraw_cap;        // raw stroke points the arrays hold (a multiple of GB_TILE)
    long long* n_sraw;   // raw stroke points of the path
    int* st;             // [0] points kept, [1] sub-strokes, [2] op of the last kept point, [3] last
                         // Move/Line/Quad/Cubic/Close op, [4] last Close/Move op, [5] outline items,
                         // [6] the 65,535-point cap was reached
    unsigned* done;      // [8] tickets
    float4* raw4;        // raw stroke points: x, y, width
    unsigned char* sfl;  // per raw point: 1 starts a sub-stroke, 2 its op is not a Move
    int* sopi;           // per raw point: its op
    int2* stile;         // per tile of raw points: kept, sub-stroke starts
    int* subt;           // per 256 sub-strokes: outline items
    int* itoff;          // per outline item: raw offset in its 256
    int* itc;            // per 256 outline items: raw vertices
    int* final_flag;     // nullable: set when the 65,535-point cap is reached (the points are complete)
    const int* skip;     // nullable: the stroke point kernels do nothing when *skip is set
};
struct GbLayout {
    size_t state, opa, opw, opn, opi, opl, raw, fl, kp, rk, tr, tr2, tp, top;
    size_t raw4, sfl, sopi, stile, subt, itoff, itc, bytes;
};
constexpr GbLayout gb_layout(size_t n_ops, size_t raw_cap, size_t sraw_cap = 0) {
    GbLayout g{};
    const size_t nbo = (n_ops + BLOCK - 1) / BLOCK, nbw = (n_ops + GB_OPB - 1) / GB_OPB,
                 ntiles = raw_cap / GB_TILE;
    // two builds' done[8] at 0 / 128, n_raw at 32 / 160, count at 40 / 168, final at 44 / 172;
    // a stroke build's st[] at 128, n_sraw at 160, done[] at 192, its probe's n_sraw at 256,
    // done[] at 288, final at 320
    g.state = 0;
    g.opa = 512;
    g.opw = align256(g.opa + nbo * 16);
    g.opn = align256(g.opw + n_ops * 4);
    g.opi = align256(g.opn + nbw * 8);
    g.opl = align256(g.opi + n_ops * 8);
    g.raw = align256(g.opl + n_ops * GB_LANES * 4);
    g.fl = align256(g.raw + raw_cap * 8);
    g.kp = align256(g.fl + raw_cap);
    g.rk = align256(g.kp + raw_cap);
    g.tr = align256(g.rk + raw_cap * 4);
    g.tr2 = align256(g.tr + ntiles * 4);
    g.tp = align256(g.tr2 + ntiles * 4);
    g.top = align256(g.tp + ntiles * 16);
    g.raw4 = align256(g.top + (size_t)GB_TOP_BLOCKS * 16);
    g.sfl = align256(g.raw4 + sraw_cap * 16);
    g.sopi = align256(g.sfl + sraw_cap);
    g.stile = align256(g.sopi + sraw_cap * 4);
    g.subt = align256(g.stile + sraw_cap / GB_TILE * 8);
    g.itoff = align256(g.subt + (sraw_cap ? (size_t)(PT_CAP / BLOCK + 1) * 4 : 0));
    g.itc = align256(g.itoff + (sraw_cap ? (size_t)GS_ITEMS_CAP * 4 : 0));
    g.bytes = align256(g.itc + (sraw_cap ? (size_t)(GS_ITEMS_CAP / BLOCK + 1) * 4 : 0));
    return g;
}

struct KParams {
    const ft_op* ops;
    const ft_path_desc* paths;
    const WorkItem* items;   // CTA work items (large paths, row ranges)
    uint32_t n_items;
    const WorkItem* items_w; // warp work items (small paths, whole rasters)
    uint32_t n_items_w;
    uint32_t* overflow;      // paths a warp handed over to the CTA kernel
    uint32_t* queue;         // [0]: next CTA item, [1]: next warp item, [2]: overflow count
    uint8_t* rasters;
    int32_t* status;         // per path, atomicMax of FT_ERR_* codes
    float* sw_out;           // per path pen width after the call (nullable)
    int host_rasters;        // rasters are mapped host memory: Matte8 rows go out as aligned words
    const float* sw_chain;   // nullable: initial pen width of every path
    unsigned char* scratch;  // gridDim.x * SCRATCH_BYTES_PER_CTA bytes
    float xf[6];
    float tol_sq;
    int join;
    float miter_limit;
    float miter_g;           // ft_miter_angle(miter_limit): the miter decision's threshold on |th/2|
    int rule;
    int fmt;
    int stroke;
    int smem_bytes;
    // ordered composite of all paths onto one raster (ft_composite_batch)
    uint32_t canvas_w, canvas_h, canvas_stride;
    int band_rows;               // rows per band
    int n_bands;
    EdgeRec* pool;               // binned edges of all paths
    unsigned long long* pool_used;  // bump counter (edges)
    unsigned long long pool_cap;    // edges
    int* bandoff;                // per path: n_bands + 1 offsets into its pool run
    int4* crec;                  // per path: rowbegin, tmin, pool offset lo, pool offset hi
    // figure builds of the ordered compositor (k_cbuild): vertex cap and scratch layout
    int pt_cap;                  // PT_CAP, or more for un-capped fills
    ScrLayout L;                 // scr_layout(pt_cap); gridDim.x * L.bytes of scratch
    // one path (split_bin): k_cbuild stops after the figure and its direction, the
    // grid-wide kernels below build and bin its edges
    int split_bin;
    int4* fig_state;             // count, direction, top row, edges fit the pool
    int* bin_hist;               // n_bands counts, then n_bands fill cursors
    // Rgba8p tile compositor (k_ctile): tile width in pixels (128, 256, 512 or 1024) and
    // whether the canvas is staged by TMA through the tensor map passed beside these
    int seg_w;
    int use_tma;
    // one fill path built over the whole GPU (launch_grid_build) instead of by k_cbuild
    GridBuildBufs gb;
    GridStrokeBufs gs;  // and the stroker's part of one stroke path (launch_grid_stroke)
};

// Ordered composite: per-path figure build and edge binning, then one CTA per band.
// `few_ctas`: at most one CTA per SM — prefer L1 over shared memory (the curve walks'
// stacks are in local memory).
cudaError_t launch_composite_build(const KParams& p, int grid, int smem_bytes, cudaStream_t s, bool few_ctas);
cudaError_t launch_composite_bands(const KParams& p, int smem_bytes, cudaStream_t s);
// Rgba8p: tiles of band_rows x seg_w pixels, canvas staged through `tmap` when use_tma.
cudaError_t launch_composite_tiles(const KParams& p, const CUtensorMap& tmap, cudaStream_t s);
int composite_tile_smem(int band_rows, int seg_w, bool staged);
// SrcOver of one call's colour onto the canvas rows r0.. from its Matte8 coverage `mask`
// (both as 2-D tensor maps with boxes of SO_COLS x SO_ROWS elements: the kernel's stage
// size and its expected transaction bytes derive from the same two constants), streamed
// by TMA.
constexpr int SO_ROWS = 8, SO_COLS = 256;
cudaError_t launch_srcover_mask(const CUtensorMap& canvas, const CUtensorMap& mask, int W, int H, int r0,
                                unsigned clr, int32_t* status, int sm_count, cudaStream_t s);
// Edges and band bins of a single path's figure (after k_cbuild with split_bin), over
// the whole GPU: edge records and band counts, a scan and pool allocation, the fill.
cudaError_t launch_figure_bins(const KParams& p, int grid, cudaStream_t s);
// The figure of one fill path (p.gb's ops) over the whole GPU, in place of k_cbuild with
// split_bin: vertices and sub-figure starts into CTA 0's scratch, fig_state[0], the pen
// width after the path and the path's status.  p.gb's state (done, n_raw, count) must be
// zero and tr all -1 (bytes 0xFF) before the launch.  When the path has more raw
// vertices than p.gb.raw_cap, *n_raw says how many and nothing else is written but a
// figure of no vertices; the caller grows the arrays and builds again.  `probe`
// (nullable): the same build over a prefix of the ops first (its own state and tr, its
// final_flag the full build's skip): when the cap is reached within the prefix the figure
// is complete and the full build does nothing.
cudaError_t launch_grid_build(const KParams& p, int sm_count, cudaStream_t s, const KParams* probe = nullptr);
// The same for one stroke path (p.gb and p.gs): stroke points, sub-strokes and outline over
// the whole GPU, then the outline's figure as launch_grid_build builds a fill's.  p.gs's
// state (st, n_sraw, done) must be zero before the launch, as p.gb's.  When the path has
// more raw stroke points than p.gs.sraw_cap, or its outline more raw vertices than
// p.gb.raw_cap, *n_sraw / *n_raw say how many and the figure is empty.
// `probe` (nullable): the stroke points first over a prefix of the ops (its own n_sraw,
// done and final_flag, the full build's skip): when the point cap is reached there the
// points are complete and the full build's point kernels do nothing.
cudaError_t launch_grid_stroke(const KParams& p, int sm_count, cudaStream_t s, const KParams* probe = nullptr);
int composite_bands_smem(int band_rows, int width);
int composite_build_blocks_per_sm(int smem_bytes, bool stroke);

// Static shared memory of the kernel besides the dynamic area buffer.
constexpr int RASTER_FIXED_SMEM = BLOCK * (int)sizeof(EdgeRec) + 3 * BLOCK * 4 + 256 + 4096;

// Launch the persistent rasteriser.  Returns the CUDA error of the launch.
cudaError_t launch_raster(const KParams& p, int grid, int smem_bytes, cudaStream_t s, bool few_ctas);
// Launch the warp rasteriser (small paths).  Its dynamic shared memory is fixed.
cudaError_t launch_raster_warp(const KParams& p, int grid, cudaStream_t s);
int raster_warp_smem();
int raster_warp_blocks_per_sm();

// Resident CTAs per SM for `smem_bytes` of dynamic shared memory.
int raster_blocks_per_sm(int smem_bytes, bool stroke);

// Maximum dynamic shared memory the kernel may be configured for.
int raster_max_smem();

}  // namespace ftk
