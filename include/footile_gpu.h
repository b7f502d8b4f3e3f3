/*
 * footile_gpu.h — C ABI of the GB300 (sm_103a) fill/stroke rasterisation path.
 *
 * This library replaces the body of footile's `Plotter::fill` / `Plotter::stroke`
 * (src/plotter.rs:339-365) — path walk, De Casteljau flattening, stroking, the
 * fixed-point `Fig` rasteriser and the 8-bit resolve/composite — with CUDA kernels.
 * Results are bit-identical to the CPU algorithm (16.16 fixed point, release-mode
 * wrapping arithmetic, IEEE f32 without contraction in the float stages).
 *
 * Plain C types only: pointers, sizes and small structs.  Every call returns an
 * `int` status (FT_OK or an FT_ERR_* code); `ft_last_error` gives a message.
 * The caller owns every buffer it passes; the library never frees them.
 * One context per host thread; a context issues all work on one CUDA stream.
 */
#ifndef FOOTILE_GPU_H
#define FOOTILE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define FT_API __declspec(dllexport)
#else
#define FT_API __attribute__((visibility("default")))
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
    FT_OK = 0,
    FT_ERR_ARG = 1,      /* bad argument, or a curve with a non-finite control point */
    FT_ERR_DEPTH = 2,    /* curve / arc subdivision reached FT_MAX_DEPTH levels       */
    FT_ERR_CAP = 3,      /* a size limit of the library was exceeded                  */
    FT_ERR_TIMEOUT = 4,  /* a bounded device wait gave up                             */
    FT_ERR_CUDA = 5,     /* a CUDA runtime call failed                                */
    FT_ERR_NOMEM = 6     /* device or pinned host allocation failed                   */
};

/* Maximum De Casteljau / round-join arc recursion depth.  footile recurses without
 * a limit (README.md:32-33); deeper subdivisions are emitted as leaves and flagged. */
#define FT_MAX_DEPTH 22
/* Single fill and stroke paths of at least this many ops build their figure over the
 * whole GPU (ft_tuning.fig_build). */
#define FT_GRID_BUILD_OPS 2048

/* Vertices kept per figure, from `Vid(u16)` (src/vid.rs:9-18, src/fig.rs:428-442). */
#define FT_MAX_POINTS 65535

/* Widest raster row the band rasteriser accepts (one row of i32 cell areas must fit
 * in shared memory). */
#define FT_MAX_WIDTH 16384

/* ---- path operations: footile `PathOp` (src/path.rs:18-31) ------------- */
enum {
    FT_OP_CLOSE = 0,     /* PathOp::Close()                        */
    FT_OP_MOVE = 1,      /* PathOp::Move(p)           v[0..2] = p  */
    FT_OP_LINE = 2,      /* PathOp::Line(p)           v[0..2] = p  */
    FT_OP_QUAD = 3,      /* PathOp::Quad(b, c)        v[0..4]      */
    FT_OP_CUBIC = 4,     /* PathOp::Cubic(b, c, d)    v[0..6]      */
    FT_OP_PEN_WIDTH = 5  /* PathOp::PenWidth(w)       v[0] = w     */
};

/* One path operation, 32 bytes.  Points are absolute (Path2D resolves relative
 * coordinates while building, src/path.rs:80-86). */
typedef struct ft_op {
    int32_t kind;
    float v[6];
    int32_t reserved;
} ft_op;

/* ---- fill rules, joins, pixel formats -------------------------------- */
enum { FT_NONZERO = 0, FT_EVENODD = 1 };                         /* FillRule, src/path.rs:8-14  */
enum { FT_JOIN_MITER = 0, FT_JOIN_BEVEL = 1, FT_JOIN_ROUND = 2 }; /* JoinStyle, src/stroker.rs:13-20 */
enum {
    FT_MATTE8 = 0,  /* pix Matte8: 1 byte / pixel; fill overwrites rows (src/fig.rs:629-636) */
    FT_RGBA8P = 1   /* pix Rgba8p: 4 bytes / pixel premultiplied; SrcOver (src/fig.rs:637-643) */
};
enum { FT_HOST = 0, FT_DEVICE = 1 };  /* where the ops / raster pointers live */
/* Output formats of ft_convert (pix SRgba8 / SGray8: straight alpha, sRGB gamma). */
enum { FT_SRGBA8 = 2, FT_SGRAY8 = 3 };

/* One path of a batch.  Each path is an independent Plotter call onto its own
 * raster (or region of one).  40 bytes. */
typedef struct ft_path_desc {
    uint32_t op_begin;       /* index of the first op of this path in `ops`          */
    uint32_t n_ops;          /* number of ops                                          */
    uint32_t width;          /* raster width in pixels                                 */
    uint32_t height;         /* raster height in pixels                                */
    uint64_t raster_offset;  /* byte offset of the raster in the raster buffer         */
    uint32_t stride;         /* bytes per raster row                                   */
    float s_width;           /* Plotter pen width when the call starts (plotter.rs:52) */
    uint8_t clr[4];          /* fill colour (premultiplied Rgba8p); ignored for Matte8  */
    uint32_t reserved;
} ft_path_desc;

typedef struct ft_ctx ft_ctx;

/* ---- context (Plotter state: tolerance, transform, join, pen width) ---- */

/* Plotter::new defaults (src/plotter.rs:96-115): tolerance 0.3, identity transform,
 * JoinStyle::Miter(4.0), pen width 1.0. */
FT_API int ft_ctx_create(int device, ft_ctx** out);
FT_API void ft_ctx_destroy(ft_ctx* ctx);
/* Issue work on `cuda_stream` (a cudaStream_t) instead of the context's own stream. */
FT_API int ft_set_stream(ft_ctx* ctx, void* cuda_stream);
/* Plotter::set_tolerance (src/plotter.rs:133-137): clamps to >= 0.01, stores t*t. */
FT_API int ft_set_tolerance(ft_ctx* ctx, float t);
/* Plotter::set_transform (src/plotter.rs:140-143): x' = m0*x + m1*y + m2,
 * y' = m3*x + m4*y + m5. */
FT_API int ft_set_transform(ft_ctx* ctx, const float m[6]);
/* Plotter::set_join (src/plotter.rs:158-161). */
FT_API int ft_set_join(ft_ctx* ctx, int32_t join, float miter_limit);
/* Plotter::pen_width state (src/plotter.rs:151-153); PenWidth ops update it and it
 * persists from call to call, as in footile. */
FT_API int ft_set_pen_width(ft_ctx* ctx, float w);
FT_API int ft_get_pen_width(ft_ctx* ctx, float* w);

/* Un-capped figures — a documented extension, not footile's behaviour.  footile keeps at
 * most FT_MAX_POINTS vertices per figure (Vid is u16; Fig::add_point ignores the rest,
 * fig.rs:428-442, vid.rs:9-70).  With a cap above that, fills (ft_fill and the fill calls
 * of ft_composite_batch) keep up to `max_points` vertices per figure, with 32-bit vertex
 * ids and otherwise footile's algorithm; vertices past the cap are still dropped.  0 (or
 * any value up to FT_MAX_POINTS) restores footile's cap.  Strokes and ft_fill_batch keep
 * footile's caps.  Each figure build holds about 45 bytes of device scratch per vertex. */
#define FT_FIG_CAP_MAX (1u << 26)
FT_API int ft_set_figure_cap(ft_ctx* ctx, uint32_t max_points);
FT_API int ft_get_figure_cap(ft_ctx* ctx, uint32_t* max_points);

/* ---- single-path calls ------------------------------------------------ */

/* Plotter::fill (src/plotter.rs:339-350).  `raster` is `h` rows of `stride` bytes in
 * `fmt`; it is read and written in place.  `clr` is the premultiplied RGBA colour
 * (ignored for FT_MATTE8, as footile ignores it, src/fig.rs:633).  With
 * where == FT_HOST the call copies, runs and copies back before returning; with
 * FT_DEVICE `ops` and `raster` are device pointers and the call is asynchronous on
 * the context stream. */
FT_API int ft_fill(ft_ctx* ctx, int32_t rule, const ft_op* ops, uint32_t n_ops,
                   int32_t fmt, const uint8_t clr[4], uint8_t* raster, uint32_t w,
                   uint32_t h, uint32_t stride, int32_t where);

/* Plotter::stroke (src/plotter.rs:356-365): stroke outline, then NonZero fill. */
FT_API int ft_stroke(ft_ctx* ctx, const ft_op* ops, uint32_t n_ops, int32_t fmt,
                     const uint8_t clr[4], uint8_t* raster, uint32_t w, uint32_t h,
                     uint32_t stride, int32_t where);

/* ---- batches: many independent Plotter calls in one persistent launch ---- */

/* Fill (stroke == 0) or stroke (stroke == 1) every path of `paths` onto its own
 * raster region.  `ops` holds all ops (n_ops_total), `rasters` all rasters
 * (raster_bytes).  `paths` is always a host array; `ops` / `rasters` live where
 * `where` says.  The per-path status of the last batch is read with
 * ft_batch_status.  The raster regions of the paths must not overlap.  With
 * FT_HOST, Matte8 rasters in page-locked host memory mapped into the device's address
 * space (cudaHostAlloc, cudaHostRegister, a pinned torch tensor) are written in place
 * by the kernels — a Matte8 fill or stroke only writes, so nothing is copied in or out
 * — and page-locked, 16-byte aligned ops are read in place (ft_tuning.host_mapped
 * switches either off).  Otherwise, with 64 MB of rasters or more, paths whose ops and
 * rasters lie in ascending order in the host buffers are drawn in two chunks, the
 * copies of one overlapping the drawing of the other (ft_tuning.host_chunks sets the
 * count). */
FT_API int ft_fill_batch(ft_ctx* ctx, int32_t stroke, int32_t rule, const ft_op* ops,
                         uint32_t n_ops_total, const ft_path_desc* paths,
                         uint32_t n_paths, int32_t fmt, uint8_t* rasters,
                         uint64_t raster_bytes, int32_t where);

/* Ordered composite: footile's sequence of Plotter calls on ONE raster.  Path i is
 * filled (stroke == 0, with `rule`) or stroked (stroke == 1) onto `raster` after
 * paths 0..i-1, with its own colour `paths[i].clr` and starting pen width
 * `paths[i].s_width` (footile carries the pen width from call to call, so set it to
 * the last PenWidth of the calls before, as the Python and C++ mirrors do).  The
 * width/height/offset/stride fields of `paths` are ignored: every path draws on the
 * w x h raster with `stride`.  Bit-identical to the calls made one after another,
 * including the alpha-0 SrcOver every call applies from its top row down.
 * Per-path status as for batches (ft_batch_status). */
FT_API int ft_composite_batch(ft_ctx* ctx, int32_t stroke, int32_t rule, const ft_op* ops,
                              uint32_t n_ops_total, const ft_path_desc* paths, uint32_t n_paths,
                              int32_t fmt, uint8_t* raster, uint32_t w, uint32_t h, uint32_t stride,
                              int32_t where);

/* Prepared batches: the path descriptors and the planned work queue stay on the
 * device, and each launch replays a captured CUDA graph (queue reset, status reset,
 * persistent rasteriser).  `ops` / `rasters` given to ft_batch_launch are device
 * pointers; the launch is asynchronous on the context stream.  A batch owns its
 * scratch memory and may be launched any number of times. */
typedef struct ft_batch ft_batch;
FT_API int ft_batch_create(ft_ctx* ctx, int32_t stroke, int32_t rule, const ft_path_desc* paths,
                           uint32_t n_paths, int32_t fmt, ft_batch** out);
FT_API int ft_batch_launch(ft_ctx* ctx, ft_batch* batch, const ft_op* ops, uint32_t n_ops_total,
                           uint8_t* rasters, uint64_t raster_bytes);
/* Per-path status codes of the last launch of `batch` (synchronises). */
FT_API int ft_batch_launch_status(ft_ctx* ctx, ft_batch* batch, int32_t* status, uint32_t n);
FT_API void ft_batch_destroy(ft_batch* batch);

/* Plan tuning — no counterpart in footile (its CPU plotter has nothing to tune).
 * The knobs of a batch plan: `warp_max_side`, the largest canvas side given whole to
 * one warp (0..512, 0 sends every path to the CTA rasteriser); `cta_smem_bytes`, the
 * CTA rasteriser's shared memory, which sets its tile: bands of as many full-width rows
 * as fit (0 = built-in choice; the ordered composite's figure builds keep their own
 * 48 KB); `split_px`, paths of at least this many pixels are
 * split into row ranges, the queue grain of large paths (0 = 1 Mpx); `grid_per_sm`,
 * resident CTAs per SM of the persistent kernels (0 = occupancy maximum).
 * Ordered composites (ft_composite_batch, and single calls of at least split_px pixels):
 * `band_rows`, rows per band (1..8, 0 = built-in: 4 for Rgba8p, 8 for Matte8) — the
 * height of a compositor tile; `tile_w`, the width of an Rgba8p compositor tile in pixels
 * (128, 256, 512 or 1024, 0 = built-in: 1024, or the narrowest that needs no more tiles);
 * `tile_stage`, how an Rgba8p compositor tile reaches the canvas: 1 = staged in shared
 * memory by TMA (when the canvas base and row stride are 16-byte aligned), 2 = read and
 * written in place, 0 = built-in; `pool_edges`, the first size of the binned-edge pool in edges (it
 * grows on demand; 0 = built-in); `fig_build`, who builds the figure of a single fill
 * or stroke path (ft_fill / ft_stroke of at least split_px pixels, or an
 * ft_composite_batch of one path): 1 = one CTA, 2 = the whole GPU (scans over the path's
 * ops, stroke points and raw vertices), 0 = built-in: the whole GPU from
 * FT_GRID_BUILD_OPS ops.  Host batches (ft_fill_batch with
 * FT_HOST): `host_chunks`, chunks of the copy pipeline (1..16, 0 = built-in: 2 from
 * 64 MB of rasters); `host_mapped`, 0 = page-locked Matte8 rasters are written and
 * page-locked ops read in place (built-in), 1 = rasters and ops are copied, 2 = rasters
 * in place, ops copied.  Results do not depend on the tuning.  ft_set_tuning(ctx, NULL) restores the
 * defaults; ft_get_tuning gives the values in effect (the defaults when none were set). */
typedef struct ft_tuning {
    int32_t warp_max_side;
    int32_t cta_smem_bytes;
    int32_t split_px;
    int32_t grid_per_sm;
    int32_t band_rows;
    int32_t pool_edges;
    int32_t host_chunks;
    int32_t host_mapped;
    int32_t tile_w;
    int32_t tile_stage;
    int32_t fig_build;
} ft_tuning;
FT_API int ft_set_tuning(ft_ctx* ctx, const ft_tuning* tuning);
FT_API int ft_get_tuning(ft_ctx* ctx, ft_tuning* tuning);

/* Autotuner: times candidate plans of this batch (prepared batches, graph replay, CUDA
 * events on the context stream), the built-in plan first, and keeps the fastest as the
 * context's tuning; a candidate displaces the plan in hand only when it is more than 1 %
 * faster, so knobs the batch does not exercise keep their built-in values.  With
 * `cache_path` (may be NULL) the choice is looked up first and appended after tuning,
 * keyed by the GPU (name, SM count), the call kind and a signature of the batch
 * (path count, mean and largest canvas side, mean op count, in powers of two).  `ops`
 * and `rasters` are device pointers; the rasters are overwritten while tuning.
 * `chosen` (may be NULL) receives the tuning; `ms` (may be NULL) its launch time
 * (0 when taken from the cache). */
FT_API int ft_autotune_batch(ft_ctx* ctx, int32_t stroke, int32_t rule, const ft_op* ops,
                             uint32_t n_ops_total, const ft_path_desc* paths, uint32_t n_paths,
                             int32_t fmt, uint8_t* rasters, uint64_t raster_bytes,
                             const char* cache_path, ft_tuning* chosen, float* ms);

/* Allocation-free fill of one path — this entry point has no counterpart in footile.
 * It is for callers that may not allocate device memory, themselves or through this
 * library: a host whose device memory belongs to another runtime's allocator (a game
 * engine's or a language runtime's pool that has to account for every allocation),
 * or a process held to a fixed device-memory budget.  It needs no context and calls
 * no allocator: the figure scratch of the call (vertices, sub-figure starts and edges
 * of one figure, about 2.9 MB) is a file-scope device array that every GPU which loads
 * this library holds until the process exits.  The caller passes the inputs and the
 * output; all pointers are device pointers; `ops` must be 16-byte aligned, Rgba8p rows
 * 4-byte aligned.  `transform` may be NULL (identity); `status` (device int, may be
 * NULL) receives FT_OK, FT_ERR_DEPTH or FT_ERR_ARG.  The call is asynchronous on
 * `stream`; its return value is the launch's own status (an error that an earlier,
 * unrelated CUDA call left behind is neither reported nor cleared).
 *
 * `pen_width` is the pen width at the start of the call (footile's Plotter state,
 * plotter.rs:151-153).  Unlike ft_fill, which keeps the width a PenWidth op leaves for
 * the next call in its context, this call has no context: a PenWidth op affects this
 * call only, and the caller carries the width to its next call itself.
 *
 * The first call on each device (and the first after a device reset) looks up the
 * array's device address and sets the kernel's shared-memory limit in the device's
 * current context; make that first call before any stream capture.  Every call shares
 * the one array, and each call leaves its figure there for the next call to overwrite:
 * calls whose kernels overlap on the GPU race on it, so serialise them (one stream, or
 * events between streams).  Widths above FT_MAX_WIDTH return FT_ERR_CAP; figures are
 * capped at FT_MAX_POINTS vertices as in footile, so every path fits the array. */
FT_API int ft_fill_noalloc(int32_t rule, const ft_op* ops, uint32_t n_ops, int32_t fmt,
                           const uint8_t clr[4], uint8_t* raster, uint32_t w, uint32_t h,
                           uint32_t stride, const float transform[6], float tolerance,
                           float pen_width, int32_t* status, void* stream);

/* Coverage adjoint — no counterpart in footile, which has no gradients.  A
 * differentiable FP32 coverage of a batch of fills and its backward pass, for a
 * torch.autograd.Function (or any reverse-mode caller) to wrap.
 *
 * Coverage: the path walk and De Casteljau subdivision of Plotter::fill
 * (plotter.rs:175-332, the same f32 subdivision tree as ft_fill), sub-figures as
 * Fig builds them (fig.rs:428-461), covered with the cell-area scheme of
 * fig.rs:285-321 in float without the 16.16 / 1/256 quantisation (the exact area of
 * the flattened polygon in each pixel), the row prefix sum of imgbuf.rs:38-51 as the
 * winding area S, then NonZero min(|S|, 1) or EvenOdd the triangle wave of period 2.
 *
 * ft_adjoint_forward writes the coverage of path i (width x height floats) into
 * `cov` at paths[i].raster_offset bytes with paths[i].stride bytes per row (both
 * multiples of 4, widths up to FT_MAX_WIDTH) and keeps in `*saved` (created when
 * NULL, reused otherwise) a copy of the ops and paths and the winding area: 4 bytes
 * per coverage byte.  ft_adjoint_backward takes dLoss/dcov in the layout of `cov`,
 * recomputes the flattened edges and writes dLoss/d(op floats) to `grad_ops`
 * (6 floats per op, the layout of ft_op.v: overwritten, zero for Close and for
 * PenWidth in a fill) and zero to `grad_width` (one float per path: a fill's coverage
 * does not depend on the pen width; may be NULL).  Gradients hold the subdivision
 * tree fixed: it is piecewise constant in the control points.  The tolerance and
 * transform are the context's at the forward call.  `where` is FT_HOST or FT_DEVICE
 * for ops, cov, grad_cov, grad_ops and grad_width; path descriptors are host memory.
 * Per-path status (FT_ERR_DEPTH, FT_ERR_ARG, FT_ERR_CAP for more than FT_MAX_POINTS
 * flattened vertices: coverage zero, gradient zero) via ft_adjoint_status.
 *
 * With `stroke` = 1 each path is Plotter::stroke'd (plotter.rs:356-365) with the
 * context's join and paths[i].s_width as the pen width at the call's start: the
 * coverage is that of footile's outline (stroker.rs:204-416: the same stroke points,
 * offsets, joins and arcs in f32, transformed a second time) filled NonZero, `rule` is
 * ignored, and the backward also differentiates the outline (offset points, miter
 * intersections, arc points; the miter and arc decisions held): gradients reach the
 * control points, the PenWidth ops (slot 0 of their grad_ops row) and, per path, the
 * starting pen width (`grad_width`).  Strokes whose outline needs more than
 * FT_MAX_POINTS vertices or 200,000 outline nodes report FT_ERR_CAP. */
typedef struct ft_adjoint ft_adjoint;
FT_API int ft_adjoint_forward(ft_ctx* ctx, int32_t stroke, int32_t rule, const ft_op* ops,
                              uint32_t n_ops_total, const ft_path_desc* paths, uint32_t n_paths,
                              float* cov, uint64_t cov_bytes, int32_t where, ft_adjoint** saved);
FT_API int ft_adjoint_backward(ft_ctx* ctx, ft_adjoint* saved, const float* grad_cov, float* grad_ops,
                               float* grad_width, int32_t where);
FT_API int ft_adjoint_status(ft_ctx* ctx, ft_adjoint* saved, int32_t* status, uint32_t n);
FT_API void ft_adjoint_destroy(ft_adjoint* saved);

/* Pixel conversion after plotting, as footile's examples do with pix
 * (`Raster::<SRgba8>::with_raster`, examples/fishy.rs:33; `Raster::<SGray8>`,
 * examples/drop.rs:22): FT_RGBA8P -> FT_SRGBA8 (straight alpha: channel / alpha, then
 * the sRGB transfer function of IEC 61966-2-1, correctly rounded; alpha kept; alpha 0
 * gives 0) and FT_MATTE8 -> FT_SGRAY8 (the mask byte as linear gray, sRGB-encoded).
 * `src` and `dst` may be the same buffer when the strides are equal.  With FT_HOST the
 * call copies in and out; with FT_DEVICE it is asynchronous on the context stream. */
FT_API int ft_convert(ft_ctx* ctx, int32_t src_fmt, const uint8_t* src, uint32_t src_stride,
                      int32_t dst_fmt, uint8_t* dst, uint32_t dst_stride, uint32_t w, uint32_t h,
                      int32_t where);

/* Ordered SrcOver of float coverage layers, and its adjoint — the differentiable
 * counterpart of ft_composite_batch, for an ordered batch of fills or strokes whose
 * coverages come from ft_adjoint_forward (one plane per path over the shared canvas).
 * Layer n (coverage plane cov + n * plane_floats, premultiplied colour clr[4n..4n+3] in
 * [0, 1]) composites as pix's SrcOver does (fig.rs:637-643):
 *   C_n = clr_n * cov_n + C_{n-1} * (1 - alpha_n * cov_n),   C_0 = init (or 0).
 * ft_srcover_forward writes C_N (n_px float4).  ft_srcover_backward takes dLoss/dC_N
 * and writes dLoss/dcov for every layer (the layout of cov) and dLoss/dC_0 (may be
 * NULL); it recomputes the canvas terms it needs (nothing is kept from the forward)
 * and divides by nothing, so opaque layers are exact.  Device pointers; asynchronous on
 * the context stream. */
FT_API int ft_srcover_forward(ft_ctx* ctx, const float* cov, uint32_t n_layers, uint64_t plane_floats,
                              const float* clr, const float* init, float* out, uint32_t n_px);
FT_API int ft_srcover_backward(ft_ctx* ctx, const float* cov, uint32_t n_layers, uint64_t plane_floats,
                               const float* clr, const float* init, const float* grad_out,
                               float* grad_cov, float* grad_init, uint32_t n_px);

/* Differentiable ordered composite of strokes on one canvas, at any canvas size and
 * stroke count: the float counterpart of ft_composite_batch with stroke = 1
 * (Plotter::stroke of each path in order onto one Rgba8p raster, plotter.rs:356-365,
 * fig.rs:637-643).  C_n = clr_n * cov_n + C_{n-1} * (1 - alpha_n * cov_n) with cov_n
 * the stroke coverage of ft_adjoint_forward (stroke = 1) over the width x height
 * canvas, C_0 = init (n_px float4, or NULL for 0); `out` receives C_N (n_px float4).
 * paths[i] gives stroke i's op range and starting pen width (op_begin, n_ops,
 * s_width; the raster fields are ignored); clr holds n_paths premultiplied float4
 * colours.  The strokes are covered in chunks of `chunk` planes (0: sized to the free
 * device memory); only the canvas before each chunk is kept, and
 * ft_stroke_composite_backward recomputes the coverage chunk by chunk, last chunk
 * first (SrcOver is affine in the canvas with a scalar factor, so the gradient reaching
 * a chunk's input is the gradient at its output scaled per pixel).  Given dLoss/dC_N it
 * writes dLoss/d(op floats) (overwritten; the layout of ft_adjoint_backward),
 * dLoss/d(starting pen width) per stroke and dLoss/dC_0 (each may be NULL except
 * grad_ops).  The join, miter limit, tolerance and transform are the context's at the
 * forward call.  `where` is FT_HOST or FT_DEVICE for ops, clr, init, out and the
 * gradients; path descriptors are host memory.  The saved state holds copies of its
 * inputs.  Per-stroke status via ft_stroke_composite_status; the chunk size in use via
 * ft_stroke_composite_chunk. */
typedef struct ft_composite_adjoint ft_composite_adjoint;
FT_API int ft_stroke_composite_forward(ft_ctx* ctx, const ft_op* ops, uint32_t n_ops_total,
                                       const ft_path_desc* paths, uint32_t n_paths, const float* clr,
                                       uint32_t width, uint32_t height, const float* init, float* out,
                                       uint32_t chunk, int32_t where, ft_composite_adjoint** saved);
FT_API int ft_stroke_composite_backward(ft_ctx* ctx, ft_composite_adjoint* saved, const float* grad_out,
                                        float* grad_ops, float* grad_width, float* grad_init, int32_t where);
FT_API int ft_stroke_composite_status(ft_ctx* ctx, ft_composite_adjoint* saved, int32_t* status, uint32_t n);
FT_API uint32_t ft_stroke_composite_chunk(ft_composite_adjoint* saved);
FT_API void ft_stroke_composite_destroy(ft_composite_adjoint* saved);

/* Per-path status codes of the last batch (synchronises the context stream). */
FT_API int ft_batch_status(ft_ctx* ctx, int32_t* status, uint32_t n);

/* Wait for all work of the context. */
FT_API int ft_sync(ft_ctx* ctx);

/* Message for the last error of this context (static storage, never NULL). */
FT_API const char* ft_last_error(ft_ctx* ctx);

/* Device time in milliseconds of the last call's kernels (CUDA events). */
FT_API int ft_last_timings(ft_ctx* ctx, float* kernel_ms);

/* Device time in milliseconds of the Rgba8p tile compositor alone in the last call (the
 * ordered SrcOver after the figures are built and binned; ft_composite_batch, and ft_fill /
 * ft_stroke of at least split_px pixels); 0 when the last call did not run it.  No
 * counterpart in footile: for measuring the compositing step against the HBM roofline. */
FT_API int ft_last_composite_ms(ft_ctx* ctx, float* ms);

/* Bounds-check build (the library compiled with -DFT_CHECK=1) — no counterpart in
 * footile; it stands in for a memory checker.  Device code checks the indices of its
 * shared-memory cell buffers, warp scratch, edge pool, compositor queues and the grid-wide
 * figure build's raw vertices and figure writes; a failed check
 * skips the access and keeps the first failing site's number.  `site` (may be NULL)
 * receives that number since the last call (0: none) and is reset; `compiled_in` (may be
 * NULL) is 1 in the check build and 0 in the shipped build, whose checks fold away. */
FT_API int ft_check_failures(int32_t* site, int32_t* compiled_in);

/* Number of kernel launches the library has issued since the context was created. */
FT_API uint64_t ft_launch_count(ft_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* FOOTILE_GPU_H */
