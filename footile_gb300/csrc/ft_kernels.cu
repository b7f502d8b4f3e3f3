// ft_kernels.cu — the GB300 fill/stroke rasteriser (sm_103a).
//
// One persistent kernel drains a device queue of work items (a path and a range
// of its raster rows).  For each item one CTA of 256 threads:
//
//  1. walks the path ops in chunks of 256 (footile plotter.rs:175-224): two block
//     max-scans give every op its pen, pen width and "starts a new sub-figure"
//     flag, so each thread then flattens its own op independently;
//  2. flattens quads / cubics by recursive De Casteljau subdivision
//     (plotter.rs:248-265, 311-332) with an explicit per-thread stack, IEEE f32
//     without contraction, in the reference's depth-first leaf order: a count
//     pass, a block scan, then an emit pass into a shared-memory window;
//  3. builds the figure (fig.rs:428-461): warp 0 drops coincident vertices, pops
//     a closing vertex equal to the sub-figure start and applies the 65,535-vertex
//     cap, with ballots over 32 vertices at a time;
//  4. finds the top vertex (min (y, x, id), the head of footile's stable (Y,X)
//     sort, fig.rs:493-496) and the figure direction (fig.rs:402-411), and turns
//     every non-horizontal segment into an edge (fig.rs:179-201) — each segment
//     yields exactly the edge the active-edge sweep would add;
//  5. rasterises bands of rows: every (edge, row) pair is independent (x at the
//     bottom of row k is x_bot0 + k*inv_slope, wrapping), and its per-cell
//     coverage (fig.rs:285-321) has a closed form, so threads take (edge, row)
//     items and add signed cell areas into a shared-memory i32 band buffer with
//     atomics.  i16 wrapping sums commute, so the i32 sums truncated to i16 equal
//     footile's;
//  6. resolves each band row with a warp scan (__shfl_up_sync) and the NonZero /
//     EvenOdd rule (imgbuf.rs:38-199), then overwrites Matte8 rows or composites
//     premultiplied RGBA with pix SrcOver (fig.rs:629-665).
//
// Rows footile writes: from max(top_row, 0) to the bottom of the raster, raster
// row r receiving scan row r + min(top_row, 0) (fig.rs:496-499, 536-553).
#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>

#include <cuda.h>

#include "ft_device.cuh"
#include "ft_kernels.cuh"

namespace ftk {

constexpr unsigned FULL = 0xFFFFFFFFu;

// Bounds checks of the check build (nvcc -DFT_CHECK=1, see _build.build_variant): a failed
// check keeps the first failing site's number in g_check and skips the access; no trap.
// In the shipped build every check folds to true.
#ifndef FT_CHECK
#define FT_CHECK 0
#endif
static __device__ int g_check = 0;
__device__ __forceinline__ bool ck(bool ok, int site) {
    if (FT_CHECK && !ok) atomicCAS(&g_check, 0, site);
    return !FT_CHECK || ok;
}
// Curve leaves of an op kept (in local memory) from the count pass for the emit pass;
// ops with more leaves are walked again.  Warp builds (small glyphs) keep 64; CTA builds
// (large figures, few CTAs, L1 to spare) keep more.
constexpr int LEAF_CACHE = 64;
constexpr int LEAF_CACHE_CTA = 256;
constexpr bool BLOCK_COMPACT = true;  // figure building by the whole CTA (false: warp 0)
constexpr int SRAW = 1024;            // stroke points per window (float4 in the raw window's bytes)

// ------------------------------------------------------------ block scans
__device__ __forceinline__ int warp_incl_sum(int v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += t;
    }
    return v;
}
__device__ __forceinline__ unsigned warp_incl_sum_u(unsigned v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += t;
    }
    return v;
}
__device__ __forceinline__ int warp_incl_max(int v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v = max(v, t);
    }
    return v;
}
// Exclusive block sum; `total` receives the block total.  tmp: NWARP ints.
__device__ int block_excl_sum(int v, int* tmp, int& total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = warp_incl_sum(v);
    if (lane == 31) tmp[w] = inc;
    __syncthreads();
    if (w == 0) {
        int t = lane < NWARP ? tmp[lane] : 0;
        t = warp_incl_sum(t);
        if (lane < NWARP) tmp[lane] = t;
    }
    __syncthreads();
    int base = w > 0 ? tmp[w - 1] : 0;
    total = tmp[NWARP - 1];
    __syncthreads();
    return base + inc - v;
}
// Inclusive block max.
__device__ int block_incl_max(int v, int* tmp) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = warp_incl_max(v);
    if (lane == 31) tmp[w] = inc;
    __syncthreads();
    if (w == 0) {
        int t = lane < NWARP ? tmp[lane] : -1;
        t = warp_incl_max(t);
        if (lane < NWARP) tmp[lane] = t;
    }
    __syncthreads();
    int r = w > 0 ? max(inc, tmp[w - 1]) : inc;
    __syncthreads();
    return r;
}
// Inclusive and exclusive block max (identity -1) in one pass.
__device__ void block_max_scan(int v, int* tmp, int& incl, int& excl) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = warp_incl_max(v);
    int wex = __shfl_up_sync(FULL, inc, 1);
    if (lane == 0) wex = -1;
    if (lane == 31) tmp[w] = inc;
    __syncthreads();
    if (w == 0) {
        int t = lane < NWARP ? tmp[lane] : -1;
        t = warp_incl_max(t);
        if (lane < NWARP) tmp[lane] = t;
    }
    __syncthreads();
    int carry = w > 0 ? tmp[w - 1] : -1;
    incl = max(inc, carry);
    excl = max(wex, carry);
    __syncthreads();
}

// Thread-group policies: the figure builder runs either on a whole CTA (large
// paths) or on one warp (small paths, many per CTA, no block barriers).
struct BlockG {
    static constexpr int N = BLOCK;
    static constexpr int RAW = RAW_CAP;
    __device__ static int rank() { return threadIdx.x; }
    __device__ static void sync() { __syncthreads(); }
    __device__ static int excl_sum(int v, int* tmp, int& total) { return block_excl_sum(v, tmp, total); }
    __device__ static int incl_max(int v, int* tmp) { return block_incl_max(v, tmp); }
    __device__ static void max_scan(int v, int* tmp, int& incl, int& excl) { block_max_scan(v, tmp, incl, excl); }
};
struct WarpG {
    static constexpr int N = 32;
    static constexpr int RAW = 256;
    __device__ static int rank() { return threadIdx.x & 31; }
    __device__ static void sync() { __syncwarp(); }
    __device__ static int excl_sum(int v, int*, int& total) {
        __syncwarp();
        const int inc = warp_incl_sum(v);
        total = __shfl_sync(FULL, inc, 31);
        return inc - v;
    }
    __device__ static int incl_max(int v, int*) {
        __syncwarp();
        return warp_incl_max(v);
    }
    __device__ static void max_scan(int v, int*, int& incl, int& excl) {
        __syncwarp();
        incl = warp_incl_max(v);
        excl = __shfl_up_sync(FULL, incl, 1);
        if ((threadIdx.x & 31) == 0) excl = -1;
    }
};

// ------------------------------------------------- De Casteljau flattening
// Stack frames of the walks: the right half of a subdivided curve.  A frame keeps no
// start point: the right half starts where the last leaf of the left half ends (that
// leaf's end point is the same value, carried down unchanged).  Fills carry no widths.
template <bool W>
struct QuadFr {
    P2 b, c;
    float wb, wc;
    int d;
};
template <>
struct QuadFr<false> {
    P2 b, c;
    int d;
};
template <bool W>
struct CubicFr {
    P2 b, c, e;
    float wb, wc, we;
    int d;
};
template <>
struct CubicFr<false> {
    P2 b, c, e;
    int d;
};

// Walk the subdivision of a quad (plotter.rs:248-265) in depth-first order.
// Leaves with index in [lo, hi) go to emit(index, point, width).  Returns the
// number of leaves walked (the total when hi == INT_MAX).  `d0`: the depth of (a, b, c)
// in the subdivision of a larger curve (0: the curve itself).
template <bool W, class Emit>
__device__ int quad_walk(P2 a, P2 b, P2 c, float wa, float wb, float wc, float tol_sq, int lo, int hi,
                         int* depth_hit, Emit emit, int d0 = 0) {
    using Fr = QuadFr<W>;
    Fr st[FT_MAX_DEPTH + 1];
    int sp = 0, leaf = 0, d = d0;
    for (;;) {
        P2 ab = pmid(a, b), bc = pmid(b, c), abbc = pmid(ab, bc), ac = pmid(a, c);
        bool within = pdist_sq(abbc, ac) <= tol_sq;
        if (within || d >= FT_MAX_DEPTH) {
            if (!within) *depth_hit = 1;
            if (leaf >= lo && leaf < hi) emit(leaf, c, wc);
            leaf++;
            if (leaf >= hi || sp == 0) break;
            --sp;
            a = c;
            b = st[sp].b;
            c = st[sp].c;
            if constexpr (W) {
                wa = wc;
                wb = st[sp].wb;
                wc = st[sp].wc;
            }
            d = st[sp].d;
        } else {
            float wab = 0, wbc = 0, wabbc = 0;
            if constexpr (W) {
                wab = fmid(wa, wb);
                wbc = fmid(wb, wc);
                wabbc = fmid(wab, wbc);
            }
            st[sp].b = bc;
            st[sp].c = c;
            if constexpr (W) {
                st[sp].wb = wbc;
                st[sp].wc = wc;
            }
            st[sp].d = d + 1;
            sp++;
            b = ab;
            c = abbc;
            if constexpr (W) {
                wb = wab;
                wc = wabbc;
            }
            d++;
        }
    }
    return leaf;
}

// The same for a cubic (plotter.rs:311-332).
template <bool W, class Emit>
__device__ int cubic_walk(P2 a, P2 b, P2 c, P2 e, float wa, float wb, float wc, float we, float tol_sq, int lo,
                          int hi, int* depth_hit, Emit emit, int d0 = 0) {
    using Fr = CubicFr<W>;
    Fr st[FT_MAX_DEPTH + 1];
    int sp = 0, leaf = 0, d = d0;
    for (;;) {
        P2 ab = pmid(a, b), bc = pmid(b, c), cd = pmid(c, e);
        P2 abbc = pmid(ab, bc), bccd = pmid(bc, cd);
        P2 pe = pmid(abbc, bccd);
        P2 ad = pmid(a, e);
        bool within = pdist_sq(pe, ad) <= tol_sq;
        if (within || d >= FT_MAX_DEPTH) {
            if (!within) *depth_hit = 1;
            if (leaf >= lo && leaf < hi) emit(leaf, e, we);
            leaf++;
            if (leaf >= hi || sp == 0) break;
            --sp;
            a = e;
            b = st[sp].b;
            c = st[sp].c;
            e = st[sp].e;
            if constexpr (W) {
                wa = we;
                wb = st[sp].wb;
                wc = st[sp].wc;
                we = st[sp].we;
            }
            d = st[sp].d;
        } else {
            float wab = 0, wbc = 0, wcd = 0, wabbc = 0, wbccd = 0, wpe = 0;
            if constexpr (W) {
                wab = fmid(wa, wb);
                wbc = fmid(wb, wc);
                wcd = fmid(wc, we);
                wabbc = fmid(wab, wbc);
                wbccd = fmid(wbc, wcd);
                wpe = fmid(wabbc, wbccd);
            }
            st[sp].b = bccd;
            st[sp].c = cd;
            st[sp].e = e;
            if constexpr (W) {
                st[sp].wb = wbccd;
                st[sp].wc = wcd;
                st[sp].we = we;
            }
            st[sp].d = d + 1;
            sp++;
            b = ab;
            c = abbc;
            e = pe;
            if constexpr (W) {
                wb = wab;
                wc = wabbc;
                we = wpe;
            }
            d++;
        }
    }
    return leaf;
}

// ------------------------------------------------------------- CTA state
struct CState {
    // path walk carried between op chunks
    float pen_x, pen_y, pen_w, sw;
    int last_pc_kind;  // kind of the last Move/Line/Quad/Cubic/Close op, -1 none
    // figure builder
    int count;
    int has_prev, prev_x, prev_y;  // previous raw vertex
    int rf_x, rf_y, rf_pos;        // first vertex of the current sub-figure and its id
    int capped;
    int overflow;  // the figure outgrew the warp's scratch: hand the path to a CTA
    int flags;     // 1: depth cap reached, 2: bad argument
    // figure summary
    int top_row;
    int dir;  // 0 forward, 1 reverse
    int last_pw;
    // stroke points (stroker.rs:204-236)
    int s_count, s_nsubs, s_capped, s_last_op, s_has_prev;
    float s_prev_x, s_prev_y;
    int s_items;  // outline items of all sub-strokes
};

template <int N, int RAW>
struct BuildSmemT {
    int kind[N];
    float pwval[N];
    float penx[N], peny[N], penw[N];
    int scan[2 * NWARP + 2];
    // 16-byte aligned: stroke points are stored here as float4
    __align__(16) int2 raw[RAW];
    unsigned char rs[RAW];
};
using BuildSmem = BuildSmemT<BLOCK, RAW_CAP>;
using WarpBuildSmem = BuildSmemT<32, 256>;

constexpr int MAP_CAP = 4096;  // (edge, row) items mapped per round

struct RasterSmem {
    EdgeRec edges[BLOCK];
    int ya[BLOCK];
    int off[BLOCK + 1];
    int scan[2 * NWARP + 2];
    unsigned char map[MAP_CAP];  // item -> edge slot of the current chunk
};
static_assert(((sizeof(RasterSmem) + 15) & ~(size_t)15) <= (size_t)RASTER_FIXED_SMEM, "raster smem layout");
static_assert(sizeof(int2) * RAW_CAP >= sizeof(float4) * SRAW && RAW_CAP >= 2 * SRAW, "stroke window layout");
static_assert(offsetof(BuildSmem, raw) % 16 == 0 && sizeof(BuildSmem) % 16 == 0, "build smem alignment");
static_assert(offsetof(WarpBuildSmem, raw) % 8 == 0, "warp build smem alignment");

// ------------------------------------------------------------ figure builder
// Sequential restatement of Fig::add_point / Fig::close (fig.rs:373-461) for one
// group of raw vertices; used for the group in which the 65,535 cap is reached.
__device__ void seq_group(CState& S, const int2* raw, const unsigned char* rsf, int n, int2* pts, int* ss,
                          int cap = PT_CAP) {
    int count = S.count, has_prev = S.has_prev;
    int px = S.prev_x, py = S.prev_y, rfx = S.rf_x, rfy = S.rf_y, rf_pos = S.rf_pos;
    for (int l = 0; l < n; l++) {
        int2 p = raw[l];
        int rs = rsf[l];
        // a close event precedes a vertex that starts a sub-figure: pop when the
        // last vertex equals the sub-figure start (fig.rs:373-383)
        if (rs && has_prev && rfx == px && rfy == py) count -= 1;
        if (count >= cap) {
            // add_point is ignored from here on (fig.rs:430).  The next close —
            // an explicit one or the one Plotter::fill ends with — pops the last
            // vertex if it equals the open sub-figure's start.
            if (!rs && rfx == px && rfy == py) count -= 1;
            S.capped = 1;
            break;
        }
        if (rs) {
            rfx = p.x;
            rfy = p.y;
            rf_pos = count;
            pts[count] = p;
            ss[count] = count;
            count++;
        } else if (p.x != px || p.y != py) {
            pts[count] = p;
            ss[count] = rf_pos;
            count++;
        }
        px = p.x;
        py = p.y;
        has_prev = 1;
    }
    S.count = count;
    S.has_prev = has_prev;
    S.prev_x = px;
    S.prev_y = py;
    S.rf_x = rfx;
    S.rf_y = rfy;
    S.rf_pos = rf_pos;
}

// Warp 0: append one window of raw vertices to the figure.  A vertex is kept when
// it starts a sub-figure or differs from the previous raw vertex; a sub-figure
// whose last vertex equals its first loses that vertex when it is closed.
__device__ void compact_window(CState& S, const int2* raw, const unsigned char* rsf, int m, int2* pts, int* ss,
                               int limit) {
    int lane = threadIdx.x & 31;
    for (int base = 0; base < m; base += 32) {
        int k = base + lane;
        bool valid = k < m;
        int2 p = valid ? raw[k] : make_int2(0, 0);
        int rs = valid ? rsf[k] : 0;
        int count = S.count, has_prev = S.has_prev;
        int prevx = S.prev_x, prevy = S.prev_y;
        int rfx0 = S.rf_x, rfy0 = S.rf_y, rf_pos0 = S.rf_pos;
        unsigned vmask = __ballot_sync(FULL, valid);
        unsigned RS = __ballot_sync(FULL, valid && rs);
        // close of the run that ended with the previous group
        int count_g = count;
        if ((RS & 1u) && has_prev && rfx0 == prevx && rfy0 == prevy) count_g -= 1;
        int qx = __shfl_up_sync(FULL, p.x, 1), qy = __shfl_up_sync(FULL, p.y, 1);
        if (lane == 0) {
            qx = prevx;
            qy = prevy;
        }
        bool keep = valid && (rs || p.x != qx || p.y != qy);
        unsigned K = __ballot_sync(FULL, keep);
        unsigned E = (RS >> 1) & vmask;  // lane l ends its run when lane l+1 starts one
        unsigned le = (lane == 31) ? FULL : ((2u << lane) - 1u);
        unsigned rsl = RS & le;
        int jf = rsl ? 31 - __clz(rsl) : -1;
        int src = jf < 0 ? 0 : jf;
        int rfx = __shfl_sync(FULL, p.x, src), rfy = __shfl_sync(FULL, p.y, src);
        if (jf < 0) {
            rfx = rfx0;
            rfy = rfy0;
        }
        bool pop = ((E >> lane) & 1u) && p.x == rfx && p.y == rfy;
        unsigned PM = __ballot_sync(FULL, pop);
        unsigned below = (1u << lane) - 1u;
        int pos = count_g + __popc(K & below) - __popc(PM & below);
        if (__any_sync(FULL, keep && pos >= limit)) {
            // more vertices than this warp's scratch holds
            if (lane == 0) S.overflow = 1;
            __syncwarp();
            return;
        }
        unsigned capm = __ballot_sync(FULL, keep && pos >= PT_CAP);
        if (capm) {
            if (lane == 0) seq_group(S, raw + base, rsf + base, min(32, m - base), pts, ss);
            __syncwarp();
            return;
        }
        bool write = keep;
        unsigned Ege = E & ~below;
        if (keep && Ege) {
            int e = __ffs(Ege) - 1;
            if ((PM >> e) & 1u) {
                unsigned upto_e = (e == 31) ? FULL : ((2u << e) - 1u);
                if ((K & upto_e & ~le) == 0) write = false;  // the popped vertex
            }
        }
        int posj = __shfl_sync(FULL, pos, src);
        int ssv = jf < 0 ? rf_pos0 : posj;
        if (write) {
            pts[pos] = p;
            ss[pos] = ssv;
        }
        int last = 31 - __clz(vmask);
        int nprevx = __shfl_sync(FULL, p.x, last), nprevy = __shfl_sync(FULL, p.y, last);
        int lrs = RS ? 31 - __clz(RS) : 0;
        int nrfx = __shfl_sync(FULL, p.x, lrs), nrfy = __shfl_sync(FULL, p.y, lrs);
        int nrfpos = __shfl_sync(FULL, pos, lrs);
        __syncwarp();
        if (lane == 0) {
            S.count = count_g + __popc(K) - __popc(PM);
            S.prev_x = nprevx;
            S.prev_y = nprevy;
            S.has_prev = 1;
            if (RS) {
                S.rf_x = nrfx;
                S.rf_y = nrfy;
                S.rf_pos = nrfpos;
            }
        }
        __syncwarp();
    }
}

// Block-wide variant of compact_window: 256 raw vertices per step, one per thread.
// Cross-lane questions (latest sub-figure start at or before a vertex, next kept
// vertex, next run end) are answered from per-warp ballot masks in shared memory.
struct CompactSmem {
    unsigned rsm[NWARP], km[NWARP], em[NWARP], pm[NWARP];
    int posv[BLOCK];
    int scan[2 * NWARP + 2];
};

// first set bit of the block-wide mask at index >= i (block-local), or BLOCK
__device__ __forceinline__ int mask_next(const unsigned* m, int i) {
    int w = i >> 5;
    unsigned bits = m[w] & (0xFFFFFFFFu << (i & 31));
    while (!bits) {
        if (++w >= NWARP) return BLOCK;
        bits = m[w];
    }
    return (w << 5) + __ffs(bits) - 1;
}
// last set bit at index <= i (block-local), or -1
__device__ __forceinline__ int mask_prev(const unsigned* m, int i) {
    int w = i >> 5;
    int sh = i & 31;
    unsigned bits = m[w] & (sh == 31 ? 0xFFFFFFFFu : ((2u << sh) - 1u));
    while (!bits) {
        if (--w < 0) return -1;
        bits = m[w];
    }
    return (w << 5) + 31 - __clz(bits);
}

__device__ void compact_window_block(CState& S, const int2* raw, const unsigned char* rsf, int m, int2* pts,
                                     int* ss, CompactSmem& C, int cap = PT_CAP) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int base = 0; base < m; base += BLOCK) {
        const int k = base + tid;
        const bool valid = k < m;
        const int2 p = valid ? raw[k] : make_int2(0, 0);
        const int rs = valid ? rsf[k] : 0;
        const int count0 = S.count, has_prev = S.has_prev;
        const int prevx = S.prev_x, prevy = S.prev_y, rfx0 = S.rf_x, rfy0 = S.rf_y, rfpos0 = S.rf_pos;
        const int nb = min(BLOCK, m - base);  // vertices in this step
        // close of the run that ended with the previous step (pop if it returned to its start)
        int count_b = count0;
        if (rsf[base] && has_prev && rfx0 == prevx && rfy0 == prevy) count_b -= 1;
        int2 q = make_int2(prevx, prevy);
        if (tid > 0 && valid) q = raw[k - 1];
        const bool keep = valid && (rs || p.x != q.x || p.y != q.y);
        // runs ending at the step's last vertex are closed at the next step (as above)
        const bool endk = valid && (tid + 1 < nb) && rsf[k + 1];
        const unsigned RS = __ballot_sync(FULL, valid && rs), K = __ballot_sync(FULL, keep),
                       E = __ballot_sync(FULL, endk);
        if (lane == 0) {
            C.rsm[w] = RS;
            C.km[w] = K;
            C.em[w] = E;
        }
        __syncthreads();
        const int jf = mask_prev(C.rsm, tid);  // first vertex of this vertex's run, in this block
        int rfx = rfx0, rfy = rfy0;
        if (jf >= 0) {
            const int2 f = raw[base + jf];
            rfx = f.x;
            rfy = f.y;
        }
        const bool pop = endk && p.x == rfx && p.y == rfy;
        const unsigned PM = __ballot_sync(FULL, pop);
        if (lane == 0) C.pm[w] = PM;
        int tot;
        const int ex = block_excl_sum((keep ? 1 : 0) - (pop ? 1 : 0), C.scan, tot);
        const int pos = count_b + ex;
        C.posv[tid] = pos;
        const int capped = __syncthreads_or(keep && pos >= cap);
        if (capped) {
            if (tid == 0) seq_group(S, raw + base, rsf + base, nb, pts, ss, cap);
            __syncthreads();
            return;
        }
        // a vertex disappears when it is the last kept one of a run that pops in this block
        bool write = keep;
        if (keep) {
            const int e = mask_next(C.em, tid);
            if (e < BLOCK && ((C.pm[e >> 5] >> (e & 31)) & 1u)) {
                const int nk = tid < BLOCK - 1 ? mask_next(C.km, tid + 1) : BLOCK;
                if (nk > e) write = false;
            }
        }
        if (write) {
            pts[pos] = p;
            ss[pos] = jf >= 0 ? C.posv[jf] : rfpos0;
        }
        __syncthreads();
        if (tid == 0) {
            const int n = nb;
            S.count = count_b + tot;
            const int2 l = raw[base + n - 1];
            S.prev_x = l.x;
            S.prev_y = l.y;
            S.has_prev = 1;
            const int lr = mask_prev(C.rsm, n - 1);
            if (lr >= 0) {
                const int2 f = raw[base + lr];
                S.rf_x = f.x;
                S.rf_y = f.y;
                S.rf_pos = C.posv[lr];
            }
        }
        __syncthreads();
    }
}

// Stroke points, block-wide (Stroke::add_point / close, stroker.rs:204-236): a point is
// kept when it starts a sub-stroke or its f32 position differs from the previous raw
// point; no closing point is popped; points past 65,535 are dropped and start nothing.
// `jpf[k]` is the `joined` value the close events before a sub-stroke start leave on
// the previous sub-stroke (false after a Move, true after a Close).
__device__ void compact_stroke_block(CState& S, const float4* raw, const unsigned char* rsf,
                                     const unsigned char* jpf, const int* opi, int m, float4* spts, SubRec* subs,
                                     CompactSmem& C) {
    const int tid = threadIdx.x;
    for (int base = 0; base < m; base += BLOCK) {
        const int k = base + tid;
        const bool valid = k < m;
        const int nb = min(BLOCK, m - base);
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        int rs = 0;
        if (valid) {
            p = raw[k];
            rs = rsf[k];
        }
        const int count0 = S.s_count, nsub0 = S.s_nsubs;
        float qx = S.s_prev_x, qy = S.s_prev_y;
        if (tid > 0 && valid) {
            qx = raw[k - 1].x;
            qy = raw[k - 1].y;
        }
        const bool keep = valid && (rs || !(p.x == qx && p.y == qy));
        int tot;
        const int pos = count0 + block_excl_sum(keep ? 1 : 0, C.scan, tot);
        const bool acc = keep && pos < PT_CAP;
        int tot_rs;
        const int sid = nsub0 + block_excl_sum((acc && rs) ? 1 : 0, C.scan, tot_rs);
        if (acc) spts[pos] = p;
        if (acc && rs) {
            subs[sid].start = pos;
            if (sid > 0) subs[sid - 1].joined = jpf[k];  // the last sub-stroke's is set by finish_subs
        }
        const int la = block_incl_max(acc ? tid : -1, C.scan);  // last accepted point of the step
        const int capped = __syncthreads_or(keep && pos >= PT_CAP);
        if (tid == BLOCK - 1) {
            S.s_count = min(count0 + tot, PT_CAP);
            S.s_nsubs = nsub0 + tot_rs;
            const float4 l = raw[base + nb - 1];
            S.s_prev_x = l.x;
            S.s_prev_y = l.y;
            S.s_has_prev = 1;
            if (la >= 0) S.s_last_op = opi[base + la];
            if (capped) S.s_capped = 1;
        }
        __syncthreads();
        if (capped) return;
    }
}

// Sizes of the sub-strokes and their outline items (stroker.rs:87-96, 239-262).  The
// last sub-stroke is joined when the last close event after its last point was a
// Close; when the 65,535 cap stopped the point stream, that is the last Close or Move
// op after the op of the last kept point.
__device__ void finish_subs(const KParams& P, const ft_path_desc& d, CState& S, SubRec* subs, int* tmp) {
    const int tid = threadIdx.x;
    const int nsub = S.s_nsubs, count = S.s_count;
    if (S.s_capped) {
        int last = -1;
        for (int i = S.s_last_op + 1 + tid; i < (int)d.n_ops; i += BLOCK) {
            const int kd = P.ops[d.op_begin + i].kind;
            if (kd == FT_OP_CLOSE || kd == FT_OP_MOVE) last = max(last, i);
        }
        last = block_incl_max(last, tmp);
        if (tid == BLOCK - 1 && nsub > 0)
            subs[nsub - 1].joined = last >= 0 ? (P.ops[d.op_begin + last].kind == FT_OP_CLOSE) : 0;
    } else if (tid == 0 && nsub > 0) {
        subs[nsub - 1].joined = S.last_pc_kind == FT_OP_CLOSE;
    }
    __syncthreads();
    int carry = 0;
    for (int s0 = 0; s0 < nsub; s0 += BLOCK) {
        const int si = s0 + tid;
        int items = 0;
        if (si < nsub) {
            SubRec r = subs[si];
            r.n = (si + 1 < nsub ? subs[si + 1].start : count) - r.start;
            // SubStroke::len with u16 arithmetic: n + 1 wraps at 65,536
            r.len = r.joined ? ((r.n + 1) & 0xFFFF) : (r.n > 0 ? r.n - 1 : 0);
            items = r.len > 0 ? 2 * r.len + 2 : 0;
            subs[si].n = r.n;
            subs[si].len = r.len;
        }
        int tot;
        const int off = block_excl_sum(items, tmp, tot);
        if (si < nsub) subs[si].item_off = carry + off;
        carry += tot;
    }
    if (tid == 0) S.s_items = carry;
    __syncthreads();
}

// stroke_offset (stroker.rs:301-309): both ends of segment (p0, p1) moved right by w/2
__device__ __forceinline__ void seg_offset(float4 p0, float4 p1, P2* r0, P2* r1) {
    const P2 vr = pnormalize(pright(psub(p2(p1.x, p1.y), p2(p0.x, p0.y))));
    *r0 = padd(p2(p0.x, p0.y), pscale(vr, __fmul_rn(p0.z, 0.5f)));
    *r1 = padd(p2(p1.x, p1.y), pscale(vr, __fmul_rn(p1.z, 0.5f)));
}

// Round-join arc (stroker.rs:399-416) walked depth first; leaves in [lo, hi) go to
// emit(index, point).  Returns the leaves walked.
template <class Emit>
__device__ int arc_walk(float4 p, P2 a, P2 b, float tol_sq, int lo, int hi, int* depth_hit, Emit emit) {
    struct Fr {
        P2 a, b;
        int d;
    };
    Fr st[FT_MAX_DEPTH + 1];
    int sp = 0, leaf = 0, d = 0;
    const float hw = __fmul_rn(p.z, 0.5f);
    for (;;) {
        const P2 vr = pnormalize(pright(psub(b, a)));
        const P2 c = padd(p2(p.x, p.y), pscale(vr, hw));
        const P2 ab = pmid(a, b);
        const bool leafy = !pfinite(c) || pdist_sq(c, ab) <= tol_sq;
        if (leafy || d >= FT_MAX_DEPTH) {
            if (!leafy) *depth_hit = 1;
            if (leaf >= lo && leaf < hi) emit(leaf, b);
            leaf++;
            if (leaf >= hi || sp == 0) break;
            --sp;
            a = st[sp].a;
            b = st[sp].b;
            d = st[sp].d;
        } else {
            st[sp].a = c;
            st[sp].b = b;
            st[sp].d = d + 1;
            sp++;
            b = c;
            d++;
        }
    }
    return leaf;
}

// One outline item of a sub-stroke: the start point, one join, or the end point of a
// side (stroker.rs:265-295, 323-396).  Emits its points in order through emit(k, pt)
// for k in [lo, hi) and returns how many it has.
template <class Emit>
__device__ int outline_item(const KParams& P, const float4* spts, const SubRec& sr, int u, int lo, int hi,
                            int* depth_hit, Emit emit) {
    const int len = sr.len, n = sr.n, s = sr.start;
    const bool joined = sr.joined != 0;
    const bool rev = u > len;
    const int j = rev ? u - len - 1 : u;  // iteration on this side; j == len is the end item
    auto v0 = [&](int jj) { return rev ? s + ((n - 1 - jj) % n + n) % n : s + (jj % n); };
    auto v1 = [&](int jj) { return rev ? s + ((n - 2 - jj) % n + n) % n : s + ((jj + 1) % n); };
    auto seg = [&](int jj, P2* r0, P2* r1) { seg_offset(spts[v0(jj)], spts[v1(jj)], r0, r1); };
    if (j == len) {  // end of an open side: the last offset point
        if (joined) return 0;
        P2 r0, r1;
        seg(len - 1, &r0, &r1);
        if (lo <= 0 && 0 < hi) emit(0, r1);
        return 1;
    }
    if (j == 0) {  // start of an open side: butt end
        if (joined) return 0;
        P2 r0, r1;
        seg(0, &r0, &r1);
        if (lo <= 0 && 0 < hi) emit(0, r0);
        return 1;
    }
    P2 a0, a1, b0, b1;
    seg(j - 1, &a0, &a1);
    seg(j, &b0, &b1);
    if (P.join == FT_JOIN_MITER) {  // stroker.rs:340-367 (the decision as ft_fmath.h takes it)
        const P2 u = psub(a1, a0), v = psub(b0, b1);
        P2 xp;
        if (ft_miter_join(u.x, u.y, v.x, v.y, P.miter_g) && pline_x(a0, a1, b0, b1, &xp)) {
            if (lo <= 0 && 0 < hi) emit(0, xp);
            return 1;
        }
    } else if (P.join == FT_JOIN_ROUND) {  // stroker.rs:380-396
        const P2 u = psub(a1, a0), v = psub(b0, b1);
        if (ft_round_join_arc(u.x, u.y, v.x, v.y)) {
            if (lo <= 0 && 0 < hi) emit(0, a1);
            const int na = arc_walk(spts[v0(j)], a1, b0, P.tol_sq, max(lo - 1, 0), hi - 1, depth_hit,
                                    [&](int k, P2 q) { emit(k + 1, q); });
            return 1 + na;
        }
    }
    // bevel (stroker.rs:370-373)
    if (lo <= 0 && 0 < hi) emit(0, a1);
    if (lo <= 1 && 1 < hi) emit(1, b0);
    return 2;
}

// Stroke outline -> figure: outline items in chunks of BLOCK (count, scan, then emit
// window by window through the second transform, plotter.rs:356-365 / 219-224) into
// the same figure builder a fill uses.
__device__ void build_outline(const KParams& P, CState& S, const float4* spts, const SubRec* subs, BuildSmem& B,
                              CompactSmem& Cs, int2* pts, int* ss) {
    const int tid = threadIdx.x;
    const int total_items = S.s_items, nsub = S.s_nsubs;
    if (tid == 0) {
        S.count = 0;
        S.has_prev = 0;
        S.prev_x = S.prev_y = 0;
        S.rf_x = S.rf_y = 0;
        S.rf_pos = 0;
        S.capped = 0;
    }
    __syncthreads();
    for (int t0 = 0; t0 < total_items; t0 += BLOCK) {
        const int t = t0 + tid;
        int n = 0, si = -1, u = 0, rsk = -1;  // rsk: index of this item's point that starts a figure run
        SubRec sr;
        int depth_hit = 0;
        P2 c0 = p2(0.f, 0.f), c1 = p2(0.f, 0.f);  // the item's first two points, kept for the emit pass
        if (t < total_items) {
            // the last sub-stroke with item_off <= t owns item t (empty ones share the
            // next one's offset and come before it)
            int lo = 0, hi = nsub - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (subs[mid].item_off <= t)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            si = lo;
            sr = subs[si];
            u = t - sr.item_off;
            n = outline_item(P, spts, sr, u, 0, INT_MAX, &depth_hit, [&](int k, P2 q) {
                if (k == 0) c0 = q;
                if (k == 1) c1 = q;
            });
            // a figure run starts at each side's first point after a Close: the forward
            // side always (after the previous sub-stroke's Close, or first), the reverse
            // side when the sub-stroke is joined (stroker.rs:255-260)
            const bool rev = u > sr.len;
            const int j = rev ? u - sr.len - 1 : u;
            const bool joined = sr.joined != 0;
            if (!rev && ((!joined && j == 0) || (joined && j == 1))) rsk = 0;
            if (rev && joined && j == 1) rsk = 0;
        }
        if (depth_hit) atomicOr(&S.flags, 1);
        int total;
        const int off = block_excl_sum(n, B.scan, total);
        for (int w0 = 0; w0 < total; w0 += RAW_CAP) {
            const int w1 = min(w0 + RAW_CAP, total);
            if (n > 0 && off < w1 && off + n > w0) {
                const int lo = max(w0, off) - off, hi = min(w1, off + n) - off;
                auto put = [&](int k, P2 q) {
                    const int idx = off + k - w0;
                    const P2 tq = xform(P.xf, q);  // the outline is transformed again (F9)
                    B.raw[idx] = make_int2(f2fx(tq.x), f2fx(tq.y));
                    B.rs[idx] = (k == rsk) ? (unsigned char)1 : (unsigned char)0;
                };
                if (n <= 2) {  // an end, a miter or a bevel: the points of the count pass
                    for (int k = lo; k < hi; k++) put(k, k == 0 ? c0 : c1);
                } else {
                    int dh = 0;
                    outline_item(P, spts, sr, u, lo, hi, &dh, put);
                }
            }
            __syncthreads();
            compact_window_block(S, B.raw, B.rs, w1 - w0, pts, ss, Cs);
            __syncthreads();
            if (S.capped) break;
        }
        __syncthreads();
        if (S.capped) break;
    }
    // Plotter::fill ends with fig.close() (plotter.rs:347)
    if (tid == 0 && !S.capped && S.has_prev && S.rf_x == S.prev_x && S.rf_y == S.prev_y) S.count -= 1;
    __syncthreads();
}

// Path walk + flattening by the thread group G.
// Fill (Plotter::fill, plotter.rs:339-350): builds the figure in pts[0..S.count) / ss[];
// `limit` is the vertex capacity of pts/ss (a warp stops with S.overflow set beyond it).
// STROKE (Plotter::stroke, plotter.rs:356-365, first half): collects the stroke points
// with their widths in spts[0..S.s_count) and the sub-strokes in subs[0..S.s_nsubs).
// Global raw store of a CTA figure build (SCR_RAWG ...); null: windows of raw
// vertices in shared memory, each emitted by re-walking the ops that reach it.
struct RawStore {
    float4* p4 = nullptr;
    unsigned char* rs = nullptr;
    unsigned char* jp = nullptr;
    int* opi = nullptr;
};
__device__ __forceinline__ RawStore raw_store(unsigned char* scr, const ScrLayout& L = scr_layout(PT_CAP)) {
    RawStore r;
    r.p4 = reinterpret_cast<float4*>(scr + L.rawg);
    r.rs = scr + L.rsg;
    r.jp = scr + L.jpg;
    r.opi = reinterpret_cast<int*>(scr + L.opig);
    return r;
}

template <class G, bool STROKE = false>
__device__ void build_fill(const KParams& P, const ft_path_desc& d, float sw0, BuildSmemT<G::N, G::RAW>& B,
                           CompactSmem* Cs, CState& S, int2* pts, int* ss, int limit, float4* spts = nullptr,
                           SubRec* subs = nullptr, int* opi = nullptr, RawStore rg = RawStore()) {
    constexpr int N = G::N;
    const int tid = G::rank();
    if (tid == 0) {
        S.pen_x = 0.f;
        S.pen_y = 0.f;
        S.pen_w = sw0;
        S.sw = sw0;
        S.last_pc_kind = -1;
        S.count = 0;
        S.has_prev = 0;
        S.prev_x = S.prev_y = 0;
        S.rf_x = S.rf_y = 0;
        S.rf_pos = 0;
        S.capped = 0;
        S.overflow = 0;
        S.flags = 0;
        S.s_count = S.s_nsubs = S.s_capped = S.s_has_prev = 0;
        S.s_last_op = -1;
        S.s_prev_x = S.s_prev_y = 0.f;
    }
    G::sync();
    constexpr int WIN = STROKE ? SRAW : G::RAW;
    const ft_op* ops = P.ops + d.op_begin;
    const int n_ops = (int)d.n_ops;
    const float tol_sq = P.tol_sq;
    for (int c0 = 0; c0 < n_ops; c0 += N) {
        const int i = c0 + tid;
        const bool valid = i < n_ops;
        ft_op op;
        if (valid) {
            const int4* src = reinterpret_cast<const int4*>(ops + i);
            int4 q0 = __ldg(src), q1 = __ldg(src + 1);
            op.kind = q0.x;
            op.v[0] = __int_as_float(q0.y);
            op.v[1] = __int_as_float(q0.z);
            op.v[2] = __int_as_float(q0.w);
            op.v[3] = __int_as_float(q1.x);
            op.v[4] = __int_as_float(q1.y);
            op.v[5] = __int_as_float(q1.z);
        } else {
            op.kind = -1;
            for (int j = 0; j < 6; j++) op.v[j] = 0.f;
        }
        int kind = op.kind;
        if (kind < -1 || kind > FT_OP_PEN_WIDTH) {
            atomicOr(&S.flags, 2);
            kind = -1;
        }
        const bool isPW = kind == FT_OP_PEN_WIDTH;
        const bool isPC = kind >= FT_OP_CLOSE && kind <= FT_OP_CUBIC;
        B.kind[tid] = kind;
        B.pwval[tid] = op.v[0];
        // pen width in effect at this op (last PenWidth at or before it)
        const int lpw = G::incl_max(isPW ? tid : -1, B.scan);
        G::sync();
        const float sw_i = lpw >= 0 ? B.pwval[lpw] : S.sw;
        if (isPC) {
            float ex = 0.f, ey = 0.f;  // Close resets the pen to the origin (plotter.rs:200-203)
            if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
                ex = op.v[0];
                ey = op.v[1];
            } else if (kind == FT_OP_QUAD) {
                ex = op.v[2];
                ey = op.v[3];
            } else if (kind == FT_OP_CUBIC) {
                ex = op.v[4];
                ey = op.v[5];
            }
            B.penx[tid] = ex;
            B.peny[tid] = ey;
            B.penw[tid] = sw_i;
        }
        // pen before this op = pen after the last Move/Line/Quad/Cubic/Close before it
        int lpc_inc, lpc;
        G::max_scan(isPC ? tid : -1, B.scan, lpc_inc, lpc);
        G::sync();
        float pen_x, pen_y, pen_w;
        int prev_pc_kind;
        if (lpc >= 0) {
            pen_x = B.penx[lpc];
            pen_y = B.peny[lpc];
            pen_w = B.penw[lpc];
            prev_pc_kind = B.kind[lpc];
        } else {
            pen_x = S.pen_x;
            pen_y = S.pen_y;
            pen_w = S.pen_w;
            prev_pc_kind = S.last_pc_kind;
        }
        // widths of a curve's control points (plotter.rs:235-236, 294-298)
        float wa = pen_w, wb = 0.f, wc = 0.f, wd = sw_i;
        if (STROKE) {
            if (kind == FT_OP_QUAD) {
                wb = __fmul_rn(__fadd_rn(pen_w, sw_i), 0.5f);
                wc = sw_i;
            } else if (kind == FT_OP_CUBIC) {
                wb = __fadd_rn(sw_i, __fmul_rn(__fsub_rn(pen_w, sw_i), 1.0f / 3.0f));
                wc = __fadd_rn(sw_i, __fmul_rn(__fsub_rn(pen_w, sw_i), 2.0f / 3.0f));
            }
        }
        // the first vertex of this op starts a sub-figure after a close event
        const int rs = (kind == FT_OP_MOVE) || prev_pc_kind == FT_OP_CLOSE || prev_pc_kind == -1;

        // ---- count the vertices this op adds
        int n = 0;
        int depth_hit = 0;
        bool nonfinite = false;
        constexpr int LC = G::N == 32 ? LEAF_CACHE : LEAF_CACHE_CTA;
        int2 cache[LC];  // leaves of the count pass, reused by the emit pass
        auto keep_leaf = [&](int k, P2 q, float) {
            if (k < LC) cache[k] = make_int2(f2fx(q.x), f2fx(q.y));
        };
        P2 A = p2(0, 0), Bq = p2(0, 0), C = p2(0, 0), D = p2(0, 0);
        if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
            A = xform(P.xf, p2(op.v[0], op.v[1]));
            n = 1;
        } else if (kind == FT_OP_QUAD) {
            A = xform(P.xf, p2(pen_x, pen_y));
            Bq = xform(P.xf, p2(op.v[0], op.v[1]));
            C = xform(P.xf, p2(op.v[2], op.v[3]));
            if (!pfinite(A) || !pfinite(Bq) || !pfinite(C)) {
                nonfinite = true;
                n = 1;
            } else if (STROKE) {
                n = quad_walk<true>(A, Bq, C, wa, wb, wc, tol_sq, 0, INT_MAX, &depth_hit, [](int, P2, float) {});
            } else {
                n = quad_walk<false>(A, Bq, C, 0.f, 0.f, 0.f, tol_sq, 0, INT_MAX, &depth_hit, keep_leaf);
            }
        } else if (kind == FT_OP_CUBIC) {
            A = xform(P.xf, p2(pen_x, pen_y));
            Bq = xform(P.xf, p2(op.v[0], op.v[1]));
            C = xform(P.xf, p2(op.v[2], op.v[3]));
            D = xform(P.xf, p2(op.v[4], op.v[5]));
            if (!pfinite(A) || !pfinite(Bq) || !pfinite(C) || !pfinite(D)) {
                nonfinite = true;
                n = 1;
            } else if (STROKE) {
                n = cubic_walk<true>(A, Bq, C, D, wa, wb, wc, wd, tol_sq, 0, INT_MAX, &depth_hit,
                                     [](int, P2, float) {});
            } else {
                n = cubic_walk<false>(A, Bq, C, D, 0.f, 0.f, 0.f, 0.f, tol_sq, 0, INT_MAX, &depth_hit,
                                      keep_leaf);
            }
        }
        if (depth_hit) atomicOr(&S.flags, 1);
        if (nonfinite) atomicOr(&S.flags, 2);
        int total;
        const int off = G::excl_sum(n, B.scan, total);
        // carry the path-walk state to the next chunk (everyone has read S by now)
        if (tid == N - 1) {
            S.sw = sw_i;
            int last_pc = isPC ? tid : lpc;
            if (last_pc >= 0) {
                S.pen_x = B.penx[last_pc];
                S.pen_y = B.peny[last_pc];
                S.pen_w = B.penw[last_pc];
                S.last_pc_kind = B.kind[last_pc];
            }
        }
        if (G::N != 32 && rg.p4 && total > WIN) {
            // ---- a chunk of several windows: emit every op's vertices once into the raw
            //      store (super-windows of RAWG when the chunk has more), then compact the
            //      store window by window
            for (int g0 = 0; g0 < total; g0 += RAWG) {
                const int g1 = min(g0 + RAWG, total);
                if (n > 0 && off < g1 && off + n > g0) {
                    const int lo = max(g0, off) - off, hi = min(g1, off + n) - off;
                    if (STROKE) {
                        auto emit = [&](int k, P2 q, float w) {
                            const int idx = off + k - g0;
                            rg.p4[idx] = make_float4(q.x, q.y, w, 0.f);
                            rg.rs[idx] = (k == 0) ? (unsigned char)rs : (unsigned char)0;
                            rg.jp[idx] = (unsigned char)(kind != FT_OP_MOVE);
                            rg.opi[idx] = i;
                        };
                        if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
                            emit(0, A, sw_i);
                        } else if (nonfinite) {
                            emit(0, kind == FT_OP_QUAD ? C : D, kind == FT_OP_QUAD ? wc : wd);
                        } else if (kind == FT_OP_QUAD) {
                            int dh = 0;
                            quad_walk<true>(A, Bq, C, wa, wb, wc, tol_sq, lo, hi, &dh, emit);
                        } else {
                            int dh = 0;
                            cubic_walk<true>(A, Bq, C, D, wa, wb, wc, wd, tol_sq, lo, hi, &dh, emit);
                        }
                    } else {
                        int2* raw2 = reinterpret_cast<int2*>(rg.p4);
                        auto emit = [&](int k, P2 q, float) {
                            const int idx = off + k - g0;
                            raw2[idx] = make_int2(f2fx(q.x), f2fx(q.y));
                            rg.rs[idx] = (k == 0) ? (unsigned char)rs : (unsigned char)0;
                        };
                        if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
                            emit(0, A, 0.f);
                        } else if (nonfinite) {
                            emit(0, kind == FT_OP_QUAD ? C : D, 0.f);
                        } else if (n <= LC) {
                            for (int k = lo; k < hi; k++) {
                                const int idx = off + k - g0;
                                raw2[idx] = cache[k];
                                rg.rs[idx] = (k == 0) ? (unsigned char)rs : (unsigned char)0;
                            }
                        } else if (kind == FT_OP_QUAD) {
                            int dh = 0;
                            quad_walk<false>(A, Bq, C, 0.f, 0.f, 0.f, tol_sq, lo, hi, &dh, emit);
                        } else {
                            int dh = 0;
                            cubic_walk<false>(A, Bq, C, D, 0.f, 0.f, 0.f, 0.f, tol_sq, lo, hi, &dh, emit);
                        }
                    }
                }
                G::sync();
                for (int w0 = g0; w0 < g1; w0 += WIN) {
                    const int w1 = min(w0 + WIN, g1), o = w0 - g0;
                    if (STROKE)
                        compact_stroke_block(S, rg.p4 + o, rg.rs + o, rg.jp + o, rg.opi + o, w1 - w0, spts, subs, *Cs);
                    else
                        compact_window_block(S, reinterpret_cast<const int2*>(rg.p4) + o, rg.rs + o, w1 - w0, pts, ss,
                                             *Cs, limit);
                    G::sync();
                    if (S.capped || S.overflow || S.s_capped) break;
                }
                if (S.capped || S.overflow || S.s_capped) break;
            }
        } else {
            // ---- emit and compact window by window
            for (int w0 = 0; w0 < total; w0 += WIN) {
                const int w1 = min(w0 + WIN, total);
                if (n > 0 && off < w1 && off + n > w0) {
                    const int lo = max(w0, off) - off, hi = min(w1, off + n) - off;
                    if (STROKE) {
                        // stroke points keep f32 coordinates and their width (stroker.rs:204-225)
                        float4* raw4 = reinterpret_cast<float4*>(B.raw);
                        auto emit = [&](int k, P2 q, float w) {
                            const int idx = off + k - w0;
                            raw4[idx] = make_float4(q.x, q.y, w, 0.f);
                            B.rs[idx] = (k == 0) ? (unsigned char)rs : (unsigned char)0;
                            // a Move closes the previous sub-stroke open, a Close joined (F7)
                            B.rs[SRAW + idx] = (unsigned char)(kind != FT_OP_MOVE);
                            opi[idx] = i;
                        };
                        if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
                            emit(0, A, sw_i);
                        } else if (nonfinite) {
                            emit(0, kind == FT_OP_QUAD ? C : D, kind == FT_OP_QUAD ? wc : wd);
                        } else if (kind == FT_OP_QUAD) {
                            int dh = 0;
                            quad_walk<true>(A, Bq, C, wa, wb, wc, tol_sq, lo, hi, &dh, emit);
                        } else {
                            int dh = 0;
                            cubic_walk<true>(A, Bq, C, D, wa, wb, wc, wd, tol_sq, lo, hi, &dh, emit);
                        }
                    } else {
                        auto emit = [&](int k, P2 q, float) {
                            int idx = off + k - w0;
                            B.raw[idx] = make_int2(f2fx(q.x), f2fx(q.y));
                            B.rs[idx] = (k == 0) ? (unsigned char)rs : (unsigned char)0;
                        };
                        if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
                            emit(0, A, 0.f);
                        } else if (nonfinite) {
                            emit(0, kind == FT_OP_QUAD ? C : D, 0.f);
                        } else if (n <= LC) {
                            for (int k = lo; k < hi; k++) {
                                const int idx = off + k - w0;
                                B.raw[idx] = cache[k];
                                B.rs[idx] = (k == 0) ? (unsigned char)rs : (unsigned char)0;
                            }
                        } else if (kind == FT_OP_QUAD) {
                            int dh = 0;
                            quad_walk<false>(A, Bq, C, 0.f, 0.f, 0.f, tol_sq, lo, hi, &dh, emit);
                        } else {
                            int dh = 0;
                            cubic_walk<false>(A, Bq, C, D, 0.f, 0.f, 0.f, 0.f, tol_sq, lo, hi, &dh, emit);
                        }
                    }
                }
                G::sync();
                if constexpr (STROKE) {
                    compact_stroke_block(S, reinterpret_cast<const float4*>(B.raw), B.rs, B.rs + SRAW, opi, w1 - w0,
                                         spts, subs, *Cs);
                } else if (N == 32) {
                    compact_window(S, B.raw, B.rs, w1 - w0, pts, ss, limit);
                } else if (BLOCK_COMPACT) {
                    compact_window_block(S, B.raw, B.rs, w1 - w0, pts, ss, *Cs, limit);
                } else if (tid < 32) {
                    compact_window(S, B.raw, B.rs, w1 - w0, pts, ss, limit);
                }
                G::sync();
                if (S.capped || S.overflow || S.s_capped) break;
            }
        }
        G::sync();
        if (S.capped || S.overflow || S.s_capped) break;
    }
    if (STROKE) {
        G::sync();
        return;
    }
    // Plotter::fill ends with fig.close() (plotter.rs:347)
    if (tid == 0 && !S.capped && !S.overflow && S.has_prev && S.rf_x == S.prev_x && S.rf_y == S.prev_y)
        S.count -= 1;
    G::sync();
}

// Direction of a figure from its top vertex `top` (fig.rs:402-411): the vertex after it
// and the one before it in its sub-figure.
__device__ int fig_dir(int top, int count, const int2* pts, const int* ss) {
    const int s = ss[top];
    const int nf = (top + 1 < count && ss[top + 1] == s) ? top + 1 : s;
    int nr;
    if (top > s) {
        nr = top - 1;
    } else {
        // last vertex of the sub-figure: ss[] is non-decreasing
        int lo = top, hi = count - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (ss[mid] == s)
                lo = mid;
            else
                hi = mid - 1;
        }
        nr = lo;
    }
    int2 p = pts[top], p0 = pts[nf], p1 = pts[nr];
    int ax = wsub(p1.x, p.x), ay = wsub(p1.y, p.y);
    int cx = wsub(p0.x, p.x), cy = wsub(p0.y, p.y);
    // (p1 - p).widdershins(p0 - p) -> Forward   (fig.rs:116-119)
    return (fxmul(ax, cy) > fxmul(cx, ay)) ? 0 : 1;
}

// min (y, x, id)
__device__ __forceinline__ bool top_less(int ay, int ax, int ai, int by, int bx, int bi) {
    return ay < by || (ay == by && (ax < bx || (ax == bx && ai < bi)));
}

// Top vertex (min (y, x, id)) and figure direction (fig.rs:402-411, 493-496).
template <class G>
__device__ void top_and_dir(CState& S, const int2* pts, const int* ss, int* tmp3) {
    const int tid = G::rank(), lane = threadIdx.x & 31, w = tid >> 5;
    const int count = S.count;
    int by = INT_MAX, bx = INT_MAX, bi = INT_MAX;
    for (int i = tid; i < count; i += G::N) {
        int2 p = pts[i];
        if (p.y < by || (p.y == by && (p.x < bx || (p.x == bx && i < bi)))) {
            by = p.y;
            bx = p.x;
            bi = i;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        int oy = __shfl_down_sync(FULL, by, o), ox = __shfl_down_sync(FULL, bx, o), oi = __shfl_down_sync(FULL, bi, o);
        if (oy < by || (oy == by && (ox < bx || (ox == bx && oi < bi)))) {
            by = oy;
            bx = ox;
            bi = oi;
        }
    }
    if (G::N > 32) {
        if (lane == 0) {
            tmp3[3 * w] = by;
            tmp3[3 * w + 1] = bx;
            tmp3[3 * w + 2] = bi;
        }
        G::sync();
    }
    if (tid == 0) {
        for (int k = 1; k < G::N / 32; k++) {
            int oy = tmp3[3 * k], ox = tmp3[3 * k + 1], oi = tmp3[3 * k + 2];
            if (oy < by || (oy == by && (ox < bx || (ox == bx && oi < bi)))) {
                by = oy;
                bx = ox;
                bi = oi;
            }
        }
        S.dir = fig_dir(bi, count, pts, ss);
        S.top_row = by >> 16;
    }
    G::sync();
}

// One edge per non-horizontal segment (fig.rs:179-201, 576-600).
// Edge from vertex i to the next vertex of its sub-figure (fig.rs:179-210, 402-411): its
// rows, slope and direction relative to the figure's; horizontal and degenerate edges
// have ed == 0.
__device__ __forceinline__ EdgeRec edge_rec(int i, int count, int figdir, const int2* pts, const int* ss) {
    const int s = ss[i];
    const int nx = (i + 1 < count && ss[i + 1] == s) ? i + 1 : s;
    EdgeRec e;
    e.ed = 0;
    e.y_upper = e.y_lower = e.x_bot0 = e.inv_slope = e.step_pix = e.start_row = e.end_row = 0;
    if (nx != i) {
        int2 a = pts[i], b = pts[nx];
        if (a.y != b.y) {
            int2 up, lo;
            int edir;
            if (b.y > a.y) {
                up = a;
                lo = b;
                edir = 0;
            } else {
                up = b;
                lo = a;
                edir = 1;
            }
            const int dx = wsub(lo.x, up.x), dy = wsub(lo.y, up.y);
            const int step = dx != 0 ? min(fxabs(fxdiv(dy, dx)), FX_ONE) : 0;
            const int inv = fxdiv(dx, dy);
            const int ybot = wsub(fxfloor(wadd(up.y, FX_ONE)), up.y);
            e.y_upper = up.y;
            e.y_lower = lo.y;
            e.x_bot0 = wadd(up.x, fxmul(inv, ybot));
            e.inv_slope = inv;
            e.step_pix = step;
            e.ed = (edir == figdir) ? 1 : -1;
            e.start_row = up.y >> 16;
            e.end_row = lo.y >> 16;
        }
    }
    return e;
}

template <class G>
__device__ void build_edges(const CState& S, const int2* pts, const int* ss, EdgeRec* edges) {
    const int count = S.count, figdir = S.dir;
    for (int i = G::rank(); i < count; i += G::N) edges[i] = edge_rec(i, count, figdir, pts, ss);
}

// Count one warp's edges by first scan row into hist[0 .. nrows) (zeroed by the
// caller) for raster_sweep_warp's buckets: the rows of edge_rec's non-horizontal
// edges, from the vertices alone (the records are built once, into their buckets).
__device__ void count_edges_warp(const CState& S, const int2* pts, const int* ss, int* hist, int nrows) {
    const int count = S.count, top_row = S.top_row;
    for (int i = threadIdx.x & 31; i < count; i += 32) {
        const int s = ss[i];
        const int nx = (i + 1 < count && ss[i + 1] == s) ? i + 1 : s;
        if (nx == i) continue;
        const int ay = pts[i].y, by = pts[nx].y;
        if (ay == by) continue;
        const long long b = (long long)(min(ay, by) >> 16) - top_row;
        if (b < nrows) atomicAdd(&hist[b], 1);
    }
}

// Signed cell areas of one edge on one scan row (fig.rs:238-321), added into
// `area` (the band row of width W).  The edge on this row: x_bot where it leaves the
// row, its inverse slope, whether the row is its first (st) or last (en), the 16.16
// fractions of its upper and lower y, the cell step (1 .. ONE) and its direction ed.
// With `spans`, the 128-pixel spans holding the touched cells are marked too.
__device__ __forceinline__ void scan_row(int x_bot, int inv, bool st, bool en, int fu, int fl, int step, int ed,
                                         int* area, int W, unsigned* spans) {
    const int ccov = en ? pixel_cov(fl) : 256;
    const int cov = st ? ccov - pixel_cov(fu) : ccov;
    if (cov <= 0) return;
    const int x0 = st ? wsub(x_bot, fxmul(inv, wsub(FX_ONE, fu))) : wsub(x_bot, inv);
    // fxceil(y_lower) - y_lower, from the fraction alone
    const int x1 = en ? wsub(x_bot, fxmul(inv, fl ? FX_ONE - fl : 0)) : x_bot;
    const int mnx = min(x0, x1), mxx = max(x0, x1);
    const int minp = mnx >> 16, maxp = mxx >> 16;
    if (minp >= W) return;
    const int full = cov << 8;
    const int r = (minp == maxp) ? fxmul(wsub(FX_ONE, fxfract(fxavg(mxx, mnx))), full)
                                 : fxmul(wsub(FX_ONE, fxfract(mnx)), FX_HALF);
    const int first = fxmul(r, step);  // fxmul(r, ONE) == r
    // fig.rs:292-301: x_cov runs first, first + step, ... capped at ONE; each cell
    // gets the growth of min(pixel_cov(x_cov), cov) until it reaches cov
    const int jmax = W - 1 - minp;  // the loop also stops at the raster's last cell
    int j, prev, x_cov;
    const int cell0 = max(minp, 0);
    int cell1 = cell0;
    if (minp < 0) {
        // cells left of the raster all land in cell 0 (fig.rs:295): their sum telescopes
        j = -minp;
        long long v = (long long)first + (long long)j * step;
        x_cov = v > FX_ONE ? FX_ONE : (int)v;
        prev = min(pixel_cov(x_cov), cov);
        if (prev && ck(W > 0, 1)) atomicAdd(&area[0], ed * prev);
        j++;
        x_cov = min(x_cov + step, FX_ONE);
    } else {
        j = 0;
        prev = 0;
        x_cov = first;
    }
    if (prev < cov) {
        for (; j <= jmax; j++) {
            const int v = min(pixel_cov(x_cov), cov);
            const int p = v - prev;
            prev = v;
            if (p && ck(minp + j >= 0 && minp + j < W, 2)) atomicAdd(&area[minp + j], ed * p);
            cell1 = minp + j;
            if (v >= cov) break;
            x_cov = min(x_cov + step, FX_ONE);
        }
    }
    if (spans)
        for (int sp = cell0 >> 7; sp <= (cell1 >> 7); sp++) atomicOr(&spans[sp >> 5], 1u << (sp & 31));
}

// The cell step of an edge, step_cov(ONE) (fig.rs:315-321): step_pix when positive,
// else ONE; first_cov's r * step equals step_cov(r) for both.
__device__ __forceinline__ int cell_step(const EdgeRec& E) { return E.step_pix > 0 ? E.step_pix : FX_ONE; }

__device__ __forceinline__ void scan_item(const EdgeRec& E, int y, int* area, int W, unsigned* spans = nullptr) {
    const int x_bot = wadd(E.x_bot0, wmul(y - E.start_row, E.inv_slope));
    scan_row(x_bot, E.inv_slope, y == E.start_row, y == E.end_row, fxfract(E.y_upper), fxfract(E.y_lower),
             cell_step(E), E.ed, area, W, spans);
}

// Edge record of the warp sweep, 16 bytes, relative to the figure's top row t (rows
// t .. t + 511 at most): x where the edge would leave row t (wrapping, like the row
// steps), the inverse slope, the two y fractions, and the cell step with the end row
// and the direction.  The first row is the bucket the record sits in.
__device__ __forceinline__ int4 sweep_rec(const EdgeRec& E, int t) {
    int4 R;
    R.x = wsub(E.x_bot0, wmul(E.start_row - t, E.inv_slope));
    R.y = E.inv_slope;
    R.z = fxfract(E.y_upper) | (fxfract(E.y_lower) << 16);
    R.w = (cell_step(E) - 1) | (min(E.end_row - t, SWEEP_END_FAR) << 16) | ((E.ed < 0) << 26);
    return R;
}
__device__ __forceinline__ int sweep_end(int4 R) { return (R.w >> 16) & 1023; }

// scan_item for a sweep record on row t + s; st: s is its first row.
__device__ __forceinline__ void scan_sweep(int4 R, int s, bool st, int* row, int W) {
    scan_row(wadd(R.x, wmul(s, R.y)), R.y, st, s == sweep_end(R), R.z & FX_MASK, (int)((unsigned)R.z >> 16),
             (R.w & FX_MASK) + 1, (R.w >> 26) & 1 ? -1 : 1, row, W, nullptr);
}

// Resolve one band row and write it (fig.rs:621-665, imgbuf.rs:38-199).  With WORDS
// (rasters in mapped host memory), Matte8 rows are written as aligned 4-byte words
// whatever the row's alignment: lane L of a step stores the word at row position x - a
// (a = the row's misalignment), made of the last a bytes of the previous lane's four
// pixels and the first 4 - a of its own; the words at the row's ends are written byte by
// byte inside the row — no partial words cross the host link.  In device memory the byte
// stores of a misaligned row cost less than the shuffles.
template <bool ZERO, bool WORDS>
__device__ __forceinline__ void resolve_row(int* arow, int W, int Wp, uint8_t* drow, int rule, int fmt,
                                            unsigned clr) {
    const int lane = threadIdx.x & 31;
    unsigned carry = 0;
    const int mis = WORDS ? (int)(reinterpret_cast<uintptr_t>(drow) & 3) : 0;
    const int xend = (WORDS && fmt == FT_MATTE8) ? W + mis : W;
    unsigned pcarry = 0;  // Matte8: the previous step's last four pixels
    for (int x0 = 0; x0 < xend; x0 += 128) {
        const int x = x0 + lane * 4;
        int4 a = make_int4(0, 0, 0, 0);
        if (x < Wp) {
            a = *reinterpret_cast<const int4*>(arow + x);
            if (ZERO) *reinterpret_cast<int4*>(arow + x) = make_int4(0, 0, 0, 0);
        }
        const unsigned s0 = (unsigned)a.x;
        const unsigned s1 = s0 + (unsigned)a.y;
        const unsigned s2 = s1 + (unsigned)a.z;
        const unsigned s3 = s2 + (unsigned)a.w;
        const unsigned inc = warp_incl_sum_u(s3);
        const unsigned ex = inc - s3 + carry;
        carry += __shfl_sync(FULL, inc, 31);
        const unsigned v0 = resolve_cov(s0 + ex, rule), v1 = resolve_cov(s1 + ex, rule);
        const unsigned v2 = resolve_cov(s2 + ex, rule), v3 = resolve_cov(s3 + ex, rule);
        if (fmt == FT_MATTE8 && !WORDS) {
            if (x >= W) continue;
            uint8_t* dp = drow + x;
            if (x + 3 < W && ((reinterpret_cast<uintptr_t>(dp) & 3) == 0)) {
                // masks are written once and not read back: stream them past L2 (evict first),
                // leaving L2 to the rasterisers' figure scratch
                const unsigned px4 = v0 | (v1 << 8) | (v2 << 16) | (v3 << 24);
                if (__isGlobal(dp))
                    __stcs(reinterpret_cast<unsigned*>(dp), px4);
                else
                    *reinterpret_cast<unsigned*>(dp) = px4;
            } else {
                dp[0] = (uint8_t)v0;
                if (x + 1 < W) dp[1] = (uint8_t)v1;
                if (x + 2 < W) dp[2] = (uint8_t)v2;
                if (x + 3 < W) dp[3] = (uint8_t)v3;
            }
            continue;
        }
        if (WORDS && fmt == FT_MATTE8) {
            const unsigned px4 = v0 | (v1 << 8) | (v2 << 16) | (v3 << 24);  // pixels x .. x + 3
            unsigned prev = __shfl_up_sync(FULL, px4, 1);
            if (lane == 0) prev = pcarry;
            pcarry = __shfl_sync(FULL, px4, 31);
            const unsigned word = mis ? (px4 << (8 * mis)) | (prev >> (32 - 8 * mis)) : px4;
            const int lo = x - mis;  // row position of the word's first byte (4-byte aligned address)
            uint8_t* wp = drow + lo;
            if (lo >= 0 && lo + 3 < W) {
                *reinterpret_cast<unsigned*>(wp) = word;
            } else {
#pragma unroll
                for (int b = 0; b < 4; b++)
                    if (lo + b >= 0 && lo + b < W) wp[b] = (uint8_t)(word >> (8 * b));
            }
            continue;
        }
        if (x >= W) continue;
        {
            unsigned* dp = reinterpret_cast<unsigned*>(drow) + x;
            const unsigned vv[4] = {v0, v1, v2, v3};
#pragma unroll
            for (int c = 0; c < 4; c++)
                if (x + c < W) dp[c] = srcover_rgba(dp[c], clr, vv[c]);
        }
    }
}

// Rasterise rows [lo, hi) of the built figure, `R` rows per band.
__device__ void raster_rows(const KParams& P, const ft_path_desc& d, const CState& S, const EdgeRec* edges, int lo,
                            int hi, int R, unsigned char* smem) {
    RasterSmem& Rs = *reinterpret_cast<RasterSmem*>(smem);
    int* area = reinterpret_cast<int*>(smem + ((sizeof(RasterSmem) + 15) & ~(size_t)15));
    const int tid = threadIdx.x, warp = tid >> 5;
    const int W = (int)d.width;
    const int Wp = (W + 3) & ~3;
    const int tmin = min(S.top_row, 0);
    const int count = S.count;
    const unsigned clr = (unsigned)d.clr[0] | ((unsigned)d.clr[1] << 8) | ((unsigned)d.clr[2] << 16) |
                         ((unsigned)d.clr[3] << 24);
    uint8_t* base = P.rasters + d.raster_offset;
    for (int r0 = lo; r0 < hi; r0 += R) {
        const int r1 = min(r0 + R, hi);
        const int nr = r1 - r0;
        int4* a4 = reinterpret_cast<int4*>(area);
        for (int i = tid; i < nr * Wp / 4; i += BLOCK) a4[i] = make_int4(0, 0, 0, 0);
        __syncthreads();
        const int yb0 = r0 + tmin, yb1 = r1 + tmin;
        for (int e0 = 0; e0 < count; e0 += BLOCK) {
            const int e = e0 + tid;
            int nrow = 0, ya = 0;
            EdgeRec E;
            E.ed = 0;
            if (e < count) {
                E = edges[e];
                if (E.ed) {
                    ya = max(E.start_row, yb0);
                    const int yb = min(E.end_row, yb1 - 1);
                    nrow = max(yb - ya + 1, 0);
                }
            }
            Rs.edges[tid] = E;
            Rs.ya[tid] = ya;
            int tot;
            const int o = block_excl_sum(nrow, Rs.scan, tot);
            Rs.off[tid] = o;
            // spread the chunk's (edge, row) items over the threads: each edge writes
            // its slot into a run of the item map, then every thread takes items
            for (int m0 = 0; m0 < tot; m0 += MAP_CAP) {
                const int ia = max(o, m0), ib = min(o + nrow, m0 + MAP_CAP);
                for (int k = ia; k < ib; k++) Rs.map[k - m0] = (unsigned char)tid;
                __syncthreads();
                const int n = min(MAP_CAP, tot - m0);
                for (int it = tid; it < n; it += BLOCK) {
                    const int jj = Rs.map[it];
                    const int y = Rs.ya[jj] + (m0 + it - Rs.off[jj]);
                    scan_item(Rs.edges[jj], y, area + (size_t)(y - yb0) * Wp, W);
                }
                __syncthreads();
            }
        }
        for (int rr = r0 + warp; rr < r1; rr += NWARP)
            resolve_row<false, false>(area + (size_t)(rr - r0) * Wp, W, Wp, base + (size_t)rr * d.stride, P.rule,
                                      P.fmt, clr);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Warp rasteriser: one warp per small path.  After building the figure, the warp
// sweeps the scan rows top to bottom like footile's Scanner (fig.rs:536-617):
// edges are bucketed by their first row, each row processes the active edges one
// per lane into a one-row i32 buffer, then resolves and writes the row.
struct WarpSmem {
    CState S;
    int tmp3[4];
    union __align__(16) {
        WarpBuildSmem B;
        int hist[WARP_MAX_SIDE];
    } u;
    __align__(16) int row[WARP_MAX_SIDE];  // read and cleared as int4 by resolve_row
};
static_assert(offsetof(WarpSmem, row) % 16 == 0 && sizeof(WarpSmem) % 16 == 0, "warp smem alignment");

// Rows of a mapped host raster staged in shared memory so that whole 128-byte lines cross
// the host link: a raster whose rows are contiguous (stride == width) is one byte range
// [lo, end); rows are resolved into `stg` (which holds the bytes from the line address L0
// on), then every complete line is stored with one aligned word per lane, and the partial
// line left over moves to the front of the buffer.  Bytes outside [lo, end) are never
// stored (the rows above the figure and other rasters keep theirs).
constexpr int STAGE_BYTES = 768;  // a partial line (< 128 B) and one row (<= WARP_MAX_SIDE B)
static_assert(127 + WARP_MAX_SIDE < STAGE_BYTES && STAGE_BYTES % 128 == 0, "staging holds a line and a row");
static_assert(sizeof(int) * WARP_MAX_SIDE + STAGE_BYTES <= sizeof(WarpBuildSmem), "row staging fits the build window");

__device__ __forceinline__ void stage_flush(unsigned char* stg, uint8_t*& L0, const uint8_t* lo, const uint8_t* end,
                                            bool final) {
    const int lane = threadIdx.x & 31;
    const int fill = (int)(end - L0);
    const int nfull = final ? (fill + 127) >> 7 : fill >> 7;
    for (int li = 0; li < nfull; li++) {
        const int o = (li << 7) + 4 * lane;
        uint8_t* a = L0 + o;
        const unsigned wv = *reinterpret_cast<const unsigned*>(stg + o);
        if (a >= lo && a + 4 <= end) {
            *reinterpret_cast<unsigned*>(a) = wv;
        } else {
#pragma unroll
            for (int b = 0; b < 4; b++)
                if (a + b >= lo && a + b < end) a[b] = (uint8_t)(wv >> (8 * b));
        }
    }
    if (final) return;
    const int rest = fill - (nfull << 7);  // < 128: the partial line moves to the front
    if (nfull > 0) {
        const unsigned v = *reinterpret_cast<const unsigned*>(stg + (nfull << 7) + 4 * lane);
        __syncwarp();
        if (4 * lane < rest) *reinterpret_cast<unsigned*>(stg + 4 * lane) = v;
        __syncwarp();
        L0 += nfull << 7;
    }
}

// The edge records (sweep_rec) are built straight into their buckets (`sorted`); the
// active edge list holds the records themselves (one load per edge and row from a list
// that stays small and hot, instead of an index and a record of the figure's edges).
// hist holds every start row's edge count (count_edges_warp).
template <bool WORDS>
__device__ void raster_sweep_warp(const KParams& P, const ft_path_desc& d, const CState& S, const int2* pts,
                                  const int* ss, int4* sorted, int4* active, int* hist, int* row,
                                  unsigned char* stg) {
    const int lane = threadIdx.x & 31;
    const int count = S.count, H = (int)d.height, W = (int)d.width, Wp = (W + 3) & ~3;
    const int top_row = S.top_row, row_begin = max(top_row, 0);
    const int nrows = H - row_begin;
    const unsigned clr = (unsigned)d.clr[0] | ((unsigned)d.clr[1] << 8) | ((unsigned)d.clr[2] << 16) |
                         ((unsigned)d.clr[3] << 24);
    uint8_t* base = P.rasters + d.raster_offset;
    // bucket the edges by their first scan row (edges below the last row never start)
    int carry = 0;
    for (int b0 = 0; b0 < nrows; b0 += 32) {
        const int b = b0 + lane;
        const int v = b < nrows ? hist[b] : 0;
        const int inc = warp_incl_sum(v);
        if (b < nrows) hist[b] = carry + inc - v;
        carry += __shfl_sync(FULL, inc, 31);
    }
    __syncwarp();
    for (int e = lane; e < count; e += 32) {  // the records themselves, in bucket order
        const EdgeRec E = edge_rec(e, count, S.dir, pts, ss);
        if (E.ed) {
            const long long b = (long long)E.start_row - top_row;
            if (b < nrows && ck(b >= 0, 3)) {
                const int k = atomicAdd(&hist[b], 1);
                if (ck(k >= 0 && k < WARP_CAP, 4)) sorted[k] = sweep_rec(E, top_row);
            }
        }
    }
    for (int x = lane; x < Wp; x += 32) row[x] = 0;
    __syncwarp();
    // mapped host rasters with contiguous rows go out in whole lines (stage_flush)
    const bool staged = WORDS && d.stride == d.width;
    uint8_t* const lo = base + (size_t)row_begin * d.stride;
    uint8_t* L0 = reinterpret_cast<uint8_t*>(reinterpret_cast<uintptr_t>(lo) & ~(uintptr_t)127);
    // hist[b] now ends bucket b
    int n_act = 0;
    for (int s = 0; s < nrows; s++) {
        const int bs = s == 0 ? 0 : hist[s - 1], be = hist[s];
        for (int k = lane; k < be - bs; k += 32)
            if (ck(n_act + k < WARP_CAP && bs + k < WARP_CAP, 5)) active[n_act + k] = sorted[bs + k];
        const int n_old = n_act;  // records from n_old on start on this row
        n_act += be - bs;
        __syncwarp();
        int nn = 0;
        for (int a0 = 0; a0 < n_act; a0 += 32) {
            const int idx = a0 + lane;
            const bool v = idx < n_act;
            int4 R;
            int end = -1;
            if (v) {
                R = active[idx];
                end = sweep_end(R);
                scan_sweep(R, s, idx >= n_old, row, W);
            }
            // an edge leaves the active list after its last row (fig.rs:582, 603-617);
            // records that keep their place are not rewritten
            const bool keep = v && end > s;
            const unsigned km = __ballot_sync(FULL, keep);
            const int dst = nn + __popc(km & ((1u << lane) - 1u));
            if (keep && dst != idx) active[dst] = R;
            nn += __popc(km);
        }
        n_act = nn;
        __syncwarp();
        uint8_t* drow = base + (size_t)(row_begin + s) * d.stride;
        if (staged) {
            resolve_row<true, false>(row, W, Wp, stg + (drow - L0), P.rule, P.fmt, clr);
            __syncwarp();
            stage_flush(stg, L0, lo, drow + W, false);
        } else {
            resolve_row<true, WORDS>(row, W, Wp, drow, P.rule, P.fmt, clr);
        }
        __syncwarp();
    }
    if (staged) stage_flush(stg, L0, lo, base + (size_t)H * d.stride, true);
}

// WORDS: the rasters are mapped host memory (Matte8 rows go out as aligned words).
template <bool WORDS>
__global__ void __launch_bounds__(BLOCK, 4) k_raster_warp(KParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpSmem& M = reinterpret_cast<WarpSmem*>(smem)[warp];
    unsigned char* scr = P.scratch + (size_t)blockIdx.x * SCRATCH_BYTES_PER_CTA + (size_t)warp * WS_BYTES;
    int2* pts = reinterpret_cast<int2*>(scr + WS_PTS);
    int* ss = reinterpret_cast<int*>(scr + WS_SS);
    int4* sorted = reinterpret_cast<int4*>(scr + WS_SORT);
    int4* active = reinterpret_cast<int4*>(scr + WS_ACT);
    for (;;) {
        int it = 0;
        if (lane == 0) it = (int)atomicAdd(&P.queue[1], 1u);
        it = __shfl_sync(FULL, it, 0);
        if (it >= (int)P.n_items_w) break;
        const WorkItem wi = P.items_w[it];
        const ft_path_desc d = P.paths[wi.path];
        const float sw0 = P.sw_chain ? *P.sw_chain : d.s_width;
        build_fill<WarpG>(P, d, sw0, M.u.B, nullptr, M.S, pts, ss, WARP_CAP);
        if (M.S.overflow) {
            // too many vertices for a warp: a CTA of the next kernel redoes this path
            if (lane == 0) P.overflow[atomicAdd(&P.queue[2], 1u)] = wi.path;
            __syncwarp();
            continue;
        }
        if (M.S.count > 0) {
            top_and_dir<WarpG>(M.S, pts, ss, M.tmp3);
            __syncwarp();
            const int nrows = (int)d.height - max(M.S.top_row, 0);
            if (nrows > 0 && d.width > 0) {
                for (int b = lane; b < nrows; b += 32) M.u.hist[b] = 0;  // the build's shared area is free
                __syncwarp();
                count_edges_warp(M.S, pts, ss, M.u.hist, nrows);
                __syncwarp();
                // the build's window is free during the sweep: its bytes after the
                // histogram stage the rows of a mapped host raster
                raster_sweep_warp<WORDS>(P, d, M.S, pts, ss, sorted, active, M.u.hist, M.row,
                                         reinterpret_cast<unsigned char*>(&M.u) + sizeof(M.u.hist));
            }
        }
        if (P.sw_out) {
            int lp = -1;
            for (int i = lane; i < (int)d.n_ops; i += 32)
                if (P.ops[d.op_begin + i].kind == FT_OP_PEN_WIDTH) lp = max(lp, i);
            lp = warp_incl_max(lp);
            if (lane == 31) P.sw_out[wi.path] = lp >= 0 ? P.ops[d.op_begin + lp].v[0] : sw0;
        }
        if (lane == 0 && M.S.flags) atomicMax(&P.status[wi.path], (M.S.flags & 1) ? FT_ERR_DEPTH : FT_ERR_ARG);
        __syncwarp();
    }
}

template <bool STROKE>
__global__ void __launch_bounds__(BLOCK) k_raster(KParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ CState S;
    __shared__ int s_item;
    __shared__ int s_tmp3[3 * NWARP];
    const int tid = threadIdx.x;
    unsigned char* scr = P.scratch + (size_t)blockIdx.x * SCRATCH_BYTES_PER_CTA;
    int2* pts = reinterpret_cast<int2*>(scr + SCR_PTS);
    int* ss = reinterpret_cast<int*>(scr + SCR_SS);
    EdgeRec* edges = reinterpret_cast<EdgeRec*>(scr + SCR_EDGES);
    float4* spts = reinterpret_cast<float4*>(scr + SCR_SPTS);
    SubRec* subs = reinterpret_cast<SubRec*>(scr + SCR_SUBS);
    // paths the warp rasteriser handed over (it ran before this kernel)
    const int n_over = P.overflow ? (int)*(volatile uint32_t*)&P.queue[2] : 0;
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(&P.queue[0], 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= (int)P.n_items + n_over) break;
        WorkItem wi;
        if (it < (int)P.n_items) {
            wi = P.items[it];
        } else {
            wi.path = P.overflow[it - (int)P.n_items];
            wi.row_begin = 0;
            wi.row_end = P.paths[wi.path].height;
            wi.band_rows = 0;
        }
        const ft_path_desc d = P.paths[wi.path];
        if (wi.band_rows == 0) {
            const int wp4 = (int)(((d.width + 3) & ~3u) * 4);
            wi.band_rows = (uint32_t)max(1, min((P.smem_bytes - RASTER_FIXED_SMEM) / max(wp4, 4), (int)d.height));
        }
        const float sw0 = P.sw_chain ? *P.sw_chain : d.s_width;
        BuildSmem& B = *reinterpret_cast<BuildSmem*>(smem);
        const size_t cs_off = (sizeof(BuildSmem) + 15) & ~(size_t)15;
        CompactSmem* Cs = reinterpret_cast<CompactSmem*>(smem + cs_off);
        if (STROKE) {
            // Plotter::stroke: stroke points, sub-strokes, outline, then the NonZero fill
            int* opi = reinterpret_cast<int*>(smem + cs_off + ((sizeof(CompactSmem) + 15) & ~(size_t)15));
            build_fill<BlockG, true>(P, d, sw0, B, Cs, S, pts, ss, PT_CAP, spts, subs, opi, raw_store(scr));
            finish_subs(P, d, S, subs, B.scan);
            build_outline(P, S, spts, subs, B, *Cs, pts, ss);
        } else {
            build_fill<BlockG>(P, d, sw0, B, Cs, S, pts, ss, PT_CAP, nullptr, nullptr, nullptr, raw_store(scr));
        }
        if (S.count > 0) {
            top_and_dir<BlockG>(S, pts, ss, s_tmp3);
            build_edges<BlockG>(S, pts, ss, edges);
            __syncthreads();
            const int row_begin = max(S.top_row, 0);
            const int lo = max((int)wi.row_begin, row_begin);
            const int hi = min((int)wi.row_end, (int)d.height);
            if (lo < hi && d.width > 0) raster_rows(P, d, S, edges, lo, hi, (int)wi.band_rows, smem);
        }
        // pen width after the call: the last PenWidth op of the path
        if (P.sw_out && wi.row_begin == 0) {
            int lp = -1;
            for (int i = tid; i < (int)d.n_ops; i += BLOCK)
                if (P.ops[d.op_begin + i].kind == FT_OP_PEN_WIDTH) lp = max(lp, i);
            lp = block_incl_max(lp, reinterpret_cast<BuildSmem*>(smem)->scan);
            if (tid == BLOCK - 1) P.sw_out[wi.path] = lp >= 0 ? P.ops[d.op_begin + lp].v[0] : sw0;
        }
        if (tid == 0 && S.flags) atomicMax(&P.status[wi.path], (S.flags & 1) ? FT_ERR_DEPTH : FT_ERR_ARG);
        __syncthreads();
    }
}

// Shared-memory carve-out (percent of the SM's unified L1) when a launch has at most
// one CTA per SM: the rest stays L1 for the curve walks' local-memory stacks.
constexpr int FEW_CTAS_CARVEOUT = 25;

cudaError_t launch_raster(const KParams& p, int grid, int smem_bytes, cudaStream_t s, bool few_ctas) {
    auto kern = p.stroke ? k_raster<true> : k_raster<false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                         few_ctas ? FEW_CTAS_CARVEOUT : (int)cudaSharedmemCarveoutDefault);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e != cudaSuccess) return e;
    kern<<<grid, BLOCK, smem_bytes, s>>>(p);
    return cudaGetLastError();
}

// The occupancy query honours the kernel's carve-out preference: a launch of at most one
// CTA per SM leaves FEW_CTAS_CARVEOUT set, under which the query would report one CTA per
// SM, the next grid would again be one CTA per SM and keep that carve-out for good.  The
// query is made with no preference; each launch then sets its own.
int raster_blocks_per_sm(int smem_bytes, bool stroke) {
    auto kern = stroke ? k_raster<true> : k_raster<false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutDefault);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, BLOCK, smem_bytes) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_raster_warp(const KParams& p, int grid, cudaStream_t s) {
    const int smem = raster_warp_smem();
    cudaError_t e = cudaFuncSetAttribute(p.host_rasters ? k_raster_warp<true> : k_raster_warp<false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    if (p.host_rasters)
        k_raster_warp<true><<<grid, BLOCK, smem, s>>>(p);
    else
        k_raster_warp<false><<<grid, BLOCK, smem, s>>>(p);
    return cudaGetLastError();
}

int raster_warp_smem() { return (int)(NWARP * sizeof(WarpSmem)); }

int raster_warp_blocks_per_sm() {
    const int smem = raster_warp_smem();
    cudaFuncSetAttribute(k_raster_warp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_raster_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster_warp<false>, BLOCK, smem) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

int raster_max_smem() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    int stat = 0;
    if (cudaFuncGetAttributes(&fa, k_raster<true>) == cudaSuccess) stat = (int)fa.sharedSizeBytes;
    return v - stat;
}

}  // namespace ftk

namespace ftk {

// ===========================================================================
// Ordered composite of many paths onto one raster: footile's repeated
// Plotter::fill / Plotter::stroke calls on one Plotter (plotter.rs:339-365).
//
// k_cbuild: one CTA per path builds its figure and edges as k_raster does, then
// bins the edges by raster band into a device pool.  k_cbands: one CTA per band
// walks the paths in call order; for each it accumulates the band's cell areas,
// resolves its rows and composites.  Every call of footile composites every pixel
// from its top row down, alpha 0 included, and SrcOver with alpha 0 maps each
// premultiplied channel d to ch8_mul(d, 255), which changes only d in 1..15 and
// is the identity after 15 applications.  So a band keeps, per row, the number of
// calls so far and, per pixel, the call count at its last covering call: a covered
// pixel first takes the pending alpha-0 maps from a 16-entry table of powers,
// uncovered pixels are not touched, and the band ends with one pending flush.

// Bin the built figure's edges by raster band into the pool (block-wide).
__device__ void bin_edges(const KParams& P, uint32_t path, const CState& S, const EdgeRec* edges, int* hist,
                          int* tmp) {
    const int tid = threadIdx.x;
    const int count = S.count, H = (int)P.canvas_h, R = P.band_rows, nb = P.n_bands;
    const int tmin = min(S.top_row, 0);
    const int rb = count > 0 ? max(S.top_row, 0) : H;  // first raster row footile writes
    for (int b = tid; b < nb; b += BLOCK) hist[b] = 0;
    __syncthreads();
    // several edges per thread per step, loaded before they are used (one CTA may bin
    // a whole figure alone: keep several L2 loads in flight); the count pass reads only
    // the half of each record with its rows (step_pix, ed, start_row, end_row)
    auto rows_of = [&](const int4& q, int& lo, int& hi) {
        lo = max(q.z - tmin, rb);
        hi = min(q.w - tmin, H - 1);
        return q.y != 0 && lo <= hi;
    };
    const int4* erec = reinterpret_cast<const int4*>(edges);
    constexpr int EU = 4;
    for (int e0 = 0; e0 < count; e0 += BLOCK * EU) {
        int4 q[EU];
#pragma unroll
        for (int u = 0; u < EU; u++) {
            const int e = e0 + u * BLOCK + tid;
            q[u] = e < count ? erec[2 * e + 1] : make_int4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < EU; u++) {
            int lo, hi;
            if (rows_of(q[u], lo, hi))
                for (int b = lo / R; b <= hi / R; b++) atomicAdd(&hist[b], 1);
        }
    }
    __syncthreads();
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += BLOCK) {
        const int b = b0 + tid;
        int tot;
        const int off = block_excl_sum(b < nb ? hist[b] : 0, tmp, tot);
        if (b < nb) hist[b] = carry + off;
        carry += tot;
    }
    __shared__ unsigned long long s_base;
    if (tid == 0) s_base = atomicAdd(P.pool_used, (unsigned long long)carry);
    __syncthreads();
    const unsigned long long base = s_base;
    const bool fits = base + (unsigned long long)carry <= P.pool_cap;
    // band offsets band-major (bandoff[b * n_items + path]): the compositors read 32 calls'
    // offsets of one band as one coalesced load
    for (int b = tid; b <= nb; b += BLOCK)
        P.bandoff[(size_t)b * P.n_items + path] = fits ? (b < nb ? hist[b] : carry) : 0;
    if (tid == 0) {
        P.crec[path] = make_int4(rb, tmin, (int)(unsigned)(base & 0xFFFFFFFFull), (int)(unsigned)(base >> 32));
        if (!fits) atomicMax(&P.status[path], FT_ERR_CAP);  // the host grows the pool and runs again
    }
    __syncthreads();
    if (fits) {
        constexpr int FU = 2;
        for (int e0 = 0; e0 < count; e0 += BLOCK * FU) {
            int4 q0[FU], q1[FU];
#pragma unroll
            for (int u = 0; u < FU; u++) {
                const int e = e0 + u * BLOCK + tid;
                q0[u] = e < count ? erec[2 * e] : make_int4(0, 0, 0, 0);
                q1[u] = e < count ? erec[2 * e + 1] : make_int4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < FU; u++) {
                int lo, hi;
                if (!rows_of(q1[u], lo, hi)) continue;
                for (int b = lo / R; b <= hi / R; b++) {
                    const unsigned long long k = base + (unsigned)atomicAdd(&hist[b], 1);
                    if (!ck(k < P.pool_cap, 11)) continue;
                    int4* dst = reinterpret_cast<int4*>(P.pool + k);
                    dst[0] = q0[u];
                    dst[1] = q1[u];
                }
            }
        }
    }
    __syncthreads();
}

// Four CTAs per SM (56 registers for strokes, no spills; 101 unbounded, two CTAs): the
// builds of an ordered composite are latency-bound chains of block scans.
template <bool STROKE>
__global__ void __launch_bounds__(BLOCK, 4) k_cbuild(KParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ CState S;
    __shared__ int s_item;
    __shared__ int s_tmp3[3 * NWARP];
    const int tid = threadIdx.x;
    const ScrLayout L = P.L;
    unsigned char* scr = P.scratch + (size_t)blockIdx.x * L.bytes;
    int2* pts = reinterpret_cast<int2*>(scr + L.pts);
    int* ss = reinterpret_cast<int*>(scr + L.ss);
    EdgeRec* edges = reinterpret_cast<EdgeRec*>(scr + L.edges);
    float4* spts = reinterpret_cast<float4*>(scr + L.spts);
    SubRec* subs = reinterpret_cast<SubRec*>(scr + L.subs);
    BuildSmem& B = *reinterpret_cast<BuildSmem*>(smem);
    const size_t cs_off = (sizeof(BuildSmem) + 15) & ~(size_t)15;
    CompactSmem* Cs = reinterpret_cast<CompactSmem*>(smem + cs_off);
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(&P.queue[0], 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= (int)P.n_items) break;
        const ft_path_desc d = P.paths[it];
        if (STROKE) {
            int* opi = reinterpret_cast<int*>(smem + cs_off + ((sizeof(CompactSmem) + 15) & ~(size_t)15));
            build_fill<BlockG, true>(P, d, d.s_width, B, Cs, S, pts, ss, PT_CAP, spts, subs, opi, raw_store(scr, L));
            finish_subs(P, d, S, subs, B.scan);
            build_outline(P, S, spts, subs, B, *Cs, pts, ss);
        } else {
            build_fill<BlockG>(P, d, d.s_width, B, Cs, S, pts, ss, P.pt_cap, nullptr, nullptr, nullptr,
                               raw_store(scr, L));
        }
        if (P.split_bin) {
            // the figure's edges are built and binned by launch_figure_bins
            if (S.count > 0) top_and_dir<BlockG>(S, pts, ss, s_tmp3);
            __syncthreads();
            if (tid == 0) P.fig_state[it] = make_int4(S.count, S.dir, S.top_row, 0);
        } else {
            if (S.count > 0) {
                top_and_dir<BlockG>(S, pts, ss, s_tmp3);
                build_edges<BlockG>(S, pts, ss, edges);
            }
            __syncthreads();
            bin_edges(P, (uint32_t)it, S, edges, reinterpret_cast<int*>(smem), s_tmp3);
        }
        if (P.sw_out) {  // pen width after the call: the last PenWidth op of the path
            int lp = -1;
            for (int i = tid; i < (int)d.n_ops; i += BLOCK)
                if (P.ops[d.op_begin + i].kind == FT_OP_PEN_WIDTH) lp = max(lp, i);
            lp = block_incl_max(lp, s_tmp3);
            if (tid == BLOCK - 1) P.sw_out[it] = lp >= 0 ? P.ops[d.op_begin + lp].v[0] : d.s_width;
        }
        if (tid == 0 && S.flags) atomicMax(&P.status[it], (S.flags & 1) ? FT_ERR_DEPTH : FT_ERR_ARG);
        __syncthreads();
    }
}

// The alpha-0 SrcOver of pix maps a premultiplied channel d to ch8_mul(d, 255), which
// leaves d >= 16 unchanged: ftab[k][d] (d < 16) is d after k such composites.
constexpr int FTAB_BYTES = 16 * 16;
__device__ __forceinline__ unsigned ftab4(const unsigned char* ftab, unsigned d, int k) {
    const unsigned char* t = ftab + (k << 4);
    unsigned out = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const unsigned c = (d >> (8 * i)) & 0xFFu;
        out |= (c < 16u ? (unsigned)t[c] : c) << (8 * i);
    }
    return out;
}

// Per-warp shared memory of the Matte8 band compositor for rows of `width` pixels: the
// row's i32 cell areas and its touched-span marks.
__host__ __device__ constexpr int row_smem_bytes(int width) {
    return (int)align256((size_t)((width + 3) & ~3) * 4 + (size_t)(((width + 127) / 128 + 31) / 32) * 4);
}

// Accumulate the cells of the `ne` band edges that cross scan row y into `row`
// (one warp; each lane takes edges), marking the touched 128-pixel spans.
__device__ __forceinline__ void row_items(const EdgeRec* edges, int ne, int y, int* row, int W, unsigned* spans) {
    const int lane = threadIdx.x & 31;
    for (int e = lane; e < ne; e += 32) {
        const EdgeRec E = edges[e];
        if (E.start_row <= y && y <= E.end_row) scan_item(E, y, row, W, spans);
    }
}

// Resolve one Matte8 row (imgbuf.rs:38-199) and overwrite every pixel of it
// (fig.rs:629-636).  Clears the row buffer and the span marks.
__device__ __forceinline__ void matte_row(int* row, unsigned* spans, int W, int Wp, uint8_t* drow, int rule) {
    const int lane = threadIdx.x & 31;
    unsigned carry = 0;
    for (int x0 = 0; x0 < W; x0 += 128) {
        const int x = x0 + lane * 4;
        int4 a = make_int4(0, 0, 0, 0);
        if (x < Wp) {
            a = *reinterpret_cast<const int4*>(row + x);
            *reinterpret_cast<int4*>(row + x) = make_int4(0, 0, 0, 0);
        }
        const unsigned s0 = (unsigned)a.x, s1 = s0 + (unsigned)a.y, s2 = s1 + (unsigned)a.z, s3 = s2 + (unsigned)a.w;
        const unsigned inc = warp_incl_sum_u(s3);
        const unsigned ex = inc - s3 + carry;
        carry += __shfl_sync(FULL, inc, 31);
        const unsigned av[4] = {resolve_cov(s0 + ex, rule), resolve_cov(s1 + ex, rule), resolve_cov(s2 + ex, rule),
                                resolve_cov(s3 + ex, rule)};
#pragma unroll
        for (int c = 0; c < 4; c++)
            if (x + c < W) drow[x + c] = (uint8_t)av[c];
    }
    __syncwarp();
    const int n_words = ((W + 127) / 128 + 31) / 32;
    for (int k = lane; k < n_words; k += 32) spans[k] = 0;
    __syncwarp();
}

// (edge, row) items of one band spread over a whole compositor CTA (a single call): the
// band's edges 256 at a time, each edge's rows in the band counted, a block scan and a
// run-length item map (as raster_rows).
struct BandStage {
    EdgeRec edges[BLOCK];
    int ya[BLOCK];
    int off[BLOCK];
    int scan[2 * NWARP + 2];
    unsigned char map[MAP_CAP];
};
constexpr int BAND_STAGE_BYTES = (int)((sizeof(BandStage) + 255) & ~(size_t)255);

// Matte8 ordered composite: every call overwrites its rows from its top row down
// (fig.rs:629-636), so a raster row shows only the last call that reaches it.  One CTA per
// band of P.band_rows rows, one warp per row: the warp finds that call and draws it.  A
// single call on bands of 8 rows spreads the band's (edge, row) items over the whole CTA
// (each edge read once, not once per row-warp).
__global__ void __launch_bounds__(BLOCK) k_cbands(KParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = (int)P.canvas_w, H = (int)P.canvas_h, Wp = (W + 3) & ~3;
    const int R = P.band_rows, b = blockIdx.x;
    const int r = b * R + warp;  // this warp's raster row
    const bool whole = P.n_items == 1 && R == NWARP && blockDim.x == BLOCK;
    if (!whole && (warp >= R || r >= H)) return;
    unsigned char* mine = smem + (size_t)warp * row_smem_bytes(W);
    int* row = reinterpret_cast<int*>(mine);
    unsigned* spans = reinterpret_cast<unsigned*>(row + Wp);
    const int n_words = ((W + 127) / 128 + 31) / 32;
    for (int x = lane * 4; x < Wp; x += 128) *reinterpret_cast<int4*>(row + x) = make_int4(0, 0, 0, 0);
    for (int k = lane; k < n_words; k += 32) spans[k] = 0;
    __syncwarp();
    uint8_t* drow = P.rasters + (size_t)r * P.canvas_stride;
    if (whole) {
        BandStage& Bs = *reinterpret_cast<BandStage*>(smem + (size_t)R * row_smem_bytes(W));
        const int4 cr = P.crec[0];
        const int rlo = max(b * R, cr.x), rhi = min(b * R + R, H);  // rows the call draws here
        if (rlo >= rhi) return;
        const int o0 = P.bandoff[b], o1 = P.bandoff[b + 1];
        const EdgeRec* edges =
            P.pool + ((unsigned long long)(unsigned)cr.z | ((unsigned long long)(unsigned)cr.w << 32)) + o0;
        const int ne = o1 - o0, yb0 = rlo + cr.y, yb1 = rhi + cr.y;  // scan rows yb0 .. yb1 - 1
        __syncthreads();  // every row buffer cleared
        for (int e0 = 0; e0 < ne; e0 += BLOCK) {
            const int e = e0 + threadIdx.x;
            int nrow = 0, ya = 0;
            EdgeRec E;
            E.ed = 0;
            if (e < ne) {
                E = edges[e];
                if (E.ed) {
                    ya = max(E.start_row, yb0);
                    nrow = max(min(E.end_row, yb1 - 1) - ya + 1, 0);
                }
            }
            Bs.edges[threadIdx.x] = E;
            Bs.ya[threadIdx.x] = ya;
            int tot;
            const int o = block_excl_sum(nrow, Bs.scan, tot);
            Bs.off[threadIdx.x] = o;
            for (int m0 = 0; m0 < tot; m0 += MAP_CAP) {
                const int ia = max(o, m0), ib = min(o + nrow, m0 + MAP_CAP);
                for (int k = ia; k < ib; k++) Bs.map[k - m0] = (unsigned char)threadIdx.x;
                __syncthreads();
                const int nm = min(MAP_CAP, tot - m0);
                for (int it = threadIdx.x; it < nm; it += BLOCK) {
                    const int jj = Bs.map[it];
                    const int y = Bs.ya[jj] + (m0 + it - Bs.off[jj]);
                    const int ri = y - cr.y - b * R;  // band row of scan row y
                    if (ck(ri >= 0 && ri < R, 15))
                        scan_item(Bs.edges[jj], y,
                                  reinterpret_cast<int*>(smem + (size_t)ri * row_smem_bytes(W)), W);
                }
                __syncthreads();
            }
        }
        if (r >= rlo && r < rhi) matte_row(row, spans, W, Wp, drow, P.rule);
        return;
    }
    const int n = (int)P.n_items;
    int found = -1;
    for (int c1 = n; c1 > 0 && found < 0; c1 -= 32) {
        const int i = c1 - 32 + lane;
        const bool hit = i >= 0 && P.crec[i].x <= r;
        const unsigned m = __ballot_sync(FULL, hit);
        if (m) found = c1 - 32 + 31 - __clz(m);
    }
    if (found < 0) return;
    const int4 cr = P.crec[found];
    const int o0 = P.bandoff[(size_t)b * n + found], o1 = P.bandoff[(size_t)(b + 1) * n + found];
    const unsigned long long first = ((unsigned long long)(unsigned)cr.z | ((unsigned long long)(unsigned)cr.w << 32)) + o0;
    row_items(P.pool + first, o1 - o0, r + cr.y, row, W, nullptr);
    __syncwarp();
    matte_row(row, spans, W, Wp, drow, P.rule);
}

// ===========================================================================
// Rgba8p ordered composite on tiles (ft_composite_batch, and single large calls).
//
// One CTA per tile of R band rows x `seg_w` pixels; one warp per tile row.  The tile's
// canvas pixels are staged in shared memory for the whole call sequence: loaded by TMA
// (cp.async.bulk.tensor.2d, boxes of at most 256 pixels x R rows, completion on an
// mbarrier) when the canvas allows a tensor map, stored back by TMA at the end.  Each
// warp walks the calls in order.  For a call, every band edge crossing the row gives its
// cells inside the segment (into a shared i32 segment row, atomics) and, from the closed
// form of the cell walk, the running sum it leaves to the left of the segment (the carry
// into the segment: the cumulative cell sum through column c of an (edge, row) item is
// min(pixel_cov(min(first + (c - minp) * step, ONE)), cov), fig.rs:285-321).  The row is
// then resolved sparsely: only the 8-pixel chunks that received cells are summed and
// resolved (32 at a time, one per lane, a warp scan placing them), and the untouched gap
// after each chunk holds that chunk's final running sum, so it is one run of a single
// alpha.  The covered pixels (alpha > 0) of the chunks and of the runs are composited
// with all lanes busy; the alpha-0 SrcOver footile applies to every other pixel from the
// call's top row down is applied lazily, as a pending count per pixel and a table of
// powers of the alpha-0 map (the map changes only channel values 1..15 and settles after
// 15 applications).

constexpr int CT_QN = 256 + 40;  // queued covered pixels of one round (32 chunks of 8) and its runs

struct CTileLayout {
    int tile, mbar, area, last, queue, bmap, bytes;
};
// Shared memory of a compositor CTA; `staged`: the canvas tile is held in shared memory.
__host__ __device__ inline CTileLayout ctile_layout(int R, int sw, bool staged) {
    CTileLayout L;
    int o = FTAB_BYTES;
    o = (o + 127) & ~127;
    L.tile = o;  // R x sw canvas pixels, [box][row][box width]
    if (staged) o += R * sw * 4;
    L.mbar = o;
    o += 16;
    L.area = o;  // per warp: sw i32 cell areas
    o += R * sw * 4;
    L.queue = o;  // per warp: CT_QN queued pixels (x << 8 | alpha) and runs
    o += R * CT_QN * 4;
    L.bmap = o;  // per warp: touched 8-pixel chunks (one bit each), then the chunk list (a byte each)
    o += R * (((sw / 8 + 31) / 32) * 4 + sw / 8);
    o = (o + 15) & ~15;
    L.last = o;  // per warp: sw u8, calls so far (mod 256) at each pixel's last cover
    o += R * sw;
    L.bytes = (o + 15) & ~15;
    return L;
}

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

// Wait on an mbarrier phase for at most about 0.2 s of GPU time (the global timer);
// false when it did not complete.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, unsigned parity) {
    const unsigned a = smem_u32(mbar);
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (int it = 0; it < (1 << 22); it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255) == 255) {
            unsigned long long t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            if (t - t0 > 200000000ull) break;
        }
    }
    return false;
}

// Cells of one (edge, row) item inside the segment [s0, s0 + sw) of a raster row of W
// pixels (fig.rs:238-321 restricted to the segment): the cells' growths go into `area`
// (segment cells), the cumulative sum the item leaves left of s0 into `carry`, and the
// 8-pixel chunks it touched into the bitmap `bmap`.  The other arguments are scan_row's.
__device__ __forceinline__ void seg_row(int x_bot, int inv, bool st, bool en, int fu, int fl, int step, int ed,
                                        int* area, int s0, int sw, int W, unsigned& carry, unsigned* bmap) {
    const int ccov = en ? pixel_cov(fl) : 256;
    const int cov = st ? ccov - pixel_cov(fu) : ccov;
    if (cov <= 0) return;
    const int s1 = min(s0 + sw, W);
    {
        // quick bounds: the item's x-range lies between x_bot and x_bot - inv (when that
        // does not wrap, neither do the exact ends below)
        const long long xa = (long long)x_bot - inv;
        if (xa == (long long)(int)xa) {
            const int lo = (int)(min((long long)x_bot, xa) >> 16), hi = (int)(max((long long)x_bot, xa) >> 16);
            if (lo >= s1) return;  // right of the segment: nothing here, nothing carried in
            // left of it, its walk complete before s0 (first + j * step >= ONE for every
            // cell left of the segment from any start <= hi): it leaves its whole coverage
            if (s0 - 1 - hi > 0 && (long long)(s0 - 1 - hi) * step >= FX_ONE) {
                carry += (unsigned)(ed * cov);
                return;
            }
        }
    }
    const int x0 = st ? wsub(x_bot, fxmul(inv, wsub(FX_ONE, fu))) : wsub(x_bot, inv);
    const int x1 = en ? wsub(x_bot, fxmul(inv, fl ? FX_ONE - fl : 0)) : x_bot;
    const int mnx = min(x0, x1), mxx = max(x0, x1);
    const int minp = mnx >> 16, maxp = mxx >> 16;
    if (minp >= W) return;
    if (minp >= s1) return;  // right of the segment: nothing here, nothing carried in
    const int full = cov << 8;
    const int r = (minp == maxp) ? fxmul(wsub(FX_ONE, fxfract(fxavg(mxx, mnx))), full)
                                 : fxmul(wsub(FX_ONE, fxfract(mnx)), FX_HALF);
    const int first = fxmul(r, step);
    int c = max(max(s0, minp), 0);
    int prev = 0;
    if (s0 > 0 && minp < s0) {
        // cumulative sum through cell s0 - 1: min(pixel_cov(min(first + j * step, ONE)), cov)
        const long long v = (long long)first + (long long)(s0 - 1 - minp) * step;
        prev = min(pixel_cov(v > FX_ONE ? FX_ONE : (int)v), cov);
        carry += (unsigned)(ed * prev);
    }
    if (prev >= cov) return;
    const long long xv = (long long)first + (long long)(c - minp) * step;
    int x_cov = xv > FX_ONE ? FX_ONE : (int)xv;
    int c_lo = -1, c_hi = -1;
    for (; c < s1; c++) {
        const int v = min(pixel_cov(x_cov), cov);
        if (v != prev) {
            if (ck(c - s0 >= 0 && c - s0 < sw, 6)) atomicAdd(&area[c - s0], ed * (v - prev));
            if (c_lo < 0) c_lo = c - s0;
            c_hi = c - s0;
        }
        prev = v;
        if (v >= cov) break;
        x_cov = min(x_cov + step, FX_ONE);
    }
    if (c_lo >= 0) {  // the touched chunks c_lo / 8 .. c_hi / 8
        const int k0 = c_lo >> 3, k1 = c_hi >> 3;
        for (int w = k0 >> 5; w <= (k1 >> 5); w++) {
            const int lo = max(k0 - 32 * w, 0), hi = min(k1 - 32 * w, 31);
            const unsigned m = (hi == 31 ? 0xFFFFFFFFu : ((1u << (hi + 1)) - 1u)) & ~((1u << lo) - 1u);
            if (ck(w < (sw / 8 + 31) / 32, 7)) atomicOr(&bmap[w], m);
        }
    }
}

__device__ __forceinline__ unsigned warp_sum_u(unsigned v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

template <bool STAGED>
__global__ void __launch_bounds__(BLOCK, 4) k_ctile(KParams P, const __grid_constant__ CUtensorMap tmap) {
    extern __shared__ __align__(128) unsigned char smem_tma[];  // TMA destinations: 128-byte aligned
    unsigned char* smem = smem_tma;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = (int)P.canvas_w, H = (int)P.canvas_h, R = P.band_rows, sw = P.seg_w;
    const int nseg = (W + sw - 1) / sw;
    const int b = (int)blockIdx.x / nseg, x0 = ((int)blockIdx.x % nseg) * sw;
    const int r = b * R + warp;
    const CTileLayout L = ctile_layout(R, sw, STAGED);
    const int BW = sw < 256 ? sw : 256;  // TMA box width (pixels)
    const int bw_shift = BW == 256 ? 8 : 7;
    const int nchunks = sw >> 3;             // 8-pixel chunks of the segment
    const int nwords = (nchunks + 31) >> 5;  // bitmap words
    unsigned char* ftab = smem;
    unsigned* tile = reinterpret_cast<unsigned*>(smem + L.tile);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + L.mbar);
    int* area = reinterpret_cast<int*>(smem + L.area) + warp * sw;
    unsigned* q = reinterpret_cast<unsigned*>(smem + L.queue) + warp * CT_QN;
    unsigned* bmap = reinterpret_cast<unsigned*>(smem + L.bmap + warp * (nwords * 4 + nchunks));
    unsigned char* clist = reinterpret_cast<unsigned char*>(bmap + nwords);
    unsigned char* last = smem + L.last + warp * sw;
    unsigned* crow = reinterpret_cast<unsigned*>(P.rasters + (size_t)r * P.canvas_stride) + x0;
    // the canvas pixel of this warp's row at segment position x: in the shared tile
    // (staged by TMA), or in place in global memory
    auto px = [&](int x) -> unsigned* {
        return STAGED ? tile + (((x >> bw_shift) * R + warp) << bw_shift) + (x & (BW - 1)) : crow + x;
    };
    const bool tma = STAGED;
    if (tma && threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tma && threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)),
                     "r"(R * sw * 4)
                     : "memory");
        for (int bx = 0; bx < sw / BW; bx++)
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
                "%3}], [%4];" ::"r"(smem_u32(tile + bx * R * BW)),
                "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(x0 + bx * BW), "r"(b * R), "r"(smem_u32(mbar))
                : "memory");
    }
    for (int i = threadIdx.x; i < FTAB_BYTES; i += blockDim.x) {
        unsigned v = (unsigned)(i & 15);
        for (int k = 0; k < (i >> 4); k++) v = ch8_mul(v, 255u);
        ftab[i] = (unsigned char)v;
    }
    for (int x = lane * 4; x < sw; x += 128) *reinterpret_cast<int4*>(area + x) = make_int4(0, 0, 0, 0);
    for (int x = lane; x < sw; x += 32) last[x] = 0;
    if (lane < nwords) bmap[lane] = 0u;
    bool ok = true;
    if (tma) ok = mbar_wait(mbar, 0);
    ok = __syncthreads_and(ok) != 0;
    if (!ok && threadIdx.x == 0) atomicMax(&P.status[0], FT_ERR_TIMEOUT);
    if (ok && r < H) {
        const int n = (int)P.n_items, rule = P.rule;
        const unsigned lt = (1u << lane) - 1u;
        const int xend = min(sw, W - x0);  // segment pixels on the canvas
        int G = 0;  // calls so far that reach this row
        for (int c0 = 0; c0 < n; c0 += 32) {
            // 32 calls' records at once, one per lane
            const int i = c0 + lane;
            const int4 cr = i < n ? P.crec[i] : make_int4(INT_MAX, 0, 0, 0);
            const bool reach = cr.x <= r;
            int o0 = 0, o1 = 0;
            if (i < n) {
                o0 = P.bandoff[(size_t)b * n + i];
                o1 = P.bandoff[(size_t)(b + 1) * n + i];
            }
            const unsigned rmask = __ballot_sync(FULL, reach);
            unsigned dmask = __ballot_sync(FULL, reach && o1 > o0);
            const unsigned long long my_first =
                ((unsigned long long)(unsigned)cr.z | ((unsigned long long)(unsigned)cr.w << 32)) + (unsigned)o0;
            unsigned my_clr = 0;
            if (reach && o1 > o0) {
                const ft_path_desc& d = P.paths[i];
                my_clr = (unsigned)d.clr[0] | ((unsigned)d.clr[1] << 8) | ((unsigned)d.clr[2] << 16) |
                         ((unsigned)d.clr[3] << 24);
            }
            while (dmask) {
                const int j = __ffs(dmask) - 1;
                dmask &= dmask - 1;
                const int Gj = G + __popc(rmask & ((1u << j) - 1u));
                const unsigned long long first = __shfl_sync(FULL, my_first, j);
                const int ne = __shfl_sync(FULL, o1 - o0, j);
                const int y = r + __shfl_sync(FULL, cr.y, j);
                const unsigned clr = __shfl_sync(FULL, my_clr, j);
                // cells of the band edges crossing scan row y, inside the segment
                unsigned carry = 0;
                const int4* E = reinterpret_cast<const int4*>(P.pool + first);
                for (int e = lane; e < ne; e += 32) {
                    const int4 hb = E[2 * e + 1];  // step_pix, ed, start_row, end_row
                    const int4 ha = E[2 * e];      // y_upper, y_lower, x_bot0, inv_slope
                    if (y < hb.z || y > hb.w) continue;
                    const int x_bot = wadd(ha.z, wmul(y - hb.z, ha.w));
                    seg_row(x_bot, ha.w, y == hb.z, y == hb.w, fxfract(ha.x), fxfract(ha.y), hb.x > 0 ? hb.x : FX_ONE,
                            hb.y, area, x0, sw, W, carry, bmap);
                }
                carry = warp_sum_u(carry);
                __syncwarp();
                // the touched chunks, in order
                int T = 0;
                for (int w = 0; w < nwords; w++) {
                    const unsigned bw = bmap[w];
                    if (((bw >> lane) & 1u) && ck(T + __popc(bw & lt) < nchunks, 8))
                        clist[T + __popc(bw & lt)] = (unsigned char)(32 * w + lane);
                    T += __popc(bw);
                }
                __syncwarp();
                if (lane < nwords) bmap[lane] = 0u;
                auto compose = [&](int x, unsigned av) {
                    if (!ck(x >= 0 && x < xend, 10)) return;
                    unsigned* p = px(x);
                    unsigned dv = *p;
                    const int kk = min((Gj - (int)last[x]) & 255, 15);
                    if (kk) dv = ftab4(ftab, dv, kk);
                    *p = srcover_rgba(dv, clr, av);
                    last[x] = (unsigned char)(Gj + 1);
                };
                // the run before the first touched chunk holds the carry
                {
                    const unsigned av0 = resolve_cov(carry, rule);
                    if (av0) {
                        const int end = min(T ? (int)clist[0] * 8 : sw, xend);
                        for (int x = lane; x < end; x += 32) compose(x, av0);
                    }
                }
                unsigned base = carry;
                for (int t0 = 0; t0 < T; t0 += 32) {
                    const int t = t0 + lane;
                    const bool valid = t < T;
                    const int ch = valid ? clist[t] : 0;
                    int4 a0 = make_int4(0, 0, 0, 0), a1 = a0;
                    if (valid) {
                        int4* ap = reinterpret_cast<int4*>(area + ch * 8);
                        a0 = ap[0];
                        a1 = ap[1];
                        ap[0] = make_int4(0, 0, 0, 0);
                        ap[1] = make_int4(0, 0, 0, 0);
                    }
                    const unsigned csum = (unsigned)a0.x + (unsigned)a0.y + (unsigned)a0.z + (unsigned)a0.w +
                                          (unsigned)a1.x + (unsigned)a1.y + (unsigned)a1.z + (unsigned)a1.w;
                    const unsigned inc = warp_incl_sum_u(csum);
                    unsigned run = base + inc - csum;
                    base += __shfl_sync(FULL, inc, 31);
                    const int av_v[8] = {(int)a0.x, (int)a0.y, (int)a0.z, (int)a0.w,
                                         (int)a1.x, (int)a1.y, (int)a1.z, (int)a1.w};
                    unsigned w0 = 0, w1 = 0;
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        run += (unsigned)av_v[k];
                        const unsigned v = (valid && ch * 8 + k < xend) ? resolve_cov(run, rule) : 0u;
                        if (k < 4)
                            w0 |= v << (8 * k);
                        else
                            w1 |= v << (8 * (k - 4));
                    }
                    // the gap after this chunk up to the next touched one holds `run`
                    const int nxt = t + 1 < T ? (int)clist[t + 1] : nchunks;
                    const unsigned gav = valid ? resolve_cov(run, rule) : 0u;
                    const int g0 = ch * 8 + 8, g1 = min(nxt * 8, xend);
                    const bool has_gap = gav && g0 < g1;
                    auto nzb = [](unsigned w) { return (((w & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | w) & 0x80808080u; };
                    const int cnt = __popc(nzb(w0)) + __popc(nzb(w1));
                    const unsigned cinc = warp_incl_sum_u((unsigned)cnt);
                    const int tot = (int)__shfl_sync(FULL, cinc, 31);
                    const unsigned gm = __ballot_sync(FULL, has_gap);
                    int pos = (int)(cinc - (unsigned)cnt);
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        const unsigned v = ((k < 4 ? w0 : w1) >> (8 * (k & 3))) & 0xFFu;
                        if (v && ck(pos < 256, 9)) q[pos++] = ((unsigned)(ch * 8 + k) << 8) | v;
                    }
                    if (has_gap) q[256 + __popc(gm & lt)] = ((unsigned)g0 << 19) | ((unsigned)(g1 - g0) << 8) | gav;
                    __syncwarp();
                    for (int k = lane; k < tot; k += 32) {
                        const unsigned e = q[k];
                        compose((int)(e >> 8), e & 255u);
                    }
                    for (unsigned m = gm; m; m &= m - 1) {  // the gap runs, all lanes on each
                        const unsigned e = q[256 + __popc(gm & ((1u << (__ffs(m) - 1)) - 1u))];
                        const int gs = (int)(e >> 19), gl = (int)((e >> 8) & 0x7FF);
                        for (int x = gs + lane; x < gs + gl; x += 32) compose(x, e & 255u);
                    }
                    __syncwarp();
                }
            }
            const int G0 = G;
            G += __popc(rmask);
            if ((G0 >> 6) != (G >> 6)) {
                // every 64 calls: pending counts of 15 or more saturate, so a pixel's stamp
                // moves up to 15 calls behind; the u8 differences then stay below 256
                __syncwarp();
                for (int x = lane; x < sw; x += 32)
                    if (((G - (int)last[x]) & 255) > 15) last[x] = (unsigned char)(G - 15);
                __syncwarp();
            }
        }
        // the alpha-0 composites still pending since each pixel's last cover
        __syncwarp();
        for (int x = lane; x < xend; x += 32) {
            const int kk = min((G - (int)last[x]) & 255, 15);
            if (kk) {
                unsigned* p = px(x);
                *p = ftab4(ftab, *p, kk);
            }
        }
    }
    if (tma) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (ok && threadIdx.x == 0) {
            for (int bx = 0; bx < sw / BW; bx++)
                asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                                 reinterpret_cast<uint64_t>(&tmap)),
                             "r"(x0 + bx * BW), "r"(b * R), "r"(smem_u32(tile + bx * R * BW))
                             : "memory");
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
    }
}

// ===========================================================================
// SrcOver of one call from its coverage mask (single large Rgba8p calls).
//
// footile's rasterize_row composites every pixel of the call's rows from its top row down
// with the row's coverage (fig.rs:637-643; alpha 0 where nothing covers).  With the
// call's Matte8 coverage already in a mask (the band compositor writes it), this pass
// streams the canvas and the mask through shared memory by TMA: per tile of 8 rows x
// 256 pixels, a 2-D tensor load of the canvas (u32 pixels) and of the mask (bytes)
// completing on the stage's mbarrier, SrcOver in place, a 2-D tensor store; three stages
// per CTA and six CTAs per SM keep loads, compute and stores in flight together (the
// fastest of 8 / 16 / 32-row tiles with 2 to 6 stages on the 4096x4096 scene).  A pixel with coverage 0
// takes the alpha-0 map, which changes only channel values 1..15: the common case of no
// such channel leaves the pixel as it is.

constexpr int SO_STAGES = 3;  // SO_ROWS x SO_COLS tiles: ft_kernels.cuh (the host's tensor-map boxes)
constexpr int SO_CANVAS_BYTES = SO_ROWS * SO_COLS * 4, SO_MASK_BYTES = SO_ROWS * SO_COLS;
constexpr int SO_STAGE_BYTES = SO_CANVAS_BYTES + SO_MASK_BYTES;
constexpr int SO_SMEM = SO_STAGES * SO_STAGE_BYTES + 128 + 1024;  // stages, mbarriers, colour table

// ch8_mul(d, b) of the four channels of d, b's 12-bit expansion (b << 4 | b >> 4) given
__device__ __forceinline__ unsigned ch8_mul4(unsigned d, unsigned bx) {
    unsigned out = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const unsigned dc = (d >> (8 * c)) & 0xFFu;
        out |= ((((dc << 4) | (dc >> 4)) * bx) >> 16) << (8 * c);
    }
    return out;
}

// Warps 0..7 composite; warp 8 moves the tiles (one lane issues every TMA operation):
// full[s] completes when stage s holds a loaded tile, done[s] when the eight compositing
// warps have finished it (each warp fences its shared-memory writes for the async proxy
// first), so no CTA-wide barrier sits in the loop.
constexpr int SO_CWARPS = 8;
constexpr int SO_THREADS = 32 * (SO_CWARPS + 1);

__global__ void __launch_bounds__(SO_THREADS, 6) k_srcover_mask(const __grid_constant__ CUtensorMap tm_canvas,
                                                                 const __grid_constant__ CUtensorMap tm_mask, int W,
                                                                 int H, int r0, unsigned clr, int32_t* status) {
    extern __shared__ __align__(128) unsigned char smem_tma[];  // TMA destinations: 128-byte aligned
    unsigned char* smem = smem_tma;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + SO_STAGES * SO_STAGE_BYTES);
    uint64_t* done = full + SO_STAGES;
    // src[a]: the colour's four channels times coverage a (pix's ch8_mul), packed; its
    // alpha byte is the SrcOver's source alpha
    unsigned* src = reinterpret_cast<unsigned*>(smem + SO_STAGES * SO_STAGE_BYTES + 128);
    for (int a = threadIdx.x; a < 256; a += SO_THREADS) src[a] = ch8_mul4(clr, ((unsigned)a << 4) | ((unsigned)a >> 4));
    const int tx = (W + SO_COLS - 1) / SO_COLS, ty = (H - r0 + SO_ROWS - 1) / SO_ROWS;
    const int ntiles = tx * ty;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t cmap = reinterpret_cast<uint64_t>(&tm_canvas), mmap = reinterpret_cast<uint64_t>(&tm_mask);
    auto canvas_s = [&](int st) { return reinterpret_cast<unsigned*>(smem + st * SO_STAGE_BYTES); };
    auto mask_s = [&](int st) { return smem + st * SO_STAGE_BYTES + SO_CANVAS_BYTES; };
    auto tile_x = [&](int t) { return (t % tx) * SO_COLS; };
    auto tile_y = [&](int t) { return r0 + (t / tx) * SO_ROWS; };
    if (threadIdx.x == 0) {
        for (int st = 0; st < SO_STAGES; st++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(full + st)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(done + st)), "r"(SO_CWARPS)
                         : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // this CTA's tiles: blockIdx.x, blockIdx.x + gridDim.x, ...
    const int mine = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    auto tile_of = [&](int k) { return (int)blockIdx.x + k * (int)gridDim.x; };
    if (warp == SO_CWARPS) {
        if (lane != 0) return;
        auto load = [&](int k, int st) {
            const int t = tile_of(k);
            const unsigned mb = smem_u32(full + st);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(SO_STAGE_BYTES)
                         : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
                "%3}], [%4];" ::"r"(smem_u32(canvas_s(st))),
                "l"(cmap), "r"(tile_x(t)), "r"(tile_y(t)), "r"(mb)
                : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
                "%3}], [%4];" ::"r"(smem_u32(mask_s(st))),
                "l"(mmap), "r"(tile_x(t)), "r"(tile_y(t)), "r"(mb)
                : "memory");
        };
        for (int k = 0; k < SO_STAGES && k < mine; k++) load(k, k);
        for (int k = 0; k < mine; k++) {
            const int st = k % SO_STAGES;
            if (!mbar_wait(done + st, (unsigned)((k / SO_STAGES) & 1))) {
                atomicMax(status, FT_ERR_TIMEOUT);
                break;
            }
            const int t = tile_of(k);
            asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(cmap),
                         "r"(tile_x(t)), "r"(tile_y(t)), "r"(smem_u32(canvas_s(st)))
                         : "memory");
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            // the stage of tile k - 1 is free once its store has read it: reload it
            if (k >= 1 && k - 1 + SO_STAGES < mine) {
                asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                load(k - 1 + SO_STAGES, (k - 1) % SO_STAGES);
            }
        }
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        return;
    }
    for (int k = 0; k < mine; k++) {
        const int st = k % SO_STAGES;
        if (!mbar_wait(full + st, (unsigned)((k / SO_STAGES) & 1))) {
            if (lane == 0) atomicMax(status, FT_ERR_TIMEOUT);
            break;
        }
        unsigned* cv = canvas_s(st);
        const unsigned* mk = reinterpret_cast<const unsigned*>(mask_s(st));
        // four pixels per step: one mask word, four canvas words
        for (int i = threadIdx.x; i < SO_ROWS * SO_COLS / 4; i += 32 * SO_CWARPS) {
            const unsigned m4 = mk[i];
            const uint4 d = reinterpret_cast<const uint4*>(cv)[i];
            unsigned dv[4] = {d.x, d.y, d.z, d.w};
            // alpha 0 changes only channels in 1..15 (nonzero bytes whose high nibble is zero)
            auto low = [](unsigned v) {
                const unsigned nz = (((v & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | v) & 0x80808080u;
                const unsigned hi = (((v & 0x70707070u) + 0x70707070u) | v) & 0x80808080u;
                return nz & ~hi;
            };
            if (!m4 && !(low(dv[0]) | low(dv[1]) | low(dv[2]) | low(dv[3]))) continue;  // four pixels unchanged
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const unsigned av = (m4 >> (8 * j)) & 0xFFu;
                const unsigned v = dv[j];
                if (!av && !low(v)) continue;
                // pix SrcOver: clr * a + d * (255 - clr_alpha * a), channel by channel; an opaque
                // source (inverse alpha 0) replaces the pixel
                const unsigned s4 = src[av];
                const unsigned inv = 255u - (s4 >> 24);
                dv[j] = inv ? __vaddus4(s4, ch8_mul4(v, (inv << 4) | (inv >> 4))) : s4;
            }
            reinterpret_cast<uint4*>(cv)[i] = make_uint4(dv[0], dv[1], dv[2], dv[3]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(done + st)) : "memory");
    }
}

cudaError_t launch_srcover_mask(const CUtensorMap& canvas, const CUtensorMap& mask, int W, int H, int r0,
                                unsigned clr, int32_t* status, int sm_count, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(k_srcover_mask, cudaFuncAttributeMaxDynamicSharedMemorySize, SO_SMEM);
    if (e != cudaSuccess) return e;
    const int ntiles = ((W + SO_COLS - 1) / SO_COLS) * ((H - r0 + SO_ROWS - 1) / SO_ROWS);
    if (ntiles <= 0) return cudaSuccess;
    const int grid = std::max(1, std::min(ntiles, 6 * sm_count));
    k_srcover_mask<<<grid, SO_THREADS, SO_SMEM, s>>>(canvas, mask, W, H, r0, clr, status);
    return cudaGetLastError();
}

int composite_tile_smem(int band_rows, int seg_w, bool staged) { return ctile_layout(band_rows, seg_w, staged).bytes; }

cudaError_t launch_composite_tiles(const KParams& p, const CUtensorMap& tmap, cudaStream_t s) {
    const bool staged = p.use_tma != 0;
    const int smem = composite_tile_smem(p.band_rows, p.seg_w, staged);
    auto kern = staged ? k_ctile<true> : k_ctile<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const int nseg = ((int)p.canvas_w + p.seg_w - 1) / p.seg_w;
    kern<<<p.n_bands * nseg, 32 * p.band_rows, smem, s>>>(p, tmap);
    return cudaGetLastError();
}

int composite_bands_smem(int band_rows, int width) { return band_rows * row_smem_bytes(width) + BAND_STAGE_BYTES; }

// ---- edges and band bins of one path's figure over the whole GPU (split_bin); the
//      figure was built by CTA 0 of k_cbuild.  Band rows follow bin_edges.
struct FigBins {
    int count, figdir, H, R, nb, tmin, rb;
};
__device__ __forceinline__ FigBins fig_bins(const KParams& P) {
    const int4 fs = P.fig_state[0];
    FigBins f;
    f.count = fs.x;
    f.figdir = fs.y;
    f.H = (int)P.canvas_h;
    f.R = P.band_rows;
    f.nb = P.n_bands;
    f.tmin = min(fs.z, 0);
    f.rb = f.count > 0 ? max(fs.z, 0) : f.H;
    return f;
}

// Bands counted in shared memory by each CTA of the edge binning (one global atomic per
// CTA and band instead of one per edge and band); more bands count in global memory.  In
// shared memory an edge adds +1 at its first band and -1 after its last (a difference
// array, two atomics per edge), and a prefix sum gives the counts.
constexpr int BIN_SMEM_BANDS = 8192;

// Counts of this CTA's edges per band: sh[0 .. nb] difference array -> counts in sh[0 .. nb).
__device__ void fig_bin_prefix(int* sh, int nb, int* tmp) {
    __syncthreads();
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += BLOCK) {
        const int b = b0 + threadIdx.x;
        int tot;
        const int v = b < nb ? sh[b] : 0;
        const int ex = block_excl_sum(v, tmp, tot);
        if (b < nb) sh[b] = carry + ex + v;
        carry += tot;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(BLOCK) k_fig_edges(KParams P) {
    extern __shared__ int sh_bins[];  // n_bands + 1 differences (when n_bands <= BIN_SMEM_BANDS)
    __shared__ int tmp[2 * NWARP + 2];
    const FigBins f = fig_bins(P);
    const bool local = f.nb <= BIN_SMEM_BANDS;
    const unsigned char* scr = P.scratch;
    const int2* pts = reinterpret_cast<const int2*>(scr + P.L.pts);
    const int* ss = reinterpret_cast<const int*>(scr + P.L.ss);
    EdgeRec* edges = reinterpret_cast<EdgeRec*>(P.scratch + P.L.edges);
    if (local) {
        for (int b = threadIdx.x; b <= f.nb; b += BLOCK) sh_bins[b] = 0;
        __syncthreads();
    }
    for (int e = blockIdx.x * BLOCK + threadIdx.x; e < f.count; e += gridDim.x * BLOCK) {
        const EdgeRec E = edge_rec(e, f.count, f.figdir, pts, ss);
        edges[e] = E;
        if (!E.ed) continue;
        const int lo = max(E.start_row - f.tmin, f.rb), hi = min(E.end_row - f.tmin, f.H - 1);
        if (lo > hi) continue;
        if (local) {
            atomicAdd(&sh_bins[lo / f.R], 1);
            atomicAdd(&sh_bins[hi / f.R + 1], -1);
        } else {
            for (int b = lo / f.R; b <= hi / f.R; b++) atomicAdd(&P.bin_hist[b], 1);
        }
    }
    if (local) {
        fig_bin_prefix(sh_bins, f.nb, tmp);
        for (int b = threadIdx.x; b < f.nb; b += BLOCK)
            if (sh_bins[b]) atomicAdd(&P.bin_hist[b], sh_bins[b]);
    }
}

__global__ void __launch_bounds__(BLOCK) k_fig_bin_scan(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    __shared__ unsigned long long s_base;
    const FigBins f = fig_bins(P);
    const int tid = threadIdx.x;
    int carry = 0;
    for (int b0 = 0; b0 < f.nb; b0 += BLOCK) {
        const int b = b0 + tid;
        int tot;
        const int off = block_excl_sum(b < f.nb ? P.bin_hist[b] : 0, tmp, tot);
        if (b < f.nb) P.bin_hist[f.nb + b] = carry + off;  // fill cursors
        carry += tot;
    }
    if (tid == 0) s_base = atomicAdd(P.pool_used, (unsigned long long)carry);
    __syncthreads();
    const unsigned long long base = s_base;
    const bool fits = base + (unsigned long long)carry <= P.pool_cap;
    for (int b = tid; b <= f.nb; b += BLOCK) P.bandoff[b] = fits ? (b < f.nb ? P.bin_hist[f.nb + b] : carry) : 0;
    if (tid == 0) {
        P.crec[0] = make_int4(f.rb, f.tmin, (int)(unsigned)(base & 0xFFFFFFFFull), (int)(unsigned)(base >> 32));
        P.fig_state[0].w = fits ? 1 : 0;
        if (!fits) atomicMax(&P.status[0], FT_ERR_CAP);  // the host grows the pool and runs again
    }
}

// (edge, band) pairs of 256 edges at a time spread over the CTA (run-length item map):
// an edge spanning many bands no longer holds one thread for all of them.
struct BinStage {
    int4 q[2 * BLOCK];  // the edges' two halves
    int b0[BLOCK];      // first band
    int off[BLOCK];
    int scan[2 * NWARP + 2];
    unsigned char map[MAP_CAP];
};

__global__ void __launch_bounds__(BLOCK) k_fig_bin_fill(KParams P) {
    // n_bands + 1 counts, then n_bands cursors (n_bands <= BIN_SMEM_BANDS), then the stage
    extern __shared__ __align__(16) int sh_bins[];
    const FigBins f = fig_bins(P);
    if (!P.fig_state[0].w) return;
    const bool local = f.nb <= BIN_SMEM_BANDS;
    const int4 cr = P.crec[0];
    const unsigned long long base = (unsigned long long)(unsigned)cr.z | ((unsigned long long)(unsigned)cr.w << 32);
    const int4* erec = reinterpret_cast<const int4*>(P.scratch + P.L.edges);
    int* cursor = P.bin_hist + f.nb;
    auto rows_of = [&](const int4& q1, int& lo, int& hi) {
        lo = max(q1.z - f.tmin, f.rb);
        hi = min(q1.w - f.tmin, f.H - 1);
        return q1.y != 0 && lo <= hi;
    };
    if (!local) {
        for (int e = blockIdx.x * BLOCK + threadIdx.x; e < f.count; e += gridDim.x * BLOCK) {
            const int4 q1 = erec[2 * e + 1];  // step_pix, ed, start_row, end_row
            int lo, hi;
            if (!rows_of(q1, lo, hi)) continue;
            const int4 q0 = erec[2 * e];
            for (int b = lo / f.R; b <= hi / f.R; b++) {
                const unsigned long long k = base + (unsigned)atomicAdd(&cursor[b], 1);
                if (!ck(k < P.pool_cap, 12)) continue;
                int4* dst = reinterpret_cast<int4*>(P.pool + k);
                dst[0] = q0;
                dst[1] = q1;
            }
        }
        return;
    }
    const int stage_at = (2 * f.nb + 1 + 3) & ~3;  // ints, 16-byte aligned
    BinStage& Bs = *reinterpret_cast<BinStage*>(sh_bins + stage_at);
    // this CTA's edges per band, then one run of slots per band taken from the cursors
    for (int b = threadIdx.x; b <= f.nb; b += BLOCK) sh_bins[b] = 0;
    __syncthreads();
    for (int e = blockIdx.x * BLOCK + threadIdx.x; e < f.count; e += gridDim.x * BLOCK) {
        int lo, hi;
        if (!rows_of(erec[2 * e + 1], lo, hi)) continue;
        atomicAdd(&sh_bins[lo / f.R], 1);
        atomicAdd(&sh_bins[hi / f.R + 1], -1);
    }
    fig_bin_prefix(sh_bins, f.nb, Bs.scan);
    for (int b = threadIdx.x; b < f.nb; b += BLOCK)
        sh_bins[f.nb + 1 + b] = sh_bins[b] ? atomicAdd(&cursor[b], sh_bins[b]) : 0;
    __syncthreads();
    int* lcur = sh_bins + f.nb + 1;
    for (int e0 = blockIdx.x * BLOCK; e0 < f.count; e0 += gridDim.x * BLOCK) {
        const int e = e0 + threadIdx.x;
        int n = 0, b0 = 0;
        int4 q0 = make_int4(0, 0, 0, 0), q1 = q0;
        if (e < f.count) {
            q1 = erec[2 * e + 1];
            int lo, hi;
            if (rows_of(q1, lo, hi)) {
                q0 = erec[2 * e];
                b0 = lo / f.R;
                n = hi / f.R - b0 + 1;
            }
        }
        Bs.q[2 * threadIdx.x] = q0;
        Bs.q[2 * threadIdx.x + 1] = q1;
        Bs.b0[threadIdx.x] = b0;
        int tot;
        const int o = block_excl_sum(n, Bs.scan, tot);
        Bs.off[threadIdx.x] = o;
        for (int m0 = 0; m0 < tot; m0 += MAP_CAP) {
            const int ia = max(o, m0), ib = min(o + n, m0 + MAP_CAP);
            for (int k = ia; k < ib; k++) Bs.map[k - m0] = (unsigned char)threadIdx.x;
            __syncthreads();
            const int nm = min(MAP_CAP, tot - m0);
            for (int it = threadIdx.x; it < nm; it += BLOCK) {
                const int jj = Bs.map[it];
                const int b = Bs.b0[jj] + (m0 + it - Bs.off[jj]);
                if (!ck(b >= 0 && b < f.nb, 12)) continue;
                const unsigned long long k = base + (unsigned)atomicAdd(&lcur[b], 1);
                if (!ck(k < P.pool_cap, 12)) continue;
                int4* dst = reinterpret_cast<int4*>(P.pool + k);
                dst[0] = Bs.q[2 * jj];
                dst[1] = Bs.q[2 * jj + 1];
            }
            __syncthreads();
        }
    }
}

cudaError_t launch_figure_bins(const KParams& p, int grid, cudaStream_t s) {
    const bool local = p.n_bands <= BIN_SMEM_BANDS;
    const int sm_e = local ? (p.n_bands + 1) * (int)sizeof(int) : 0;
    const int sm_f = local ? ((2 * p.n_bands + 1 + 3) & ~3) * (int)sizeof(int) + (int)sizeof(BinStage) : 0;
    cudaError_t e = cudaFuncSetAttribute(k_fig_bin_fill, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         ((2 * BIN_SMEM_BANDS + 1 + 3) & ~3) * (int)sizeof(int) + (int)sizeof(BinStage));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_fig_edges, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (BIN_SMEM_BANDS + 1) * (int)sizeof(int));
    if (e != cudaSuccess) return e;
    k_fig_edges<<<grid, BLOCK, sm_e, s>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_fig_bin_scan<<<1, BLOCK, 0, s>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_fig_bin_fill<<<grid, BLOCK, sm_f, s>>>(p);
    return cudaGetLastError();
}

// ---- grid-wide figure build of one fill path
//
// footile builds the figure sequentially (Fig::add_point / Fig::close, fig.rs:373-461):
// a raw vertex is kept when it starts a sub-figure or differs from the raw vertex before
// it, and a close event (a Move or a Close before the next vertex, and the close that
// Plotter::fill ends with, plotter.rs:347) pops the last vertex when it equals the
// sub-figure's first.  Each of these decisions is a function of the raw stream alone:
//   keep(k) = starts(k) or raw(k) != raw(k-1)
//   pop(k)  = (starts(k+1) or k is the last raw vertex) and raw(k) == raw(R(k)),
//             R(k) the last sub-figure start at or before k,
// and the vertex count when raw vertex l is reached (the pops before it applied) is the
// exclusive prefix sum pos(l) of keep - pop.  A kept vertex goes to position pos(k) with
// sub-figure start pos(R(k)), unless it is the last kept vertex of a sub-figure that pops
// (the next sub-figure's first vertex takes its position).  The cap (65,535, or
// ft_set_figure_cap's) is reached at the first l with pos(l) >= cap: raw vertices from l
// on are ignored, and the count is the cap less one when l starts no sub-figure and
// raw(l-1) equals its sub-figure's first vertex (the close after the cap, as seq_group
// takes it).  Without the cap the count is the sum of keep - pop over all raw vertices.
//
// pos(k) and pos(R(k)) come out of one scan under an associative combination of
// (s: sum of keep - pop, h: has a sub-figure start, r: pos of the last start relative
// to the range's beginning, mp: largest exclusive prefix in the range); mp finds the
// first tile that reaches the cap.  Kernels, in stream order (each scan is run by the
// last CTA of its kernel to finish):
//   k_gb_ops    per 256 ops: the last Move/Line/Quad/Cubic/Close op and the last PenWidth op
//   k_gb_count  every op's pen (the end point of the last such op before it) and raw
//               vertex count (the count walk, GB_LANES lanes per op); scan of the counts
//   k_gb_emit   every op's raw vertices at its offset (the emit walk); per tile of 1,024
//               raw vertices its last sub-figure start, scanned
//   k_gb_keep   keep, pop and R per raw vertex; tile aggregates, scanned
//   k_gb_write  positions, the cap, the vertex and sub-figure start writes
//   k_gb_top    the top vertex (min (y, x, id)), the direction, the figure state
struct PAgg {
    int s, h, r, mp;
};
constexpr int GB_NEG = -(1 << 30);  // mp of the empty range (sums stay within +-2^29)
static_assert(GB_RAW_MAX <= (1ll << 29), "position sums fit the aggregate");
__device__ __forceinline__ PAgg pa_id() { return PAgg{0, 0, 0, GB_NEG}; }
__device__ __forceinline__ PAgg pa_comb(const PAgg& a, const PAgg& b) {
    return PAgg{a.s + b.s, a.h | b.h, b.h ? a.s + b.r : a.r, max(a.mp, a.s + b.mp)};
}
// one raw vertex: keep - pop, and whether it starts a sub-figure
__device__ __forceinline__ PAgg pa_elem(int v, int starts) { return PAgg{v, starts, 0, 0}; }
__device__ __forceinline__ PAgg pa_shfl_up(const PAgg& a, int o) {
    return PAgg{__shfl_up_sync(FULL, a.s, o), __shfl_up_sync(FULL, a.h, o), __shfl_up_sync(FULL, a.r, o),
                __shfl_up_sync(FULL, a.mp, o)};
}
__device__ __forceinline__ PAgg pa_load(const int4* p) {
    const int4 x = __ldcg(p);
    return PAgg{x.x, x.y, x.z, x.w};
}
// Exclusive block scan under pa_comb; `total` receives the whole block's combination.
__device__ PAgg block_scan_pa(PAgg v, PAgg* wt, PAgg& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    PAgg inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const PAgg t = pa_shfl_up(inc, o);
        if (lane >= o) inc = pa_comb(t, inc);
    }
    PAgg ex = pa_shfl_up(inc, 1);
    if (lane == 0) ex = pa_id();
    if (lane == 31) wt[w] = inc;
    __syncthreads();
    PAgg base = pa_id(), all = pa_id();
    for (int k = 0; k < NWARP; k++) {
        if (k == w) base = all;
        all = pa_comb(all, wt[k]);
    }
    total = all;
    __syncthreads();
    return pa_comb(base, ex);
}
__device__ long long block_excl_sum_ll(long long v, long long* tmp, long long& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) tmp[w] = inc;
    __syncthreads();
    long long base = 0, all = 0;
    for (int k = 0; k < NWARP; k++) {
        if (k == w) base = all;
        all += tmp[k];
    }
    total = all;
    __syncthreads();
    return base + inc - v;
}

// True in the last CTA of the grid to get here (after every CTA's global writes).
__device__ bool gb_last_block(unsigned* ticket) {
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1 ? 1 : 0;
    __syncthreads();
    const bool last = s_last != 0;
    if (last) __threadfence();
    return last;
}

__device__ __forceinline__ ft_op gb_op(const ft_op* ops, int i) {
    const int4* src = reinterpret_cast<const int4*>(ops + i);
    const int4 q0 = __ldg(src), q1 = __ldg(src + 1);
    ft_op op;
    op.kind = q0.x;
    op.v[0] = __int_as_float(q0.y);
    op.v[1] = __int_as_float(q0.z);
    op.v[2] = __int_as_float(q0.w);
    op.v[3] = __int_as_float(q1.x);
    op.v[4] = __int_as_float(q1.y);
    op.v[5] = __int_as_float(q1.z);
    op.reserved = 0;
    return op;
}
// Pen after op j, a Move/Line/Quad/Cubic/Close (a Close puts it at the origin,
// plotter.rs:200-203), and j's kind; j < 0: the origin and kind -1.
__device__ __forceinline__ void gb_pen(const ft_op* ops, int j, float& x, float& y, int& kind) {
    x = 0.f;
    y = 0.f;
    kind = -1;
    if (j < 0) return;
    const ft_op op = gb_op(ops, j);
    kind = op.kind;
    if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
        x = op.v[0];
        y = op.v[1];
    } else if (kind == FT_OP_QUAD) {
        x = op.v[2];
        y = op.v[3];
    } else if (kind == FT_OP_CUBIC) {
        x = op.v[4];
        y = op.v[5];
    }
}
// Raw vertices of a Move/Line/Quad/Cubic op with the pen at (px, py), as build_fill
// flattens them for a fill, split over GB_LANES lanes: lane s takes the subtree of the
// curve's subdivision whose path from the root is the GB_D0 bits of s (left half 0, in
// the depth-first order of the walk); a leaf above that depth goes to the first lane of
// its range, a Move or Line to lane 0.  Each subtree is the walk's own arithmetic, so the
// lanes' leaves in lane order are the walk's leaves.  emit(k, vertex) for the lane's k-th
// leaf; returns the lane's leaf count.  flags: 1 depth cap reached, 2 non-finite control
// point.
template <class Emit>
__device__ int gb_walk(const KParams& P, const ft_op& op, int kind, float px, float py, int lane, int& flags,
                       Emit emit) {
    if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
        if (lane) return 0;
        const P2 A = xform(P.xf, p2(op.v[0], op.v[1]));
        emit(0, make_int2(f2fx(A.x), f2fx(A.y)));
        return 1;
    }
    P2 a = xform(P.xf, p2(px, py)), b = xform(P.xf, p2(op.v[0], op.v[1])), c = xform(P.xf, p2(op.v[2], op.v[3]));
    auto leaf = [&](int k, P2 q, float) { emit(k, make_int2(f2fx(q.x), f2fx(q.y))); };
    const float tol_sq = P.tol_sq;
    int dh = 0, n;
    if (kind == FT_OP_QUAD) {
        if (!pfinite(a) || !pfinite(b) || !pfinite(c)) {
            if (lane) return 0;
            flags |= 2;
            emit(0, make_int2(f2fx(c.x), f2fx(c.y)));
            return 1;
        }
        for (int d = 0; d < GB_D0; d++) {
            const P2 ab = pmid(a, b), bc = pmid(b, c), abbc = pmid(ab, bc), ac = pmid(a, c);
            const bool within = pdist_sq(abbc, ac) <= tol_sq;
            if (within || d >= FT_MAX_DEPTH) {
                if (lane & ((1 << (GB_D0 - d)) - 1)) return 0;
                if (!within) flags |= 1;
                emit(0, make_int2(f2fx(c.x), f2fx(c.y)));
                return 1;
            }
            if ((lane >> (GB_D0 - 1 - d)) & 1) {
                a = abbc;
                b = bc;
            } else {
                b = ab;
                c = abbc;
            }
        }
        n = quad_walk<false>(a, b, c, 0.f, 0.f, 0.f, tol_sq, 0, INT_MAX, &dh, leaf, GB_D0);
    } else {
        P2 e = xform(P.xf, p2(op.v[4], op.v[5]));
        if (!pfinite(a) || !pfinite(b) || !pfinite(c) || !pfinite(e)) {
            if (lane) return 0;
            flags |= 2;
            emit(0, make_int2(f2fx(e.x), f2fx(e.y)));
            return 1;
        }
        for (int d = 0; d < GB_D0; d++) {
            const P2 ab = pmid(a, b), bc = pmid(b, c), cd = pmid(c, e);
            const P2 abbc = pmid(ab, bc), bccd = pmid(bc, cd);
            const P2 pe = pmid(abbc, bccd), ad = pmid(a, e);
            const bool within = pdist_sq(pe, ad) <= tol_sq;
            if (within || d >= FT_MAX_DEPTH) {
                if (lane & ((1 << (GB_D0 - d)) - 1)) return 0;
                if (!within) flags |= 1;
                emit(0, make_int2(f2fx(e.x), f2fx(e.y)));
                return 1;
            }
            if ((lane >> (GB_D0 - 1 - d)) & 1) {
                a = pe;
                b = bccd;
                c = cd;
            } else {
                b = ab;
                c = abbc;
                e = pe;
            }
        }
        n = cubic_walk<false>(a, b, c, e, 0.f, 0.f, 0.f, 0.f, tol_sq, 0, INT_MAX, &dh, leaf, GB_D0);
    }
    if (dh) flags |= 1;
    return n;
}

__global__ void __launch_bounds__(BLOCK) k_gb_ops(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    __shared__ int s_tot[3];
    const GridBuildBufs& G = P.gb;
    const int tid = threadIdx.x, i = blockIdx.x * BLOCK + tid;
    const int kind = i < G.n_ops ? __ldg(&G.ops[i].kind) : -1;
    int mpc, lpc;
    block_max_scan((kind >= FT_OP_CLOSE && kind <= FT_OP_CUBIC) ? i : -1, tmp, mpc, lpc);
    const int mpw = block_incl_max(kind == FT_OP_PEN_WIDTH ? i : -1, tmp);
    const int mcm = block_incl_max((kind == FT_OP_CLOSE || kind == FT_OP_MOVE) ? i : -1, tmp);
    if (i < G.n_ops) {
        G.opi[i].x = lpc;  // the block's part; k_gb_count adds the blocks before
        G.opw[i] = mpw;
    }
    if (tid == BLOCK - 1) G.opa[blockIdx.x] = make_int4(mpc, mpw, mcm, 0);
    if (!gb_last_block(&G.done[0])) return;
    // exclusive max over the blocks, in place
    const int nb = (int)gridDim.x;
    int cpc = -1, cpw = -1, ccm = -1;
    for (int b0 = 0; b0 < nb; b0 += BLOCK) {
        const int b = b0 + tid;
        const int4 a = b < nb ? __ldcg(&G.opa[b]) : make_int4(-1, -1, -1, 0);
        int ipc, epc, ipw, epw, icm, ecm;
        block_max_scan(a.x, tmp, ipc, epc);
        if (tid == BLOCK - 1) s_tot[0] = ipc;
        block_max_scan(a.y, tmp, ipw, epw);
        if (tid == BLOCK - 1) s_tot[1] = ipw;
        block_max_scan(a.z, tmp, icm, ecm);
        if (tid == BLOCK - 1) s_tot[2] = icm;
        __syncthreads();
        if (b < nb) G.opa[b] = make_int4(max(cpc, epc), max(cpw, epw), max(ccm, ecm), 0);
        cpc = max(cpc, s_tot[0]);
        cpw = max(cpw, s_tot[1]);
        ccm = max(ccm, s_tot[2]);
        __syncthreads();
    }
    if (tid == 0) {
        // pen width after the call: the last PenWidth op of the path
        if (P.sw_out) P.sw_out[0] = cpw >= 0 ? G.ops[cpw].v[0] : G.s_width;
        if (P.gs.st) {
            P.gs.st[3] = cpc;
            P.gs.st[4] = ccm;
        }
    }
}

// Op i of a CTA of k_gb_count / k_gb_emit (GB_OPB ops, GB_LANES lanes each) and its pen.
struct GbOp {
    int i, lane, kind, lpc, rs;
    float px, py;
    ft_op op;
};
__device__ __forceinline__ GbOp gb_op_of(const GridBuildBufs& G, int& flags) {
    GbOp o;
    o.i = blockIdx.x * GB_OPB + (int)(threadIdx.x / GB_LANES);
    o.lane = (int)(threadIdx.x % GB_LANES);
    o.kind = -1;
    o.lpc = -1;
    o.rs = 0;
    o.px = o.py = 0.f;
    if (o.i >= G.n_ops) return o;
    o.op = gb_op(G.ops, o.i);
    o.kind = o.op.kind;
    if (o.kind < -1 || o.kind > FT_OP_PEN_WIDTH) {
        if (o.lane == 0) flags |= 2;
        o.kind = -1;
    }
    o.lpc = max(G.opi[o.i].x, G.opa[o.i / BLOCK].x);
    int pk = -1;
    if (o.kind >= FT_OP_MOVE && o.kind <= FT_OP_CUBIC) gb_pen(G.ops, o.lpc, o.px, o.py, pk);
    // the first vertex of this op starts a sub-figure after a close event
    o.rs = o.kind == FT_OP_MOVE || pk == FT_OP_CLOSE || pk == -1;
    return o;
}

__global__ void __launch_bounds__(BLOCK) k_gb_count(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    __shared__ long long ltmp[NWARP];
    const GridBuildBufs& G = P.gb;
    if (G.skip && *G.skip) return;  // a probe over a prefix of the ops completed the figure
    const int tid = threadIdx.x;
    int flags = 0;
    const GbOp o = gb_op_of(G, flags);
    int n = 0;
    if (o.kind >= FT_OP_MOVE && o.kind <= FT_OP_CUBIC)
        n = gb_walk(P, o.op, o.kind, o.px, o.py, o.lane, flags, [](int, int2) {});
    if (flags) atomicMax(&P.status[0], (flags & 1) ? FT_ERR_DEPTH : FT_ERR_ARG);
    // the lanes' offsets within the op, the ops' offsets within the CTA
    int inc = n;
#pragma unroll
    for (int d = 1; d < GB_LANES; d <<= 1) {
        const int t = __shfl_up_sync(FULL, inc, d, GB_LANES);
        if (o.lane >= d) inc += t;
    }
    const int n_op = __shfl_sync(FULL, inc, GB_LANES - 1, GB_LANES);
    int tot;
    const int ex = block_excl_sum(o.lane == 0 ? n_op : 0, tmp, tot);
    if (o.i < G.n_ops) {
        G.opl[o.i * GB_LANES + o.lane] = inc - n;
        if (o.lane == 0) G.opi[o.i].y = ex;
    }
    if (tid == 0) G.opn[blockIdx.x] = tot;
    if (!gb_last_block(&G.done[1])) return;
    // exclusive sum over the CTAs, in place; the total is the path's raw vertex count
    const int nb = (int)gridDim.x;
    long long carry = 0;
    for (int b0 = 0; b0 < nb; b0 += BLOCK) {
        const int b = b0 + tid;
        long long t;
        const long long e = block_excl_sum_ll(b < nb ? __ldcg(&G.opn[b]) : 0ll, ltmp, t);
        if (b < nb) G.opn[b] = carry + e;
        carry += t;
    }
    if (tid == 0) *G.n_raw = carry;
}

// Exclusive max of the tiles' last sub-figure starts, in place (one CTA).
__device__ void gb_scan_tr(const GridBuildBufs& G, long long n_raw, int* tmp, int& s_c) {
    const int tid = threadIdx.x, nt = (int)((n_raw + GB_TILE - 1) / GB_TILE);
    int carry = -1;
    for (int b0 = 0; b0 < nt; b0 += BLOCK) {
        const int b = b0 + tid;
        int inc, exc;
        block_max_scan(b < nt ? __ldcg(&G.tr[b]) : -1, tmp, inc, exc);
        if (tid == BLOCK - 1) s_c = inc;
        __syncthreads();
        if (b < nt) G.tr[b] = max(carry, exc);
        carry = max(carry, s_c);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(BLOCK) k_gb_emit(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    __shared__ int s_c;
    const GridBuildBufs& G = P.gb;
    if (G.skip && *G.skip) return;  // a probe over a prefix of the ops completed the figure
    const long long n_raw = *G.n_raw;
    if (n_raw > G.raw_cap) return;  // every CTA: the caller grows the arrays
    int flags = 0;
    const GbOp o = gb_op_of(G, flags);
    if (o.kind >= FT_OP_MOVE && o.kind <= FT_OP_CUBIC) {
        const long long off0 = G.opn[blockIdx.x] + G.opi[o.i].y;
        const int off = (int)(off0 + G.opl[o.i * GB_LANES + o.lane]);
        int2* raw = G.raw;
        unsigned char* fl = G.fl;
        const int cap = G.raw_cap;
        const unsigned char rs0 = (o.lane == 0 && o.rs) ? 1 : 0;
        gb_walk(P, o.op, o.kind, o.px, o.py, o.lane, flags, [&](int k, int2 q) {
            if (ck(off + k < cap, 13) && off + k < cap) {
                raw[off + k] = q;
                fl[off + k] = k == 0 ? rs0 : (unsigned char)0;
            }
        });
        if (rs0 && ck(off < cap, 13) && off < cap) atomicMax(&G.tr[off / GB_TILE], off);
    }
    if (!gb_last_block(&G.done[2])) return;
    gb_scan_tr(G, n_raw, tmp, s_c);
}

__global__ void __launch_bounds__(BLOCK) k_gb_keep(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    __shared__ PAgg wt[NWARP];
    const GridBuildBufs& G = P.gb;
    if (G.skip && *G.skip) return;  // a probe over a prefix of the ops completed the figure
    const long long n_raw = *G.n_raw;
    if (n_raw > G.raw_cap) return;
    const int M = (int)n_raw, nt = (M + GB_TILE - 1) / GB_TILE, tid = threadIdx.x;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const int k0 = t * GB_TILE + GB_PER * tid;
        int2 p[GB_PER];
        int rl[GB_PER];
        int st = 0, run = -1;
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            const int k = k0 + j;
            p[j] = make_int2(0, 0);
            if (k < M) {
                p[j] = G.raw[k];
                if (G.fl[k] & 1) {
                    st |= 1 << j;
                    run = k;
                }
            }
            rl[j] = run;
        }
        int inc, exc;
        block_max_scan(run, tmp, inc, exc);
        const int carry = max(G.tr[t], exc);
        int2 q = (k0 > 0 && k0 <= M) ? G.raw[k0 - 1] : make_int2(0, 0);  // raw predecessor
        PAgg a = pa_id();
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            const int k = k0 + j;
            if (k < M) {
                const int R = max(0, max(carry, rl[j]));  // raw vertex 0 always starts one
                const int2 f = G.raw[R];
                const int s = (st >> j) & 1;
                const bool keep = s || p[j].x != q.x || p[j].y != q.y;
                const bool ends = k + 1 >= M || (G.fl[k + 1] & 1);
                const bool pop = ends && p[j].x == f.x && p[j].y == f.y;
                G.kp[k] = (unsigned char)((keep ? 1 : 0) | (pop ? 2 : 0));
                G.rk[k] = R;
                a = pa_comb(a, pa_elem((keep ? 1 : 0) - (pop ? 1 : 0), s));
            }
            q = p[j];
        }
        PAgg tot;
        block_scan_pa(a, wt, tot);
        if (tid == 0) G.tp[t] = make_int4(tot.s, tot.h, tot.r, tot.mp);
    }
    if (!gb_last_block(&G.done[3])) return;
    // exclusive scan of the tiles, in place, GB_PER tiles a thread; the total is the
    // vertex count when the cap is not reached
    PAgg carry = pa_id();
    for (int b0 = 0; b0 < nt; b0 += GB_TILE) {
        const int b = b0 + GB_PER * tid;
        PAgg v[GB_PER], a = pa_id();
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            v[j] = b + j < nt ? pa_load(&G.tp[b + j]) : pa_id();
            a = pa_comb(a, v[j]);
        }
        PAgg tot;
        PAgg ex = pa_comb(carry, block_scan_pa(a, wt, tot));
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            if (b + j < nt) G.tp[b + j] = make_int4(ex.s, ex.h, ex.r, ex.mp);
            ex = pa_comb(ex, v[j]);
        }
        carry = pa_comb(carry, tot);
    }
    if (tid == 0) *G.count = carry.s;
}

__global__ void __launch_bounds__(BLOCK) k_gb_write(KParams P) {
    __shared__ PAgg wt[NWARP];
    __shared__ int s_l;
    const GridBuildBufs& G = P.gb;
    if (G.skip && *G.skip) return;  // a probe over a prefix of the ops completed the figure
    const long long n_raw = *G.n_raw;
    if (n_raw > G.raw_cap) return;
    const int M = (int)n_raw, nt = (M + GB_TILE - 1) / GB_TILE, tid = threadIdx.x, cap = P.pt_cap;
    int2* pts = reinterpret_cast<int2*>(P.scratch + P.L.pts);
    int* ss = reinterpret_cast<int*>(P.scratch + P.L.ss);
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const PAgg C = pa_load(&G.tp[t]);
        if (C.mp >= cap) continue;  // the cap was reached before this tile
        const int k0 = t * GB_TILE + GB_PER * tid;
        int kp[GB_PER], st[GB_PER];
        PAgg a = pa_id();
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            const int k = k0 + j;
            kp[j] = 0;
            st[j] = 0;
            if (k < M) {
                kp[j] = G.kp[k];
                st[j] = G.fl[k] & 1;
                a = pa_comb(a, pa_elem((kp[j] & 1) - ((kp[j] >> 1) & 1), st[j]));
            }
        }
        if (tid == 0) s_l = INT_MAX;
        PAgg tot;
        PAgg run = pa_comb(C, block_scan_pa(a, wt, tot));
        int pos[GB_PER], posr[GB_PER], lc = INT_MAX;
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            const int k = k0 + j;
            pos[j] = run.s;
            if (k < M) {
                if (run.s >= cap) lc = min(lc, k);
                run = pa_comb(run, pa_elem((kp[j] & 1) - ((kp[j] >> 1) & 1), st[j]));
            }
            posr[j] = run.r;
        }
        if (lc != INT_MAX) atomicMin(&s_l, lc);
        __syncthreads();
        const int l = s_l;  // first raw vertex at the cap, INT_MAX: not in this tile
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            const int k = k0 + j;
            if (k >= M || k >= l || !(kp[j] & 1)) continue;
            const int2 v = G.raw[k], f = G.raw[G.rk[k]];
            bool gone = false;
            if (v.x == f.x && v.y == f.y) {
                // the last kept vertex of a sub-figure that pops: the next kept vertex
                // starts a sub-figure (or there is none)
                int m = k + 1;
                while (m < M && !(G.kp[m] & 1)) m++;
                gone = m >= M || (G.fl[m] & 1);
            }
            if (!gone && ck(pos[j] >= 0 && pos[j] < cap, 14) && pos[j] >= 0 && pos[j] < cap) {
                pts[pos[j]] = v;
                ss[pos[j]] = posr[j];
            }
        }
        if (l != INT_MAX && l >= k0 && l < k0 + GB_PER) {
            // the close after the cap pops the last vertex if it equals its sub-figure's first
            const int2 v = G.raw[l - 1], f = G.raw[G.rk[l - 1]];
            *G.count = cap - ((!(G.fl[l] & 1) && v.x == f.x && v.y == f.y) ? 1 : 0);
            if (G.final_flag) *G.final_flag = 1;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(BLOCK) k_gb_top(KParams P) {
    __shared__ int4 wb[NWARP];
    const GridBuildBufs& G = P.gb;
    if (G.skip && *G.skip) return;  // a probe over a prefix of the ops completed the figure
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int count = *G.n_raw > G.raw_cap ? 0 : *G.count;
    const int2* pts = reinterpret_cast<const int2*>(P.scratch + P.L.pts);
    const int* ss = reinterpret_cast<const int*>(P.scratch + P.L.ss);
    int by = INT_MAX, bx = INT_MAX, bi = INT_MAX;
    for (int i = blockIdx.x * BLOCK + tid; i < count; i += gridDim.x * BLOCK) {
        const int2 p = pts[i];
        if (top_less(p.y, p.x, i, by, bx, bi)) {
            by = p.y;
            bx = p.x;
            bi = i;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int oy = __shfl_down_sync(FULL, by, o), ox = __shfl_down_sync(FULL, bx, o),
                  oi = __shfl_down_sync(FULL, bi, o);
        if (top_less(oy, ox, oi, by, bx, bi)) {
            by = oy;
            bx = ox;
            bi = oi;
        }
    }
    if (lane == 0) wb[w] = make_int4(by, bx, bi, 0);
    __syncthreads();
    if (tid == 0) {
        int4 b = wb[0];
        for (int k = 1; k < NWARP; k++)
            if (top_less(wb[k].x, wb[k].y, wb[k].z, b.x, b.y, b.z)) b = wb[k];
        G.top[blockIdx.x] = b;
    }
    if (!gb_last_block(&G.done[4])) return;
    by = bx = bi = INT_MAX;
    for (int k = tid; k < (int)gridDim.x; k += BLOCK) {
        const int4 o = __ldcg(&G.top[k]);
        if (top_less(o.x, o.y, o.z, by, bx, bi)) {
            by = o.x;
            bx = o.y;
            bi = o.z;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int oy = __shfl_down_sync(FULL, by, o), ox = __shfl_down_sync(FULL, bx, o),
                  oi = __shfl_down_sync(FULL, bi, o);
        if (top_less(oy, ox, oi, by, bx, bi)) {
            by = oy;
            bx = ox;
            bi = oi;
        }
    }
    __syncthreads();
    if (lane == 0) wb[w] = make_int4(by, bx, bi, 0);
    __syncthreads();
    if (tid == 0) {
        int4 b = wb[0];
        for (int k = 1; k < NWARP; k++)
            if (top_less(wb[k].x, wb[k].y, wb[k].z, b.x, b.y, b.z)) b = wb[k];
        P.fig_state[0] = count > 0 ? make_int4(count, fig_dir(b.z, count, pts, ss), b.x >> 16, 0)
                                   : make_int4(0, 0, 0, 0);
    }
}

cudaError_t launch_grid_build(const KParams& p, int sm_count, cudaStream_t s, const KParams* probe) {
    const int nbo = (p.gb.n_ops + BLOCK - 1) / BLOCK;
    if (nbo <= 0 || p.gb.raw_cap % GB_TILE || p.gb.raw_cap > GB_RAW_MAX) return cudaErrorInvalidValue;
    if (probe && (probe->gb.n_ops <= 0 || probe->gb.n_ops > p.gb.n_ops)) return cudaErrorInvalidValue;
    const int gt = std::max(1, 4 * sm_count);
    k_gb_ops<<<nbo, BLOCK, 0, s>>>(p);  // pens of every op (the probe's too) and the pen width after
    for (const KParams* q : {probe, &p}) {
        if (!q) continue;
        const int nbw = (q->gb.n_ops + GB_OPB - 1) / GB_OPB;
        k_gb_count<<<nbw, BLOCK, 0, s>>>(*q);
        k_gb_emit<<<nbw, BLOCK, 0, s>>>(*q);
        k_gb_keep<<<gt, BLOCK, 0, s>>>(*q);
        k_gb_write<<<gt, BLOCK, 0, s>>>(*q);
        k_gb_top<<<GB_TOP_BLOCKS, BLOCK, 0, s>>>(*q);
    }
    return cudaGetLastError();
}

// ---- grid-wide build of one stroke path
//
// Plotter::stroke (plotter.rs:356-365) collects the stroke points (Stroke::add_point and
// close, stroker.rs:204-236), makes every sub-stroke's outline (stroker.rs:239-416) and
// fills it NonZero.  Over the whole GPU, in stream order:
//   k_gb_ops    pens, the last PenWidth op at or before each op, the last Close/Move op
//   k_gs_count  every op's raw stroke points (the walk carrying widths, GB_LANES lanes
//               per op), scanned
//   k_gs_emit   the raw points (x, y, width), whether each starts a sub-stroke, its op
//   k_gs_keep   per raw point: kept when it starts a sub-stroke or its f32 position
//               differs from the raw point before it (no closing point is popped); per
//               tile the kept points and sub-stroke starts, scanned
//   k_gs_write  a kept point's position is the kept points before it and its sub-stroke
//               the starts before it; points from 65,535 on are dropped and start
//               nothing; a start sets its sub-stroke's first point and the joined flag the
//               close events before it leave on the sub-stroke before
//   k_gs_subs   per sub-stroke: its points, the last one's joined flag (the last Close or
//               Move op after its last point when the cap stopped the points, else the
//               path's last Move/Line/Quad/Cubic/Close op), SubStroke::len in u16
//               arithmetic and 2 len + 2 outline items, scanned
//   k_go_count  every outline item's points (outline_item), scanned
//   k_go_emit   the outline's raw vertices through the second transform (plotter.rs:
//               219-224), the figure runs' starts per tile, scanned
// then k_gb_keep, k_gb_write and k_gb_top build the outline's figure as they do a fill's.

// width in effect at op j: its path's last PenWidth op at or before it, else the width
// the path starts with
__device__ __forceinline__ float gs_width(const GridBuildBufs& G, int j) {
    if (j < 0) return G.s_width;
    const int lpw = max(G.opw[j], G.opa[j / BLOCK].y);
    return lpw >= 0 ? __ldg(&G.ops[lpw].v[0]) : G.s_width;
}

// Raw stroke points of a Move/Line/Quad/Cubic op with the pen at (px, py) and widths
// pen_w (at the pen) and sw (at the op), as build_fill's STROKE walk makes them
// (plotter.rs:233-236, 294-298), split over GB_LANES lanes as gb_walk splits a fill's:
// emit(k, point, width) for the lane's k-th leaf; returns the lane's leaf count.
template <class Emit>
__device__ int gs_walk(const KParams& P, const ft_op& op, int kind, float px, float py, float pen_w, float sw,
                       int lane, int& flags, Emit emit) {
    if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
        if (lane) return 0;
        emit(0, xform(P.xf, p2(op.v[0], op.v[1])), sw);
        return 1;
    }
    P2 a = xform(P.xf, p2(px, py)), b = xform(P.xf, p2(op.v[0], op.v[1])), c = xform(P.xf, p2(op.v[2], op.v[3]));
    const float tol_sq = P.tol_sq;
    int dh = 0, n;
    if (kind == FT_OP_QUAD) {
        float wa = pen_w, wb = __fmul_rn(__fadd_rn(pen_w, sw), 0.5f), wc = sw;
        if (!pfinite(a) || !pfinite(b) || !pfinite(c)) {
            if (lane) return 0;
            flags |= 2;
            emit(0, c, wc);
            return 1;
        }
        for (int d = 0; d < GB_D0; d++) {
            const P2 ab = pmid(a, b), bc = pmid(b, c), abbc = pmid(ab, bc), ac = pmid(a, c);
            const bool within = pdist_sq(abbc, ac) <= tol_sq;
            if (within || d >= FT_MAX_DEPTH) {
                if (lane & ((1 << (GB_D0 - d)) - 1)) return 0;
                if (!within) flags |= 1;
                emit(0, c, wc);
                return 1;
            }
            const float wab = fmid(wa, wb), wbc = fmid(wb, wc), wabbc = fmid(wab, wbc);
            if ((lane >> (GB_D0 - 1 - d)) & 1) {
                a = abbc;
                b = bc;
                wa = wabbc;
                wb = wbc;
            } else {
                b = ab;
                c = abbc;
                wb = wab;
                wc = wabbc;
            }
        }
        n = quad_walk<true>(a, b, c, wa, wb, wc, tol_sq, 0, INT_MAX, &dh, emit, GB_D0);
    } else {
        P2 e = xform(P.xf, p2(op.v[4], op.v[5]));
        float wa = pen_w, wb = __fadd_rn(sw, __fmul_rn(__fsub_rn(pen_w, sw), 1.0f / 3.0f)),
              wc = __fadd_rn(sw, __fmul_rn(__fsub_rn(pen_w, sw), 2.0f / 3.0f)), we = sw;
        if (!pfinite(a) || !pfinite(b) || !pfinite(c) || !pfinite(e)) {
            if (lane) return 0;
            flags |= 2;
            emit(0, e, we);
            return 1;
        }
        for (int d = 0; d < GB_D0; d++) {
            const P2 ab = pmid(a, b), bc = pmid(b, c), cd = pmid(c, e);
            const P2 abbc = pmid(ab, bc), bccd = pmid(bc, cd);
            const P2 pe = pmid(abbc, bccd), ad = pmid(a, e);
            const bool within = pdist_sq(pe, ad) <= tol_sq;
            if (within || d >= FT_MAX_DEPTH) {
                if (lane & ((1 << (GB_D0 - d)) - 1)) return 0;
                if (!within) flags |= 1;
                emit(0, e, we);
                return 1;
            }
            const float wab = fmid(wa, wb), wbc = fmid(wb, wc), wcd = fmid(wc, we);
            const float wabbc = fmid(wab, wbc), wbccd = fmid(wbc, wcd), wpe = fmid(wabbc, wbccd);
            if ((lane >> (GB_D0 - 1 - d)) & 1) {
                a = pe;
                b = bccd;
                c = cd;
                wa = wpe;
                wb = wbccd;
                wc = wcd;
            } else {
                b = ab;
                c = abbc;
                e = pe;
                wb = wab;
                wc = wabbc;
                we = wpe;
            }
        }
        n = cubic_walk<true>(a, b, c, e, wa, wb, wc, we, tol_sq, 0, INT_MAX, &dh, emit, GB_D0);
    }
    if (dh) flags |= 1;
    return n;
}

__device__ __forceinline__ bool gs_over(const GridStrokeBufs& S) { return *S.n_sraw > S.sraw_cap; }

__global__ void __launch_bounds__(BLOCK) k_gs_count(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    __shared__ long long ltmp[NWARP];
    const GridBuildBufs& G = P.gb;
    const GridStrokeBufs& S = P.gs;
    if (S.skip && *S.skip) return;  // a probe over a prefix of the ops completed the points
    const int tid = threadIdx.x;
    int flags = 0;
    const GbOp o = gb_op_of(G, flags);
    int n = 0;
    if (o.kind >= FT_OP_MOVE && o.kind <= FT_OP_CUBIC)
        n = gs_walk(P, o.op, o.kind, o.px, o.py, gs_width(G, o.lpc), gs_width(G, o.i), o.lane, flags,
                    [](int, P2, float) {});
    if (flags) atomicMax(&P.status[0], (flags & 1) ? FT_ERR_DEPTH : FT_ERR_ARG);
    int inc = n;
#pragma unroll
    for (int d = 1; d < GB_LANES; d <<= 1) {
        const int t = __shfl_up_sync(FULL, inc, d, GB_LANES);
        if (o.lane >= d) inc += t;
    }
    const int n_op = __shfl_sync(FULL, inc, GB_LANES - 1, GB_LANES);
    int tot;
    const int ex = block_excl_sum(o.lane == 0 ? n_op : 0, tmp, tot);
    if (o.i < G.n_ops) {
        G.opl[o.i * GB_LANES + o.lane] = inc - n;
        if (o.lane == 0) G.opi[o.i].y = ex;
    }
    if (tid == 0) G.opn[blockIdx.x] = tot;
    if (!gb_last_block(&S.done[0])) return;
    const int nb = (int)gridDim.x;
    long long carry = 0;
    for (int b0 = 0; b0 < nb; b0 += BLOCK) {
        const int b = b0 + tid;
        long long t;
        const long long e = block_excl_sum_ll(b < nb ? __ldcg(&G.opn[b]) : 0ll, ltmp, t);
        if (b < nb) G.opn[b] = carry + e;
        carry += t;
    }
    if (tid == 0) *S.n_sraw = carry;
}

__global__ void __launch_bounds__(BLOCK) k_gs_emit(KParams P) {
    const GridBuildBufs& G = P.gb;
    const GridStrokeBufs& S = P.gs;
    if (S.skip && *S.skip) return;  // a probe over a prefix of the ops completed the points
    if (gs_over(S)) return;  // every CTA: the caller grows the arrays
    int flags = 0;
    const GbOp o = gb_op_of(G, flags);
    if (o.kind < FT_OP_MOVE || o.kind > FT_OP_CUBIC) return;
    const long long off0 = G.opn[blockIdx.x] + G.opi[o.i].y;
    const int off = (int)(off0 + G.opl[o.i * GB_LANES + o.lane]);
    const int cap = S.sraw_cap;
    // a Move ends the sub-stroke before it open, a Close joined (stroker.rs:87-96)
    const unsigned char f0 = (unsigned char)(((o.lane == 0 && o.rs) ? 1 : 0) | (o.kind != FT_OP_MOVE ? 2 : 0));
    const unsigned char f1 = (unsigned char)(o.kind != FT_OP_MOVE ? 2 : 0);
    float4* raw4 = S.raw4;
    unsigned char* sfl = S.sfl;
    int* sopi = S.sopi;
    const int i = o.i;
    gs_walk(P, o.op, o.kind, o.px, o.py, gs_width(G, o.lpc), gs_width(G, o.i), o.lane, flags,
            [&](int k, P2 q, float w) {
                if (ck(off + k < cap, 13) && off + k < cap) {
                    raw4[off + k] = make_float4(q.x, q.y, w, 0.f);
                    sfl[off + k] = k == 0 ? f0 : f1;
                    sopi[off + k] = i;
                }
            });
}

// Kept raw stroke points and sub-stroke starts per tile, packed (kept << 32 | starts).
__global__ void __launch_bounds__(BLOCK) k_gs_keep(KParams P) {
    __shared__ long long ltmp[NWARP];
    const GridStrokeBufs& S = P.gs;
    if (S.skip && *S.skip) return;  // a probe over a prefix of the ops completed the points
    if (gs_over(S)) return;
    const int M = (int)*S.n_sraw, nt = (M + GB_TILE - 1) / GB_TILE, tid = threadIdx.x;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const int k0 = t * GB_TILE + GB_PER * tid;
        long long v = 0;
        float2 q = make_float2(0.f, 0.f);
        if (k0 > 0 && k0 <= M) {
            const float4 p = S.raw4[k0 - 1];
            q = make_float2(p.x, p.y);
        }
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            const int k = k0 + j;
            if (k >= M) break;
            const float4 p = S.raw4[k];
            const int rs = S.sfl[k] & 1;
            const bool keep = rs || !(p.x == q.x && p.y == q.y);
            v += ((long long)(keep ? 1 : 0) << 32) | rs;
            q = make_float2(p.x, p.y);
        }
        long long tot;
        block_excl_sum_ll(v, ltmp, tot);
        if (tid == 0) S.stile[t] = make_int2((int)(tot >> 32), (int)(tot & 0xFFFFFFFFll));
    }
    if (!gb_last_block(&S.done[1])) return;
    long long carry = 0;
    for (int b0 = 0; b0 < nt; b0 += BLOCK) {
        const int b = b0 + tid;
        long long x = 0;
        if (b < nt) {
            const int2 a = __ldcg(&S.stile[b]);
            x = ((long long)a.x << 32) | (unsigned)a.y;
        }
        long long t;
        const long long e = carry + block_excl_sum_ll(x, ltmp, t);
        if (b < nt) S.stile[b] = make_int2((int)(e >> 32), (int)(e & 0xFFFFFFFFll));
        carry += t;
    }
    if (tid == 0) {
        const int kept = (int)(carry >> 32);
        S.st[0] = min(kept, PT_CAP);
        S.st[6] = kept > PT_CAP ? 1 : 0;
        if (S.final_flag && kept > PT_CAP) *S.final_flag = 1;
    }
}

__global__ void __launch_bounds__(BLOCK) k_gs_write(KParams P) {
    __shared__ long long ltmp[NWARP];
    const GridStrokeBufs& S = P.gs;
    if (S.skip && *S.skip) return;  // a probe over a prefix of the ops completed the points
    if (gs_over(S)) return;
    const int M = (int)*S.n_sraw, nt = (M + GB_TILE - 1) / GB_TILE, tid = threadIdx.x;
    const int count = S.st[0];
    float4* spts = reinterpret_cast<float4*>(P.scratch + P.L.spts);
    SubRec* subs = reinterpret_cast<SubRec*>(P.scratch + P.L.subs);
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const int2 c = S.stile[t];
        const int k0 = t * GB_TILE + GB_PER * tid;
        float4 p[GB_PER];
        int f[GB_PER], keep = 0;
        long long v = 0;
        float2 q = make_float2(0.f, 0.f);
        if (k0 > 0 && k0 <= M) {
            const float4 pp = S.raw4[k0 - 1];
            q = make_float2(pp.x, pp.y);
        }
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            const int k = k0 + j;
            p[j] = make_float4(0.f, 0.f, 0.f, 0.f);
            f[j] = 0;
            if (k < M) {
                p[j] = S.raw4[k];
                f[j] = S.sfl[k];
                const int rs = f[j] & 1;
                if (rs || !(p[j].x == q.x && p[j].y == q.y)) keep |= 1 << j;
                v += ((long long)((keep >> j) & 1) << 32) | rs;
                q = make_float2(p[j].x, p[j].y);
            }
        }
        long long tot;
        const long long e = block_excl_sum_ll(v, ltmp, tot);
        int pos = c.x + (int)(e >> 32), sid = c.y + (int)(e & 0xFFFFFFFFll);
#pragma unroll
        for (int j = 0; j < GB_PER; j++) {
            if (!((keep >> j) & 1)) continue;
            const int rs = f[j] & 1;
            if (pos < PT_CAP) {
                spts[pos] = p[j];
                if (rs) {
                    subs[sid].start = pos;
                    if (sid > 0) subs[sid - 1].joined = (f[j] >> 1) & 1;
                    atomicMax(&S.st[1], sid + 1);
                }
                if (pos == count - 1) S.st[2] = S.sopi[k0 + j];  // the op of the last kept point
            }
            pos++;
            sid += rs;
        }
    }
}

// Sub-strokes (stroker.rs:87-96, 239-262), 256 a CTA step.
__global__ void __launch_bounds__(BLOCK) k_gs_subs(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    const GridBuildBufs& G = P.gb;
    const GridStrokeBufs& S = P.gs;
    if (gs_over(S)) return;
    const int tid = threadIdx.x, nsub = S.st[1], count = S.st[0];
    SubRec* subs = reinterpret_cast<SubRec*>(P.scratch + P.L.subs);
    const int nc = (nsub + BLOCK - 1) / BLOCK;
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int si = c * BLOCK + tid;
        int items = 0;
        if (si < nsub) {
            const SubRec r = subs[si];
            const int n = (si + 1 < nsub ? subs[si + 1].start : count) - r.start;
            int joined = r.joined;
            if (si == nsub - 1) {
                // the last sub-stroke: the close events after its last point
                const int cm = S.st[4], pc = S.st[3];
                if (S.st[6])
                    joined = cm > S.st[2] ? (__ldg(&G.ops[cm].kind) == FT_OP_CLOSE) : 0;
                else
                    joined = pc >= 0 ? (__ldg(&G.ops[pc].kind) == FT_OP_CLOSE) : 0;
                subs[si].joined = joined;
            }
            // SubStroke::len with u16 arithmetic: n + 1 wraps at 65,536
            const int len = joined ? ((n + 1) & 0xFFFF) : (n > 0 ? n - 1 : 0);
            items = len > 0 ? 2 * len + 2 : 0;
            subs[si].n = n;
            subs[si].len = len;
        }
        int tot;
        const int off = block_excl_sum(items, tmp, tot);
        if (si < nsub) subs[si].item_off = off;
        if (tid == 0) S.subt[c] = tot;
    }
    if (!gb_last_block(&S.done[2])) return;
    int carry = 0;
    for (int b0 = 0; b0 < nc; b0 += BLOCK) {
        const int b = b0 + tid;
        int tot;
        const int e = block_excl_sum(b < nc ? __ldcg(&S.subt[b]) : 0, tmp, tot);
        if (b < nc) S.subt[b] = carry + e;
        carry += tot;
    }
    if (tid == 0) S.st[5] = carry;
}

// Outline item t: its sub-stroke (the last with item offset <= t: empty sub-strokes share
// the next one's offset and come before it) and its index u in it.
__device__ __forceinline__ SubRec go_item(const GridStrokeBufs& S, const SubRec* subs, int nsub, int t, int& u) {
    int lo = 0, hi = nsub - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (subs[mid].item_off + S.subt[mid / BLOCK] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    SubRec sr = subs[lo];
    sr.item_off += S.subt[lo / BLOCK];
    u = t - sr.item_off;
    return sr;
}

__global__ void __launch_bounds__(BLOCK) k_go_count(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    __shared__ long long ltmp[NWARP];
    const GridBuildBufs& G = P.gb;
    const GridStrokeBufs& S = P.gs;
    if (gs_over(S)) return;
    const int tid = threadIdx.x, nsub = S.st[1], n_items = min(S.st[5], GS_ITEMS_CAP);
    const float4* spts = reinterpret_cast<const float4*>(P.scratch + P.L.spts);
    const SubRec* subs = reinterpret_cast<const SubRec*>(P.scratch + P.L.subs);
    const int nc = (n_items + BLOCK - 1) / BLOCK;
    int depth_hit = 0;
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int t = c * BLOCK + tid;
        int n = 0;
        if (t < n_items) {
            int u;
            const SubRec sr = go_item(S, subs, nsub, t, u);
            n = outline_item(P, spts, sr, u, INT_MAX, INT_MAX, &depth_hit, [](int, P2) {});
        }
        int tot;
        const int off = block_excl_sum(n, tmp, tot);
        if (t < n_items) S.itoff[t] = off;
        if (tid == 0) S.itc[c] = tot;
    }
    if (depth_hit) atomicMax(&P.status[0], FT_ERR_DEPTH);
    if (!gb_last_block(&S.done[3])) return;
    long long carry = 0;
    for (int b0 = 0; b0 < nc; b0 += BLOCK) {
        const int b = b0 + tid;
        long long t;
        const long long e = block_excl_sum_ll(b < nc ? (long long)__ldcg(&S.itc[b]) : 0ll, ltmp, t);
        if (b < nc) S.itc[b] = (int)min(carry + e, (long long)INT_MAX);
        carry += t;
    }
    if (tid == 0) *G.n_raw = carry;
}

__global__ void __launch_bounds__(BLOCK) k_go_emit(KParams P) {
    __shared__ int tmp[2 * NWARP + 2];
    __shared__ int s_c;
    const GridBuildBufs& G = P.gb;
    const GridStrokeBufs& S = P.gs;
    if (gs_over(S)) return;
    const long long n_raw = *G.n_raw;
    if (n_raw > G.raw_cap) return;
    const int tid = threadIdx.x, nsub = S.st[1], n_items = min(S.st[5], GS_ITEMS_CAP), cap = G.raw_cap;
    const float4* spts = reinterpret_cast<const float4*>(P.scratch + P.L.spts);
    const SubRec* subs = reinterpret_cast<const SubRec*>(P.scratch + P.L.subs);
    for (int t = blockIdx.x * BLOCK + tid; t < n_items; t += gridDim.x * BLOCK) {
        int u;
        const SubRec sr = go_item(S, subs, nsub, t, u);
        const int off = S.itc[t / BLOCK] + S.itoff[t];
        // a figure run starts at each side's first point after a Close: the forward side
        // always (after the previous sub-stroke's Close, or first), the reverse side when
        // the sub-stroke is joined (stroker.rs:255-260)
        const bool rev = u > sr.len, joined = sr.joined != 0;
        const int j = rev ? u - sr.len - 1 : u;
        const int rsk = ((!rev && ((!joined && j == 0) || (joined && j == 1))) || (rev && joined && j == 1)) ? 0 : -1;
        int dh = 0;
        const int n = outline_item(P, spts, sr, u, 0, INT_MAX, &dh, [&](int k, P2 q) {
            const P2 tq = xform(P.xf, q);  // the outline is transformed again (F9)
            if (ck(off + k < cap, 16) && off + k < cap) {
                G.raw[off + k] = make_int2(f2fx(tq.x), f2fx(tq.y));
                G.fl[off + k] = k == rsk ? (unsigned char)1 : (unsigned char)0;
            }
        });
        if (rsk == 0 && n > 0 && off < cap) atomicMax(&G.tr[off / GB_TILE], off);
    }
    if (!gb_last_block(&G.done[2])) return;
    gb_scan_tr(G, n_raw, tmp, s_c);
}

cudaError_t launch_grid_stroke(const KParams& p, int sm_count, cudaStream_t s, const KParams* probe) {
    const int nbo = (p.gb.n_ops + BLOCK - 1) / BLOCK;
    if (nbo <= 0 || p.gb.raw_cap % GB_TILE || p.gb.raw_cap > GB_RAW_MAX || p.gs.sraw_cap % GB_TILE ||
        p.gs.sraw_cap > GB_RAW_MAX || !p.gs.st || p.pt_cap != PT_CAP)
        return cudaErrorInvalidValue;
    if (probe && (probe->gb.n_ops <= 0 || probe->gb.n_ops > p.gb.n_ops)) return cudaErrorInvalidValue;
    const int gt = std::max(1, 4 * sm_count);
    k_gb_ops<<<nbo, BLOCK, 0, s>>>(p);  // pens and widths of every op (the probe's too)
    for (const KParams* q : {probe, &p}) {
        if (!q) continue;
        const int nbw = (q->gb.n_ops + GB_OPB - 1) / GB_OPB;
        k_gs_count<<<nbw, BLOCK, 0, s>>>(*q);
        k_gs_emit<<<nbw, BLOCK, 0, s>>>(*q);
        k_gs_keep<<<gt, BLOCK, 0, s>>>(*q);
        k_gs_write<<<gt, BLOCK, 0, s>>>(*q);
    }
    k_gs_subs<<<std::max(1, std::min(gt, PT_CAP / BLOCK + 1)), BLOCK, 0, s>>>(p);
    k_go_count<<<gt, BLOCK, 0, s>>>(p);
    k_go_emit<<<gt, BLOCK, 0, s>>>(p);
    k_gb_keep<<<gt, BLOCK, 0, s>>>(p);
    k_gb_write<<<gt, BLOCK, 0, s>>>(p);
    k_gb_top<<<GB_TOP_BLOCKS, BLOCK, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_composite_build(const KParams& p, int grid, int smem_bytes, cudaStream_t s, bool few_ctas) {
    auto kern = p.stroke ? k_cbuild<true> : k_cbuild<false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                         few_ctas ? FEW_CTAS_CARVEOUT : (int)cudaSharedmemCarveoutDefault);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e != cudaSuccess) return e;
    kern<<<grid, BLOCK, smem_bytes, s>>>(p);
    return cudaGetLastError();
}

// As raster_blocks_per_sm: the query is made with no carve-out preference.
int composite_build_blocks_per_sm(int smem_bytes, bool stroke) {
    auto kern = stroke ? k_cbuild<true> : k_cbuild<false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutDefault);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, BLOCK, smem_bytes) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_composite_bands(const KParams& p, int smem_bytes, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(k_cbands, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e != cudaSuccess) return e;
    k_cbands<<<p.n_bands, 32 * p.band_rows, smem_bytes, s>>>(p);
    return cudaGetLastError();
}

}  // namespace ftk

// ===========================================================================
// Allocation-free single-path fill (ft_fill_noalloc).
//
// For callers that may not allocate device memory themselves or through this
// library: a host whose device memory belongs to another runtime's allocator (a game
// engine's or a language runtime's pool that must see every allocation), or a
// process held to a fixed device-memory budget.  The figure scratch of one CTA lives
// in a file-scope device array that every GPU loading this library holds until the
// process exits; the caller passes only inputs and outputs.  One CTA rasterises the
// whole path.
namespace ftk {

// vertices, sub-figure starts and edges of one figure of up to FT_MAX_POINTS vertices
constexpr size_t NOALLOC_SCRATCH_BYTES = align256(SCR_EDGES + (size_t)PT_CAP * sizeof(EdgeRec));
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

__global__ void __launch_bounds__(BLOCK) k_fill_noalloc(KParams P, ft_path_desc d, unsigned char* scratch,
                                                        int32_t* status_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ CState S;
    __shared__ int s_tmp3[3 * NWARP];
    int2* pts = reinterpret_cast<int2*>(scratch + SCR_PTS);
    int* ss = reinterpret_cast<int*>(scratch + SCR_SS);
    EdgeRec* edges = reinterpret_cast<EdgeRec*>(scratch + SCR_EDGES);
    BuildSmem& B = *reinterpret_cast<BuildSmem*>(smem);
    CompactSmem* Cs = reinterpret_cast<CompactSmem*>(smem + ((sizeof(BuildSmem) + 15) & ~(size_t)15));
    build_fill<BlockG>(P, d, d.s_width, B, Cs, S, pts, ss, PT_CAP);
    if (S.count > 0) {
        top_and_dir<BlockG>(S, pts, ss, s_tmp3);
        build_edges<BlockG>(S, pts, ss, edges);
        __syncthreads();
        const int lo = max(S.top_row, 0), hi = (int)d.height;
        const int wp4 = (int)(((d.width + 3) & ~3u) * 4);
        const int R = max(1, min((P.smem_bytes - RASTER_FIXED_SMEM) / max(wp4, 4), max(hi, 1)));
        if (lo < hi && d.width > 0) raster_rows(P, d, S, edges, lo, hi, R, smem);
    }
    if (threadIdx.x == 0 && status_out)
        *status_out = S.flags ? ((S.flags & 1) ? FT_ERR_DEPTH : FT_ERR_ARG) : FT_OK;
}

}  // namespace ftk

#include <cuda.h>
#include <mutex>

namespace {
// Set-up of ft_fill_noalloc per device: the device address of g_noalloc_scratch and the
// kernel's dynamic shared-memory limit, both belonging to the device's current context.
// A device reset (cudaDeviceReset) destroys that context and unloads the module, so the
// set-up is keyed by the context's unique id and done again in a new context.
constexpr int NOALLOC_MAX_DEVICES = 64;
struct NoallocDev {
    unsigned long long ctx_id = 0;  // 0: not set up
    void* scratch = nullptr;
    int smem_max = 0;
};
NoallocDev g_noalloc[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_mu;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current context (0 when none is current yet),
// through the runtime's driver entry points (no link against the driver library).
unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    CUcontext cu = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&cu) != CUDA_SUCCESS || !cu || get_id(cu, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// The set-up of `dev` (current) for its current context; false when a CUDA call fails.
bool noalloc_setup(int dev, NoallocDev& out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoallocDev& D = g_noalloc[dev];
    unsigned long long id = current_ctx_id();
    if (id == 0 || id != D.ctx_id) {
        void* p = nullptr;
        // also makes the device's primary context current when none was
        if (cudaGetSymbolAddress(&p, ftk::g_noalloc_scratch) != cudaSuccess || !p) return false;
        int optin = 0;
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
        const int smem_max = optin - 1024;
        if (cudaFuncSetAttribute(ftk::k_fill_noalloc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max) !=
            cudaSuccess)
            return false;
        id = current_ctx_id();
        if (id == 0) return false;
        D.ctx_id = id;
        D.scratch = p;
        D.smem_max = smem_max;
    }
    out = D;
    return true;
}
}  // namespace

extern "C" FT_API int ft_fill_noalloc(int32_t rule, const ft_op* ops, uint32_t n_ops, int32_t fmt,
                                      const uint8_t clr[4], uint8_t* raster, uint32_t w, uint32_t h,
                                      uint32_t stride, const float transform[6], float tolerance, float pen_width,
                                      int32_t* status, void* stream) {
    if ((rule != FT_NONZERO && rule != FT_EVENODD) || (fmt != FT_MATTE8 && fmt != FT_RGBA8P)) return FT_ERR_ARG;
    if ((n_ops && !ops) || (w && h && !raster)) return FT_ERR_ARG;
    if (w > FT_MAX_WIDTH) return FT_ERR_CAP;  // one band row of cell areas must fit in shared memory
    const uint32_t bpp = fmt == FT_RGBA8P ? 4 : 1;
    if (h && stride < (uint64_t)w * bpp) return FT_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(ops) & 15) ||
        (fmt == FT_RGBA8P && ((reinterpret_cast<uintptr_t>(raster) | stride) & 3)))
        return FT_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) return FT_ERR_CUDA;
    NoallocDev D;
    if (!noalloc_setup(dev, D)) return FT_ERR_CUDA;
    ft_path_desc d;
    memset(&d, 0, sizeof(d));
    d.n_ops = n_ops;
    d.width = w;
    d.height = h;
    d.stride = stride;
    d.s_width = pen_width;
    if (clr) memcpy(d.clr, clr, 4);
    ftk::KParams p;
    memset(&p, 0, sizeof(p));
    p.ops = ops;
    p.rasters = raster;
    p.rule = rule;
    p.fmt = fmt;
    static const float ident[6] = {1, 0, 0, 0, 1, 0};
    for (int i = 0; i < 6; i++) p.xf[i] = transform ? transform[i] : ident[i];
    const float t = tolerance > 0.01f ? tolerance : 0.01f;
    p.tol_sq = t * t;
    const int wp = (int)((w + 3) & ~3u);
    int smem = std::max(ftk::RASTER_FIXED_SMEM + 16 * wp * 4, 40 * 1024);
    smem = std::min(smem, D.smem_max);
    p.smem_bytes = smem;
    unsigned char* scratch = static_cast<unsigned char*>(D.scratch);
    // the launch's own status: an error some earlier, unrelated call left in the runtime
    // is neither consumed nor reported here
    void* args[] = {&p, &d, &scratch, &status};
    const cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(ftk::k_fill_noalloc), dim3(1),
                                           dim3(ftk::BLOCK), args, (size_t)smem, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? FT_OK : FT_ERR_CUDA;
}

// Check build: the first failing bounds check's site since the last call (0: none), and
// whether the checks are compiled in.  No counterpart in footile.
extern "C" FT_API int ft_check_failures(int32_t* site, int32_t* compiled_in) {
    if (compiled_in) *compiled_in = FT_CHECK;
    if (!site) return FT_OK;
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, ftk::g_check, sizeof(int)) != cudaSuccess) return FT_ERR_CUDA;
    *site = v;
    const int zero = 0;
    if (cudaMemcpyToSymbol(ftk::g_check, &zero, sizeof(int)) != cudaSuccess) return FT_ERR_CUDA;
    return FT_OK;
}
