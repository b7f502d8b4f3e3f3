// Stroke points of the adjoint: the block walk (stroke_points_block) against a walk of
// the ops one by one on one thread (Plotter's pen walk into Stroke::add_point / close,
// plotter.rs:175-332, stroker.rs:204-236), path by path, bit for bit: the stroke points
// (position, width, t and provenance) and the sub-strokes (start, count, joined, done).
// Seeded random paths with coincident points, closes, moves, pen widths, NaN and
// infinite controls and unknown op kinds, one path past the 65,535-point cap and one
// chunk of ops with more raw points than a window, under two transforms and tolerances.
// Exit status 0 when every path agrees.  Compiled with the product's flags by
// tests/test_gpu_stroke_points.py.
#include "ft_adjoint.cu"
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <vector>
#include <random>
using namespace fta;
namespace fta { namespace {
// One thread: the stroke points and sub-strokes of the path, op by op.  Returns the
// stroke point count; *n_sub gets the sub-stroke count, *status the path status.
__device__ int stroke_points_serial(const AParams& p, const ft_op* ops, int n, float sw0, const StrokeScr& S,
                                 int* n_sub, int* status) {
    const float* m = p.xf;
    // ---- stroke points (plotter.rs:175-332 into Stroke::add_point / close)
    float sw = sw0;
    int cur_pw = -1, pen = -1, pen_wsrc = -1;
    P2 penp = p2(0.0f, 0.0f);
    float penw = sw0;
    int ns = 0, nsub = 0;
    SSub cur{0, 0, 0, 0};  // the sub-stroke being built (stored when the next one starts)
    P2 last = p2(0.0f, 0.0f);
    auto close = [&](int joined) {
        if (ns > 0) {
            cur.joined = joined;
            cur.done = 1;
        }
    };
    auto add = [&](P2 q, float w, int op, int form, float t, int pn, int w0, int w1) {
        if (ns >= VCAP) return;  // the stroke keeps 65,535 points (stroker.rs:204-216)
        const int done = cur.done;
        if (done) {
            S.subs[nsub++] = cur;
            cur = SSub{ns, 0, 0, 0};
        }
        const bool coincident = ns > 0 && last.x == q.x && last.y == q.y;
        if (done || !coincident) {
            S.sp[ns++] = SPt{q.x, q.y, w, t, op, form, pn, w0, w1, 0};
            last = q;
            cur.n++;
        }
    };
    for (int i = 0; i < n; i++) {
        const ft_op o = load_op(ops, i);
        switch (o.kind) {
            case FT_OP_CLOSE:
                close(1);
                pen = -1;
                pen_wsrc = cur_pw;
                penp = p2(0.0f, 0.0f);
                penw = sw;
                break;
            case FT_OP_MOVE:
            case FT_OP_LINE: {
                const P2 q = op_pt(o, 0);
                if (o.kind == FT_OP_MOVE) close(0);
                add(xform(m, q), sw, i, F_POINT, 1.0f, -1, cur_pw, cur_pw);
                pen = i;
                pen_wsrc = cur_pw;
                penp = q;
                penw = sw;
                break;
            }
            case FT_OP_QUAD:
            case FT_OP_CUBIC: {
                const bool cubic = o.kind == FT_OP_CUBIC;
                const P2 A = xform(m, penp), B = xform(m, op_pt(o, 0)), C = xform(m, op_pt(o, 1));
                const P2 D = cubic ? xform(m, op_pt(o, 2)) : C;
                float wb, wc, wd;
                if (cubic) {  // float_lerp (geom.rs:14-16)
                    wb = __fadd_rn(sw, __fmul_rn(__fsub_rn(penw, sw), 1.0f / 3.0f));
                    wc = __fadd_rn(sw, __fmul_rn(__fsub_rn(penw, sw), 2.0f / 3.0f));
                    wd = sw;
                } else {
                    wb = ftk::fmid(penw, sw);
                    wc = sw;
                    wd = sw;
                }
                if (!pfinite(A) || !pfinite(B) || !pfinite(C) || !pfinite(D)) {
                    *status = max(*status, (int)FT_ERR_ARG);
                    add(D, sw, i, F_POINT, 1.0f, -1, cur_pw, cur_pw);
                } else {
                    int dh = 0;
                    const int pn = pen, w0 = pen_wsrc, w1 = cur_pw;
                    auto leaf = [&](int, P2 q, float w, float t) { add(q, w, i, cubic ? F_CUBIC : F_QUAD, t, pn, w0, w1); };
                    if (cubic)
                        curve_walk_w<true>(A, B, C, D, penw, wb, wc, wd, p.tol_sq, &dh, leaf);
                    else
                        curve_walk_w<false>(A, B, C, D, penw, wb, wc, wd, p.tol_sq, &dh, leaf);
                    if (dh) *status = max(*status, (int)FT_ERR_DEPTH);
                }
                pen = i;
                pen_wsrc = cur_pw;
                penp = cubic ? op_pt(o, 2) : op_pt(o, 1);
                penw = sw;
                break;
            }
            case FT_OP_PEN_WIDTH:
                sw = o.v[0];
                cur_pw = i;
                break;
            default:
                break;
        }
    }
    S.subs[nsub++] = cur;
    *n_sub = nsub;
    return ns;
}

}}

__global__ void k_cmp(AParams p, unsigned char* scrA, unsigned char* scrB, int* out) {
    __shared__ ASmem sm;
    __shared__ int sres[4];
    const int tid = threadIdx.x;
    const StrokeScr SA = stroke_scr(scrA + (size_t)blockIdx.x * A_SCRATCH_STROKE);
    const StrokeScr SB = stroke_scr(scrB + (size_t)blockIdx.x * A_SCRATCH_STROKE);
    for (uint32_t path = blockIdx.x; path < p.n_paths; path += gridDim.x) {
        const ft_path_desc d = p.paths[path];
        const ft_op* ops = p.ops + d.op_begin;
        if (tid == 0) {
            int st = FT_OK, nsub = 0;
            sres[0] = stroke_points_serial(p, ops, (int)d.n_ops, d.s_width, SA, &nsub, &st);
            sres[1] = nsub;
            sres[2] = st;
            sm.status = FT_OK;
        }
        __syncthreads();
        int nsubB = 0;
        const int nsB = stroke_points_block(p, sm, ops, (int)d.n_ops, d.s_width, SB, &nsubB);
        __syncthreads();
        const int nsA = sres[0], nsubA = sres[1];
        __shared__ int first_sp, first_sub;
        if (tid == 0) first_sp = first_sub = INT_MAX;
        __syncthreads();
        const int nsm = min(nsA, nsB);
        for (int k = tid; k < nsm; k += ABLOCK) {
            const int* a = reinterpret_cast<const int*>(SA.sp + k);
            const int* b = reinterpret_cast<const int*>(SB.sp + k);
            bool eq = true;
            for (int f = 0; f < 10; f++) eq = eq && a[f] == b[f];
            if (!eq) atomicMin(&first_sp, k);
        }
        const int nbm = min(nsubA, nsubB);
        for (int k = tid; k < nbm; k += ABLOCK) {
            const SSub a = SA.subs[k], b = SB.subs[k];
            if (a.start != b.start || a.n != b.n || a.joined != b.joined || a.done != b.done) atomicMin(&first_sub, k);
        }
        __syncthreads();
        if (tid == 0) {
            int* o = out + (size_t)path * 8;
            o[0] = nsA; o[1] = nsB; o[2] = nsubA; o[3] = nsubB; o[4] = sres[2]; o[5] = sm.status;
            o[6] = first_sp; o[7] = first_sub;
        }
        __syncthreads();
    }
}

static void op(std::vector<ft_op>& v, int kind, float a = 0, float b = 0, float c = 0, float d = 0, float e = 0, float f = 0) {
    ft_op o{};
    o.kind = kind;
    o.v[0] = a; o.v[1] = b; o.v[2] = c; o.v[3] = d; o.v[4] = e; o.v[5] = f;
    v.push_back(o);
}

int main() {
    std::mt19937 rng(12345);
    std::vector<ft_op> ops;
    std::vector<ft_path_desc> paths;
    auto coord = [&](float grid, float span) {
        if (rng() % 4 == 0) return std::floor((float)(rng() % 1000) / 1000.f * span / grid) * grid;
        return (float)(rng() % 100000) / 100000.f * span;
    };
    const int NP = 600;
    for (int pi = 0; pi < NP; pi++) {
        ft_path_desc d{};
        d.op_begin = (uint32_t)ops.size();
        d.s_width = 1.0f + (rng() % 8);
        int n;
        int mode = pi % 10;
        if (pi == 0) n = 0;
        else if (mode == 9) n = 300 + rng() % 900;           // several chunks
        else n = 1 + rng() % 120;
        float span = (mode == 8) ? 4.0f : 200.0f;  // tiny span: many coincident points
        float last_x = 0, last_y = 0;
        for (int k = 0; k < n; k++) {
            int r = rng() % 100;
            float x = coord(1.0f, span), y = coord(1.0f, span);
            if (rng() % 6 == 0) { x = last_x; y = last_y; }  // repeat the pen
            if (r < 10) op(ops, FT_OP_MOVE, x, y);
            else if (r < 40) op(ops, FT_OP_LINE, x, y);
            else if (r < 60) op(ops, FT_OP_QUAD, coord(1, span), coord(1, span), x, y);
            else if (r < 78) op(ops, FT_OP_CUBIC, coord(1, span), coord(1, span), coord(1, span), coord(1, span), x, y);
            else if (r < 88) op(ops, FT_OP_CLOSE);
            else if (r < 97) op(ops, FT_OP_PEN_WIDTH, 0.5f + (rng() % 20) * 0.5f);
            else if (r < 98) op(ops, FT_OP_LINE, NAN, y);
            else if (r < 99) op(ops, FT_OP_QUAD, INFINITY, 1.0f, x, y);
            else op(ops, 17);  // unknown kind
            last_x = x; last_y = y;
        }
        d.n_ops = (uint32_t)(ops.size() - d.op_begin);
        paths.push_back(d);
    }
    // past the stroke point cap: many lines
    {
        ft_path_desc d{};
        d.op_begin = (uint32_t)ops.size();
        d.s_width = 2.0f;
        op(ops, FT_OP_MOVE, 0, 0);
        for (int k = 0; k < 70000; k++) {
            op(ops, FT_OP_LINE, (float)(k % 300), (float)(k / 300));
            if (k == 65533) op(ops, FT_OP_CLOSE);
            if (k == 65540) op(ops, FT_OP_CLOSE);
            if (k == 66000) op(ops, FT_OP_MOVE, 5, 5);
        }
        op(ops, FT_OP_CLOSE);
        d.n_ops = (uint32_t)(ops.size() - d.op_begin);
        paths.push_back(d);
    }
    // a chunk of big cubics: more raw points than one window
    {
        ft_path_desc d{};
        d.op_begin = (uint32_t)ops.size();
        d.s_width = 2.0f;
        op(ops, FT_OP_MOVE, 0, 0);
        for (int k = 0; k < 250; k++) {
            op(ops, FT_OP_CUBIC, 3000, (float)(k * 7 % 3000), -2000, 2500, (float)(k % 50), (float)(k % 70));
            if (k % 50 == 49) op(ops, FT_OP_CLOSE);
        }
        d.n_ops = (uint32_t)(ops.size() - d.op_begin);
        paths.push_back(d);
    }
    const int np = (int)paths.size();
    ft_op* dops; ft_path_desc* dpaths; int* dout; unsigned char *sa, *sb;
    const int grid = 32;
    cudaMalloc(&dops, sizeof(ft_op) * ops.size());
    cudaMalloc(&dpaths, sizeof(ft_path_desc) * np);
    cudaMalloc(&dout, sizeof(int) * 8 * np);
    cudaMalloc(&sa, (size_t)grid * A_SCRATCH_STROKE);
    cudaMalloc(&sb, (size_t)grid * A_SCRATCH_STROKE);
    cudaMemcpy(dops, ops.data(), sizeof(ft_op) * ops.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(dpaths, paths.data(), sizeof(ft_path_desc) * np, cudaMemcpyHostToDevice);
    int bad = 0, total_pts = 0, maxns = 0;
    for (int variant = 0; variant < 2; variant++) {
        AParams p{};
        p.ops = dops; p.paths = dpaths; p.n_paths = np;
        float xf0[6] = {1, 0, 0, 0, 1, 0}, xf1[6] = {0.7f, 0.2f, 3.5f, -0.3f, 1.3f, -2.0f};
        for (int k = 0; k < 6; k++) p.xf[k] = variant ? xf1[k] : xf0[k];
        p.tol_sq = variant ? 0.0001f : 0.09f;
        p.stroke = 1;
        cudaMemset(dout, 0, sizeof(int) * 8 * np);
        k_cmp<<<grid, ABLOCK>>>(p, sa, sb, dout);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) { printf("CUDA error %s\n", cudaGetErrorString(e)); return 1; }
        std::vector<int> out(8 * np);
        cudaMemcpy(out.data(), dout, sizeof(int) * 8 * np, cudaMemcpyDeviceToHost);
        for (int i = 0; i < np; i++) {
            const int* o = &out[8 * i];
            total_pts += o[0];
            maxns = std::max(maxns, o[0]);
            if (o[0] != o[1] || o[2] != o[3] || o[4] != o[5] || o[6] != INT_MAX || o[7] != INT_MAX) {
                if (bad < 20)
                    printf("variant %d path %d: ns %d/%d nsub %d/%d status %d/%d first sp %d first sub %d\n", variant, i,
                           o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7]);
                bad++;
            }
        }
    }
    printf("paths %d x 2, stroke points %d (max %d per path), mismatching paths %d\n", np, total_pts, maxns, bad);
    return bad ? 2 : 0;
}
