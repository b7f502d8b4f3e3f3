// ft_adjoint.cuh — launch interface of the coverage adjoint kernels (ft_adjoint.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/footile_gpu.h"

namespace fta {

constexpr int ABLOCK = 256;                 // threads per CTA (one CTA per path at a time)
constexpr int VCAP = FT_MAX_POINTS;         // flattened vertices per path
constexpr int BAND_FLOATS = 16384;          // 64 KB shared band of accumulation / gradient cells

constexpr size_t a_align(size_t x) { return (x + 255) & ~(size_t)255; }
// Per-CTA scratch in global memory (L2-resident for small paths): vertex positions,
// the first vertex of each vertex's sub-figure, vertex gradients and per-sub-figure
// flags.
constexpr size_t AS_POS = 0;                                              // float2[VCAP]
constexpr size_t AS_SUB = a_align(AS_POS + (size_t)VCAP * 8);             // int[VCAP]
constexpr size_t AS_GRAD = a_align(AS_SUB + (size_t)VCAP * 4);            // float2[VCAP]
constexpr size_t AS_FLAG = a_align(AS_GRAD + (size_t)VCAP * 8);           // int[VCAP]
// Edges binned by row band, built once per path: band k's edges are
// blist[boff[k] .. boff[k + 1]).  Paths with more bands or (edge, band) pairs scan
// every edge for every band instead.
constexpr int NB_CAP = BAND_FLOATS - 1;     // bands (the shared band buffer is the histogram)
constexpr int PAIR_CAP = 1 << 18;           // (edge, band) pairs
constexpr size_t AS_BOFF = a_align(AS_FLAG + (size_t)VCAP * 4);          // int[NB_CAP + 1]
constexpr size_t AS_BLIST = a_align(AS_BOFF + (size_t)(NB_CAP + 1) * 4);  // int[PAIR_CAP]
constexpr size_t A_SCRATCH_PER_CTA = a_align(AS_BLIST + (size_t)PAIR_CAP * 4);

// Strokes add, after the fill arrays: the node of each outline vertex, stroke points,
// sub-strokes, outline nodes (offset points, miter intersections, arc points) and
// their gradients.
constexpr int NODE_CAP = 200000;            // outline nodes per stroke
constexpr size_t SPT_BYTES = 40, SND_BYTES = 32, SSUB_BYTES = 16;
constexpr size_t AS_VNODE = A_SCRATCH_PER_CTA;                                   // int[VCAP]
constexpr size_t AS_SPT = a_align(AS_VNODE + (size_t)VCAP * 4);                  // stroke points
constexpr size_t AS_SSUB = a_align(AS_SPT + (size_t)VCAP * SPT_BYTES);           // sub-strokes
constexpr size_t AS_SND = a_align(AS_SSUB + (size_t)(VCAP + 1) * SSUB_BYTES);    // nodes
constexpr size_t AS_NG = a_align(AS_SND + (size_t)NODE_CAP * SND_BYTES);         // float2 node gradients
constexpr size_t AS_SPG = a_align(AS_NG + (size_t)NODE_CAP * 8);                 // float4 stroke point gradients
constexpr size_t AS_SOFF = a_align(AS_SPG + (size_t)VCAP * 16);                  // int[VCAP + 2] segment offsets
constexpr size_t AS_GST = a_align(AS_SOFF + (size_t)(VCAP + 2) * 4);             // int2[VCAP + 1] side starts
constexpr size_t A_SCRATCH_STROKE = a_align(AS_GST + (size_t)(VCAP + 1) * 8);

struct AParams {
    const ft_op* ops;
    const ft_path_desc* paths;
    uint32_t n_paths;
    float* cov;             // forward: coverage, width x height floats at raster_offset / stride
    float* area;            // forward: winding area (same layout); backward: read
    const float* grad_cov;  // backward: dLoss/dcov (layout of cov)
    float* grad_ops;        // backward: 6 floats per op, zeroed by the host, accumulated
    int* status;            // per path
    unsigned char* scratch; // A_SCRATCH_PER_CTA (fills) or A_SCRATCH_STROKE (strokes) per CTA
    float* grad_width;      // backward, strokes: d/d(starting pen width) per path, zeroed by the host
    float xf[6];
    float tol_sq;
    int rule;
    int stroke;             // Plotter::stroke: the outline of each path is filled NonZero
    int join;
    float miter_limit;
    float miter_g;  // ft_miter_angle(miter_limit)
    int no_area;            // NonZero only: keep no winding area; the backward takes dcov/dS from cov
                            // (0 < cov < 1 exactly where 0 < S < 1) and reads grad_cov only there
};

cudaError_t launch_adjoint(bool backward, const AParams& p, int grid, cudaStream_t s);
int adjoint_blocks_per_sm(bool backward);

}  // namespace fta
