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
constexpr size_t A_SCRATCH_PER_CTA = a_align(AS_FLAG + (size_t)VCAP * 4);

struct AParams {
    const ft_op* ops;
    const ft_path_desc* paths;
    uint32_t n_paths;
    float* cov;             // forward: coverage, width x height floats at raster_offset / stride
    float* area;            // forward: winding area (same layout); backward: read
    const float* grad_cov;  // backward: dLoss/dcov (layout of cov)
    float* grad_ops;        // backward: 6 floats per op, zeroed by the host, accumulated
    int* status;            // per path
    unsigned char* scratch; // A_SCRATCH_PER_CTA per CTA
    float xf[6];
    float tol_sq;
    int rule;
};

cudaError_t launch_adjoint(bool backward, const AParams& p, int grid, cudaStream_t s);
int adjoint_blocks_per_sm(bool backward);

}  // namespace fta
