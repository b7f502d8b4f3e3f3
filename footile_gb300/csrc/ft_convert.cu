// ft_convert.cu — Rgba8p -> SRgba8 and Matte8 -> SGray8 on the device, and the float
// ordered SrcOver of coverage layers with its adjoint.
//
// footile plots in linear premultiplied Rgba8p / Matte8; its examples then convert with
// pix (`Raster::<SRgba8>::with_raster`, examples/fishy.rs:33; `Raster::<SGray8>`,
// examples/drop.rs:22): straight alpha (channel / alpha) and the sRGB transfer
// function.  The conversion of one channel depends only on (alpha, channel), so it is a
// 256 x 256 byte table the host builds once (correctly rounded sRGB encoding of
// channel / alpha, IEC 61966-2-1) and every thread reads from shared memory.  The
// kernel streams 16-byte vectors: 4 Rgba8p or 16 Matte8 pixels per thread and step.
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/footile_gpu.h"

namespace ftc {

constexpr int CBLOCK = 256;

__device__ __forceinline__ uint4 convert16(uint4 v, int src_fmt, const uint8_t* lut) {
    unsigned* u = reinterpret_cast<unsigned*>(&v);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const unsigned p = u[j];
        if (src_fmt == FT_RGBA8P) {
            const unsigned a = p >> 24, row = a << 8;
            u[j] = (unsigned)lut[row | (p & 0xFF)] | ((unsigned)lut[row | ((p >> 8) & 0xFF)] << 8) |
                   ((unsigned)lut[row | ((p >> 16) & 0xFF)] << 16) | (a << 24);
        } else {  // Matte8: the mask byte is linear gray at full alpha
            u[j] = (unsigned)lut[0xFF00 | (p & 0xFF)] | ((unsigned)lut[0xFF00 | ((p >> 8) & 0xFF)] << 8) |
                   ((unsigned)lut[0xFF00 | ((p >> 16) & 0xFF)] << 16) | ((unsigned)lut[0xFF00 | (p >> 24)] << 24);
        }
    }
    return v;
}

// Persistent grid (one CTA per resident slot, each loads the table once).  Rows are
// cut into 16-byte groups; a thread takes UNROLL groups per step and issues all their
// loads before converting, which keeps enough bytes in flight for HBM.  Row tails
// (and rows that are not 16-byte aligned) go byte by byte.  `lut[a * 256 + c]`:
// straight, sRGB-encoded channel.
constexpr int UNROLL = 4;
__global__ void __launch_bounds__(CBLOCK) k_convert(int src_fmt, const uint8_t* __restrict__ src, uint32_t src_stride,
                                                    uint8_t* __restrict__ dst, uint32_t dst_stride, uint32_t w,
                                                    uint32_t h, const uint8_t* __restrict__ lut_g) {
    __shared__ __align__(16) uint8_t lut[256 * 256];
    for (int i = threadIdx.x; i < 256 * 256 / 16; i += CBLOCK)
        reinterpret_cast<uint4*>(lut)[i] = reinterpret_cast<const uint4*>(lut_g)[i];
    __syncthreads();
    const uint32_t row_bytes = src_fmt == FT_RGBA8P ? 4 * w : w;
    const bool vec = ((src_stride | dst_stride) & 15) == 0 &&
                     ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
    const uint32_t groups = vec ? row_bytes / 16 : 0;  // 16-byte groups per row
    const uint64_t n_groups = (uint64_t)groups * h;
    const uint64_t nthreads = (uint64_t)gridDim.x * CBLOCK;
    for (uint64_t t0 = (uint64_t)blockIdx.x * CBLOCK + threadIdx.x; t0 < n_groups; t0 += nthreads * UNROLL) {
        uint4 v[UNROLL];
        uint64_t g[UNROLL];
#pragma unroll
        for (int j = 0; j < UNROLL; j++) {
            g[j] = t0 + (uint64_t)j * nthreads;
            if (g[j] < n_groups) {
                const uint32_t y = (uint32_t)(g[j] / groups), k = (uint32_t)(g[j] - (uint64_t)y * groups);
                v[j] = reinterpret_cast<const uint4*>(src + (size_t)y * src_stride)[k];
            }
        }
#pragma unroll
        for (int j = 0; j < UNROLL; j++) {
            if (g[j] < n_groups) {
                const uint32_t y = (uint32_t)(g[j] / groups), k = (uint32_t)(g[j] - (uint64_t)y * groups);
                reinterpret_cast<uint4*>(dst + (size_t)y * dst_stride)[k] = convert16(v[j], src_fmt, lut);
            }
        }
    }
    // row tails
    const uint32_t tail = row_bytes - groups * 16;
    const uint64_t n_tail = (uint64_t)tail * h;
    for (uint64_t t = (uint64_t)blockIdx.x * CBLOCK + threadIdx.x; t < n_tail; t += nthreads) {
        const uint32_t y = (uint32_t)(t / tail), b = groups * 16 + (uint32_t)(t - (uint64_t)y * tail);
        const uint8_t* s = src + (size_t)y * src_stride;
        uint8_t* d = dst + (size_t)y * dst_stride;
        if (src_fmt == FT_RGBA8P) {
            const uint32_t px = b >> 2, ch = b & 3;
            const unsigned a = s[4 * px + 3];
            d[b] = ch == 3 ? (uint8_t)a : lut[(a << 8) | s[b]];
        } else {
            d[b] = lut[0xFF00 | s[b]];
        }
    }
}

int convert_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_convert, CBLOCK, 0) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_convert(int src_fmt, const uint8_t* src, uint32_t src_stride, uint8_t* dst, uint32_t dst_stride,
                           uint32_t w, uint32_t h, const uint8_t* lut, int grid, cudaStream_t s) {
    k_convert<<<grid, CBLOCK, 0, s>>>(src_fmt, src, src_stride, dst, dst_stride, w, h, lut);
    return cudaGetLastError();
}


// ------------------------------------------------------ ordered SrcOver adjoint
// The composite of an ordered batch in float: layer n (coverage cov_n, premultiplied
// colour c_n with alpha a_n, as footile's pix SrcOver, fig.rs:637-643) gives
//   C_n = c_n * cov_n + C_{n-1} * (1 - a_n * cov_n).
// With G = dLoss/dC_N, the factor (1 - a_n cov_n) is one scalar for all four channels,
// so dLoss/dcov_n = P_n * (G . c_n - a_n * E_{n-1}) with P_n the product of the later
// factors and E_n = G . C_n following the same recurrence as C (scalar).  Backward:
// one pass forward for E (recomputed, nothing kept from the forward call), written
// into the gradient planes, then one pass backward for P.  No division, so opaque
// layers (factor 0) are exact.  One thread per pixel; planes are n_layers x n_px floats.
// Layers are read SB at a time (independent streaming loads, then the recurrence), so
// that each thread keeps SB coverage loads in flight.
constexpr int SB = 8;

__global__ void k_srcover_fwd(const float* __restrict__ cov, uint32_t n_layers, uint64_t plane,
                              const float4* __restrict__ clr, const float4* __restrict__ init,
                              float4* __restrict__ out, uint32_t n_px) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_px;
         p += (uint64_t)gridDim.x * blockDim.x) {
        float4 c = init ? init[p] : make_float4(0.f, 0.f, 0.f, 0.f);
        auto layer = [&](uint32_t n, float v) {
            if (v == 0.0f) return;
            const float4 k = clr[n];
            const float f = 1.0f - k.w * v;
            c = make_float4(k.x * v + c.x * f, k.y * v + c.y * f, k.z * v + c.z * f, k.w * v + c.w * f);
        };
        uint32_t n = 0;
        for (; n + SB <= n_layers; n += SB) {
            float v[SB];
#pragma unroll
            for (int u = 0; u < SB; u++) v[u] = __ldcs(cov + (uint64_t)(n + u) * plane + p);
#pragma unroll
            for (int u = 0; u < SB; u++) layer(n + u, v[u]);
        }
        for (; n < n_layers; n++) layer(n, __ldcs(cov + (uint64_t)n * plane + p));
        out[p] = c;
    }
}

// PARTIAL: dLoss/dcov only where 0 < cov < 1 (elsewhere the plane is neither read nor
// written) — all a NonZero coverage adjoint needs, since dcov/dS is 0 at cov 0 and 1.
template <bool PARTIAL>
__global__ void k_srcover_bwd(const float* __restrict__ cov, uint32_t n_layers, uint64_t plane,
                              const float4* __restrict__ clr, const float4* __restrict__ init,
                              const float4* __restrict__ grad_out, float* __restrict__ grad_cov,
                              float4* __restrict__ grad_init, uint32_t n_px) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_px;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const float4 g = grad_out[p];
        const float4 c0 = init ? init[p] : make_float4(0.f, 0.f, 0.f, 0.f);
        float e = g.x * c0.x + g.y * c0.y + g.z * c0.z + g.w * c0.w;
        auto keep = [](float v) { return !PARTIAL || (v > 0.0f && v < 1.0f); };
        // E_{n-1} = g . C_{n-1} into the gradient plane
        auto up = [&](uint32_t n, float v) {
            if (keep(v)) grad_cov[(uint64_t)n * plane + p] = e;
            if (v == 0.0f) return;
            const float4 k = clr[n];
            e = (g.x * k.x + g.y * k.y + g.z * k.z + g.w * k.w) * v + e * (1.0f - k.w * v);
        };
        uint32_t n = 0;
        for (; n + SB <= n_layers; n += SB) {
            float v[SB];
#pragma unroll
            for (int u = 0; u < SB; u++) v[u] = __ldcs(cov + (uint64_t)(n + u) * plane + p);
#pragma unroll
            for (int u = 0; u < SB; u++) up(n + u, v[u]);
        }
        for (; n < n_layers; n++) up(n, __ldcs(cov + (uint64_t)n * plane + p));
        // then the suffix products P, last layer first
        float P = 1.0f;
        auto down = [&](uint32_t n, float v, float en) {
            const float4 k = clr[n];
            if (keep(v)) grad_cov[(uint64_t)n * plane + p] = P * ((g.x * k.x + g.y * k.y + g.z * k.z + g.w * k.w) - k.w * en);
            P *= 1.0f - k.w * v;
        };
        uint32_t m = n_layers;
        for (; m >= SB; m -= SB) {
            float v[SB], en[SB];
#pragma unroll
            for (int u = 0; u < SB; u++) v[u] = __ldcs(cov + (uint64_t)(m - 1 - u) * plane + p);
#pragma unroll
            for (int u = 0; u < SB; u++) en[u] = keep(v[u]) ? grad_cov[(uint64_t)(m - 1 - u) * plane + p] : 0.0f;
#pragma unroll
            for (int u = 0; u < SB; u++) down(m - 1 - u, v[u], en[u]);
        }
        for (; m > 0; m--) {
            const float v = __ldcs(cov + (uint64_t)(m - 1) * plane + p);
            down(m - 1, v, keep(v) ? grad_cov[(uint64_t)(m - 1) * plane + p] : 0.0f);
        }
        if (grad_init) grad_init[p] = make_float4(g.x * P, g.y * P, g.z * P, g.w * P);
    }
}

cudaError_t launch_srcover(bool backward, const float* cov, uint32_t n_layers, uint64_t plane, const float4* clr,
                           const float4* init, float4* out, const float4* grad_out, float* grad_cov,
                           float4* grad_init, uint32_t n_px, int grid, cudaStream_t s, bool partial) {
    if (backward && partial)
        k_srcover_bwd<true><<<grid, 256, 0, s>>>(cov, n_layers, plane, clr, init, grad_out, grad_cov, grad_init, n_px);
    else if (backward)
        k_srcover_bwd<false><<<grid, 256, 0, s>>>(cov, n_layers, plane, clr, init, grad_out, grad_cov, grad_init, n_px);
    else
        k_srcover_fwd<<<grid, 256, 0, s>>>(cov, n_layers, plane, clr, init, out, n_px);
    return cudaGetLastError();
}

}  // namespace ftc
