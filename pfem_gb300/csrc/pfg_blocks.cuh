// Node-pair block products shared by the mixed incompressible Krylov solver (pfg_pspg_mixed.cu)
// and the multigrid preconditioner (pfg_mg.cu).  Header-only device code.
//
// Layout: the scaled system is stored as one (d+1)x(d+1) block per node pair p = (n, m) of the
// adjacency, p = nbr_ptr[n] + rank of m in n's sorted neighbour list, row-major inside the block
// (k_mx_scale_bsr): in FP32 for the Krylov products and, for the multigrid's level-0 sweeps, a
// bfloat16 copy (FP32 range, 8-bit significand; accumulation stays FP32) whose rows are padded
// to four values (bf16_stride), so every row is one 8-byte load.

// bfloat16 values per block of the copy: B rows of 4 (3D: the 4x4 block itself)
template <int B>
constexpr int bf16_stride() {
    return B * 4;
}
#pragma once

#include "pfg_device.cuh"

namespace pfg {

// Lanes per node of the node-row products (mean valence ~7 in 2D, ~15 in 3D) and the threads
// of a segment kernel: one pass over the segment's NB nodes.
template <int DIM>
constexpr int node_lanes() {
    return DIM == 2 ? 4 : 8;
}

// FP32 block row of node n times x over GN lanes: sum over n's neighbours m of blk(n,m) x_m,
// with the blocks of the node-pair layout (k_mx_scale_bsr); 3D blocks are read as 4 float4.
template <int DIM, int GN>
__device__ __forceinline__ void block_row_f32(int n, bool act, int N, const int* __restrict__ nbr_ptr,
                                              const int* __restrict__ nbr, const float* __restrict__ blk,
                                              const float* __restrict__ x, int lane, float (&y)[DIM + 1]) {
    constexpr int B = DIM + 1;
#pragma unroll
    for (int f = 0; f < B; ++f) y[f] = 0;
    const int b0 = act ? nbr_ptr[n] : 0;
    const int b1 = act ? nbr_ptr[n + 1] : 0;
    for (int p = b0 + lane; p < b1; p += GN) {
        const int mn = __ldg(nbr + p);
        float xm[B];
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) xm[f2] = __ldg(x + (size_t)f2 * N + mn);
        if constexpr (B == 4) {
            const float4* a4 = reinterpret_cast<const float4*>(blk + (size_t)p * 16);
#pragma unroll
            for (int f1 = 0; f1 < 4; ++f1) {
                const float4 a = __ldg(a4 + f1);
                y[f1] += a.x * xm[0] + a.y * xm[1] + a.z * xm[2] + a.w * xm[3];
            }
        } else {
            const float* a = blk + (size_t)p * B * B;
#pragma unroll
            for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
                for (int f2 = 0; f2 < B; ++f2) y[f1] += __ldg(a + f1 * B + f2) * xm[f2];
        }
    }
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int o = GN / 2; o > 0; o >>= 1) y[f1] += __shfl_xor_sync(0xffffffffu, y[f1], o, GN);
}

// bfloat16 (stored as its 16 bits) -> FP32: the upper half of an FP32 bit pattern
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// The same block-row product with the bfloat16 copy of the blocks: 3D blocks are 32 bytes, read
// as two 16-byte loads; 2D blocks are three padded rows of 8 bytes.  The iterate comes from a
// functor, xf.load(m, v) filling v with the d+1 values at node m, so a multigrid sweep can read
// a prolonged coarse correction directly.
template <int DIM, int GN, class XF>
__device__ __forceinline__ void block_row_bf16(int n, bool act, const int* __restrict__ nbr_ptr,
                                               const int* __restrict__ nbr, const uint16_t* __restrict__ blk,
                                               const XF& xf, int lane, float (&y)[DIM + 1]) {
    constexpr int B = DIM + 1;
#pragma unroll
    for (int f = 0; f < B; ++f) y[f] = 0;
    const int b0 = act ? nbr_ptr[n] : 0;
    const int b1 = act ? nbr_ptr[n + 1] : 0;
    for (int p = b0 + lane; p < b1; p += GN) {
        const int mn = __ldg(nbr + p);
        float xm[B];
        xf.load(mn, xm);
        if constexpr (B == 4) {
            const uint4* a4 = reinterpret_cast<const uint4*>(blk + (size_t)p * 16);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint4 w = __ldg(a4 + h);  // rows 2h and 2h + 1
                y[2 * h] += bf16_lo(w.x) * xm[0] + bf16_hi(w.x) * xm[1] + bf16_lo(w.y) * xm[2] + bf16_hi(w.y) * xm[3];
                y[2 * h + 1] +=
                    bf16_lo(w.z) * xm[0] + bf16_hi(w.z) * xm[1] + bf16_lo(w.w) * xm[2] + bf16_hi(w.w) * xm[3];
            }
        } else {
            const uint2* a2 = reinterpret_cast<const uint2*>(blk + (size_t)p * bf16_stride<B>());
#pragma unroll
            for (int f1 = 0; f1 < B; ++f1) {
                const uint2 w = __ldg(a2 + f1);  // row f1: (a0, a1 | a2, pad)
                y[f1] += bf16_lo(w.x) * xm[0] + bf16_hi(w.x) * xm[1] + bf16_lo(w.y) * xm[2];
            }
        }
    }
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int o = GN / 2; o > 0; o >>= 1) y[f1] += __shfl_xor_sync(0xffffffffu, y[f1], o, GN);
}

}  // namespace pfg
