// Device-side helpers shared by the kernels (header-only; each .cu is its own module).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "pfg_internal.cuh"

namespace pfg {

constexpr int BLOCK = 256;

__host__ __device__ inline int div_up(long long a, int b) { return (int)((a + b - 1) / b); }

// Element geometry from node positions, in FP64, with the reference's closed forms
// (Element::computeJ / computeDetJ / computeInvJ, srcs/mesh/Element.cpp:15-135).
template <int DIM>
struct Geom {
    double J[DIM][DIM];
    double invJ[DIM][DIM];
    double detJ;
};

template <int DIM>
__device__ __forceinline__ void compute_geom(const double* __restrict__ pos, int N, const int (&nd)[DIM + 1],
                                             Geom<DIM>& g) {
    if constexpr (DIM == 2) {
        const double x0 = pos[nd[0]], x1 = pos[nd[1]], x2 = pos[nd[2]];
        const double y0 = pos[N + nd[0]], y1 = pos[N + nd[1]], y2 = pos[N + nd[2]];
        g.J[0][0] = x1 - x0;
        g.J[0][1] = x2 - x0;
        g.J[1][0] = y1 - y0;
        g.J[1][1] = y2 - y0;
        g.detJ = g.J[0][0] * g.J[1][1] - g.J[1][0] * g.J[0][1];
        const double d = g.detJ;
        g.invJ[0][0] = g.J[1][1] / d;
        g.invJ[0][1] = -g.J[0][1] / d;
        g.invJ[1][0] = -g.J[1][0] / d;
        g.invJ[1][1] = g.J[0][0] / d;
    } else {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const double o = pos[(size_t)r * N + nd[0]];
#pragma unroll
            for (int c = 0; c < 3; ++c) g.J[r][c] = pos[(size_t)r * N + nd[c + 1]] - o;
        }
        const auto& J = g.J;
        g.detJ = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1]
               - J[2][0] * J[1][1] * J[0][2] - J[2][1] * J[1][2] * J[0][0] - J[2][2] * J[1][0] * J[0][1];
        const double d = g.detJ;
        g.invJ[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / d;
        g.invJ[0][1] = (J[2][1] * J[0][2] - J[2][2] * J[0][1]) / d;
        g.invJ[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
        g.invJ[1][0] = (J[2][0] * J[1][2] - J[1][0] * J[2][2]) / d;
        g.invJ[1][1] = (J[0][0] * J[2][2] - J[2][0] * J[0][2]) / d;
        g.invJ[1][2] = (J[1][0] * J[0][2] - J[0][0] * J[1][2]) / d;
        g.invJ[2][0] = (J[1][0] * J[2][1] - J[2][0] * J[1][1]) / d;
        g.invJ[2][1] = (J[2][0] * J[0][1] - J[0][0] * J[2][1]) / d;
        g.invJ[2][2] = (J[0][0] * J[1][1] - J[1][0] * J[0][1]) / d;
    }
}

// Shape-function gradients gradN[f][i] = dN_i/dx_f (MatrixBuilder::getGradN,
// srcs/simulation/matricesBuilder/MatricesBuilder.inl:92-127).
template <int DIM>
__device__ __forceinline__ void grad_n(const Geom<DIM>& g, double (&G)[DIM][DIM + 1]) {
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        double s = 0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) s += g.invJ[k][f];
        G[f][0] = -s;
#pragma unroll
        for (int k = 0; k < DIM; ++k) G[f][k + 1] = g.invJ[k][f];
    }
}

template <int DIM>
__device__ __forceinline__ void load_nodes(const int* __restrict__ conn, int E, int e, int (&nd)[DIM + 1]) {
#pragma unroll
    for (int k = 0; k <= DIM; ++k) nd[k] = __ldg(conn + (size_t)k * E + e);
}

// Block-wide sum of one double per thread; result valid in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = 0;
    if (wid == 0) {
        v = lane < NT / 32 ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    __syncthreads();
    return v;
}

template <int NT>
__device__ __forceinline__ double block_min(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = 1.0e308;
    if (wid == 0) {
        v = lane < NT / 32 ? sh[lane] : 1.0e308;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    __syncthreads();
    return v;
}

template <int NT>
__device__ __forceinline__ double block_max(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = -1.0e308;
    if (wid == 0) {
        v = lane < NT / 32 ? sh[lane] : -1.0e308;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    __syncthreads();
    return v;
}

// Deterministic grid reduction: every block writes its partial, the last block to finish
// (atomic ticket) sums the partials in block order and resets the ticket.  `out` receives
// the total.  Must be called by all threads of the block.
template <int NT>
__device__ __forceinline__ bool grid_sum_last(double v, double* partials, unsigned* ticket, double* sh,
                                              double* out) {
    v = block_sum<NT>(v, sh);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v;
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += NT) s += ((volatile double*)partials)[i];
    s = block_sum<NT>(s, sh);
    if (threadIdx.x == 0) {
        *out = s;
        *ticket = 0u;
    }
    return true;
}

}  // namespace pfg
