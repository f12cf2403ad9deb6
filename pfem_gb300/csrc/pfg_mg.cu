// Node-aggregation multigrid: the preconditioner of the FP32 correction solves of the mixed
// incompressible form.
//
// The reference solves each Picard system with a sparse LU (MomContEquation.hpp:11).  On the
// GPU the solve is Krylov, and with the node-block Jacobi preconditioner its iteration count
// grows with the mesh (the pressure block is a discrete Laplacian): hundreds of iterations on
// 3D meshes, thousands on fine 2D columns.  One V-cycle of this multigrid replaces the block
// Jacobi apply and makes the count nearly mesh independent.
//
// Hierarchy (built on the host once per mesh upload, from the node adjacency only):
//   * level 0 is the assembled system: the scaled values S A S in node-pair blocks, read by the
//     sweeps from a bfloat16 copy (half the bytes of FP32; a smoother needs no more digits,
//     and the Krylov products keep the FP32 blocks);
//   * each coarser level aggregates the nodes of the finer one: greedy, in node order, a node
//     whose neighbours are all unaggregated starts an aggregate with them; every node left
//     joins the aggregate of its first aggregated neighbour.  Nodes without neighbours (free
//     nodes) take no part: only the smoother acts on them.  Aggregates follow the adjacency,
//     so they never join two instances of a batch;
//   * prolongation is piecewise constant per aggregate and per field (P = aggregate indicator
//     (x) I_{d+1}), so the Galerkin operator P^T A P sums the (d+1)^2 blocks of the fine node
//     pairs (i, j) into the block of (agg i, agg j): a fixed gather list per coarse block,
//     summed in ascending fine-block order (deterministic, no atomics);
//   * coarsening stops when a level is block diagonal (every connected component, i.e. every
//     instance, is one aggregate): its block inverse is the exact coarse solve.
// Coarse levels are stored as block CSR with node-major (d+1)-vectors.
//
// Cycle: V(0,2) in 2D, V(1,1) in 3D, with damped node-block Jacobi (omega = 0.7 in 2D, 0.55 in
// 3D) on every level; the block
// inverses are computed in FP64 from the FP32 blocks (the PSPG block's Schur complement cancels
// heavily) and stored in FP32.  The values are refreshed after every assembly (one gather pass
// over the FP32 matrix plus the coarse levels).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "pfg_blocks.cuh"
#include "pfg_device.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

// Damping of the block-Jacobi smoother, by block size (d+1): the 3D blocks need more damping
// (at 0.6 the smoother already amplifies some modes of a 3D PSPG system; 0.55 took 9% fewer
// Krylov iterations than 0.5 on the 3D dam break).  In 2D 0.9 took the fewest iterations on dam
// breaks but stalled the mixed solves of sloshing tanks, so 2D keeps 0.7.
__host__ __device__ constexpr float mg_omega(int B) { return B == 3 ? 0.7f : 0.55f; }

// ---- level 0 (field-major CSR) ---------------------------------------------------------------

// Iterate readers for the sweeps.  X0/XB: the current iterate (level 0 field-major, coarse
// levels node-major).  P0/PB: the prolonged coarse correction P xc, the iterate right after the
// coarse-grid correction (the cycle has no pre-smoothing, so the iterate is zero before it).
template <int B>
struct X0 {
    const float* x;
    int N;
    __device__ __forceinline__ void load(int m, float (&v)[B]) const {
#pragma unroll
        for (int f = 0; f < B; ++f) v[f] = __ldg(x + (size_t)f * N + m);
    }
};
template <int B>
struct XB {
    const float* x;
    __device__ __forceinline__ void load(int m, float (&v)[B]) const {
#pragma unroll
        for (int f = 0; f < B; ++f) v[f] = x[(size_t)m * B + f];
    }
};
template <int B>
struct PC {
    const int* agg;
    const float* xc;
    __device__ __forceinline__ void load(int m, float (&v)[B]) const {
        const int I = agg[m];
#pragma unroll
        for (int f = 0; f < B; ++f) v[f] = I >= 0 ? xc[(size_t)I * B + f] : 0.0f;
    }
};

// x + P xc: the pre-smoothed iterate plus the prolonged coarse correction (V(1,1) cycles)
template <int B, bool FIELD_MAJOR>
struct XPC {
    const float* x;
    int N;
    const int* agg;
    const float* xc;
    __device__ __forceinline__ void load(int m, float (&v)[B]) const {
        const int I = agg[m];
#pragma unroll
        for (int f = 0; f < B; ++f) {
            const float xv = FIELD_MAJOR ? __ldg(x + (size_t)f * N + m) : x[(size_t)m * B + f];
            v[f] = I >= 0 ? xv + xc[(size_t)I * B + f] : xv;
        }
    }
};

// Lanes per aggregate of the restrictions: aggregates hold ~7 (2D) to ~20 (3D) members, and a
// single thread summing them is a chain of dependent loads.
constexpr int RL = 8;

// x = omega Binv b, the first sweep from a zero iterate (V(1,1) cycles); x = Binv b, the exact
// solve, for a node without neighbours
template <int DIM>
__global__ void k_mg0_smooth0(int N, const int* __restrict__ nbr_ptr, const float* __restrict__ binv,
                              const float* __restrict__ b, float* __restrict__ x) {
    constexpr int B = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const float w = nbr_ptr[n + 1] - nbr_ptr[n] == 1 ? 1.0f : mg_omega(B);
    float v[B];
#pragma unroll
    for (int f = 0; f < B; ++f) v[f] = b[(size_t)f * N + n];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        float s = 0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) s += binv[(size_t)(f1 * B + f2) * N + n] * v[f2];
        x[(size_t)f1 * N + n] = w * s;
    }
}

// r = b - A x at level 0 (V(1,1) cycles), x read through xf
template <int DIM, int GN, class XF>
__global__ void __launch_bounds__(256) k_mg0_resid(int N, const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                                                   const uint16_t* __restrict__ blk, const float* __restrict__ b, XF xf,
                                                   float* __restrict__ r) {
    constexpr int B = DIM + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = t / GN, lane = t % GN;
    const bool act = n < N;
    float y[B];
    block_row_bf16<DIM, GN>(act ? n : 0, act, nbr_ptr, nbr, blk, xf, lane, y);
    if (!act || lane != 0) return;
#pragma unroll
    for (int f = 0; f < B; ++f) r[(size_t)f * N + n] = b[(size_t)f * N + n] - y[f];
}

// One smoothing sweep at level 0, node n over GN lanes: out_n = x_n + omega Binv_n (b - A x)_n,
// the iterate x read through xf.  A node without neighbours is solved exactly: out_n = Binv_n b_n.
template <int DIM, int GN, class XF>
__global__ void __launch_bounds__(256) k_mg0_post(int N, const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                                                  const uint16_t* __restrict__ blk, const float* __restrict__ binv,
                                                  const float* __restrict__ b, XF xf, float* __restrict__ out) {
    constexpr int B = DIM + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = t / GN, lane = t % GN;
    const bool act = n < N;
    float y[B];
    block_row_bf16<DIM, GN>(act ? n : 0, act, nbr_ptr, nbr, blk, xf, lane, y);
    if (!act || lane != 0) return;
    const bool lone = nbr_ptr[n + 1] - nbr_ptr[n] == 1;
    float xn[B], r[B];
    xf.load(n, xn);
#pragma unroll
    for (int f = 0; f < B; ++f) {
        const float bv = b[(size_t)f * N + n];
        r[f] = lone ? bv : bv - y[f];
    }
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        float s = 0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) s += binv[(size_t)(f1 * B + f2) * N + n] * r[f2];
        out[(size_t)f1 * N + n] = lone ? s : xn[f1] + mg_omega(B) * s;
    }
}

// bc[I] = sum over the members n of aggregate I of r[n] (level 0: field-major r); RL lanes per
// aggregate, strided over the members, then a fixed shuffle tree.
template <int DIM>
__global__ void k_mg0_restrict(int nc, const int* __restrict__ mem_ptr, const int* __restrict__ mem, int N,
                               const float* __restrict__ r, float* __restrict__ bc) {
    constexpr int B = DIM + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = t / RL, lane = t % RL;
    const bool act = I < nc;
    float s[B];
#pragma unroll
    for (int f = 0; f < B; ++f) s[f] = 0;
    const int q1 = act ? mem_ptr[I + 1] : 0;
    for (int q = (act ? mem_ptr[I] : 0) + lane; q < q1; q += RL) {
        const int n = mem[q];
#pragma unroll
        for (int f = 0; f < B; ++f) s[f] += r[(size_t)f * N + n];
    }
#pragma unroll
    for (int f = 0; f < B; ++f)
#pragma unroll
        for (int o = RL / 2; o > 0; o >>= 1) s[f] += __shfl_xor_sync(0xffffffffu, s[f], o, RL);
    if (act && lane == 0)
#pragma unroll
        for (int f = 0; f < B; ++f) bc[(size_t)I * B + f] = s[f];
}

// ---- coarse levels (block CSR, node-major vectors) --------------------------------------------
// Row operations as device functions, used by the one-level kernels and by the single-block
// kernel that runs the small coarse levels (k_mg_tail).

// One sweep on block row i over GN lanes (all lanes of the group call it with the same i and
// act): out_i = x_i + omega Binv_i (b - A x)_i; a row without off-diagonal blocks is solved
// exactly (out_i = Binv_i b_i).
template <int B, int GN, class XF>
__device__ __forceinline__ void post_row(int i, bool act, int lane, const int* __restrict__ bptr,
                                         const int* __restrict__ bcol, const float* __restrict__ val,
                                         const float* __restrict__ binv, const float* __restrict__ b, const XF& xf,
                                         float* __restrict__ out) {
    float y[B];
#pragma unroll
    for (int f = 0; f < B; ++f) y[f] = 0;
    const int k0 = act ? bptr[i] : 0, k1 = act ? bptr[i + 1] : 0;
    for (int k = k0 + lane; k < k1; k += GN) {
        float xj[B];
        xf.load(bcol[k], xj);
        const float* a = val + (size_t)k * B * B;
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) y[f1] += a[f1 * B + f2] * xj[f2];
    }
#pragma unroll
    for (int f = 0; f < B; ++f)
#pragma unroll
        for (int o = GN / 2; o > 0; o >>= 1) y[f] += __shfl_xor_sync(0xffffffffu, y[f], o, GN);
    if (!act || lane != 0) return;
    const bool lone = k1 - k0 == 1;
    float xi[B], r[B];
    xf.load(i, xi);
#pragma unroll
    for (int f = 0; f < B; ++f) {
        const float bv = b[(size_t)i * B + f];
        r[f] = lone ? bv : bv - y[f];
    }
    const float* bi = binv + (size_t)i * B * B;
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        float s = 0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) s += bi[f1 * B + f2] * r[f2];
        out[(size_t)i * B + f1] = lone ? s : xi[f1] + mg_omega(B) * s;
    }
}

// r_i = b_i - (A x)_i over GN lanes (V(1,1) cycles)
template <int B, int GN, class XF>
__device__ __forceinline__ void resid_row(int i, bool act, int lane, const int* __restrict__ bptr,
                                          const int* __restrict__ bcol, const float* __restrict__ val,
                                          const float* __restrict__ b, const XF& xf, float* __restrict__ r) {
    float y[B];
#pragma unroll
    for (int f = 0; f < B; ++f) y[f] = 0;
    const int k0 = act ? bptr[i] : 0, k1 = act ? bptr[i + 1] : 0;
    for (int k = k0 + lane; k < k1; k += GN) {
        float xj[B];
        xf.load(bcol[k], xj);
        const float* a = val + (size_t)k * B * B;
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) y[f1] += a[f1 * B + f2] * xj[f2];
    }
#pragma unroll
    for (int f = 0; f < B; ++f)
#pragma unroll
        for (int o = GN / 2; o > 0; o >>= 1) y[f] += __shfl_xor_sync(0xffffffffu, y[f], o, GN);
    if (!act || lane != 0) return;
#pragma unroll
    for (int f = 0; f < B; ++f) r[(size_t)i * B + f] = b[(size_t)i * B + f] - y[f];
}

// x_i = omega Binv_i b_i, the first sweep from zero (exact for a row without off-diagonal blocks)
template <int B>
__device__ __forceinline__ void smooth0_row(int i, const int* __restrict__ bptr, const float* __restrict__ binv,
                                            const float* __restrict__ b, float* __restrict__ x) {
    const float w = bptr[i + 1] - bptr[i] == 1 ? 1.0f : mg_omega(B);
    float v[B];
#pragma unroll
    for (int f = 0; f < B; ++f) v[f] = b[(size_t)i * B + f];
    const float* bi = binv + (size_t)i * B * B;
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        float s = 0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) s += bi[f1 * B + f2] * v[f2];
        x[(size_t)i * B + f1] = w * s;
    }
}

// bc_I = sum of r over aggregate I's members, RL lanes (same I and act on all lanes)
template <int B>
__device__ __forceinline__ void restrict_row(int I, bool act, int lane, const int* __restrict__ mem_ptr,
                                             const int* __restrict__ mem, const float* __restrict__ r,
                                             float* __restrict__ bc) {
    float s[B];
#pragma unroll
    for (int f = 0; f < B; ++f) s[f] = 0;
    const int q1 = act ? mem_ptr[I + 1] : 0;
    for (int q = (act ? mem_ptr[I] : 0) + lane; q < q1; q += RL) {
        const int i = mem[q];
#pragma unroll
        for (int f = 0; f < B; ++f) s[f] += r[(size_t)i * B + f];
    }
#pragma unroll
    for (int f = 0; f < B; ++f)
#pragma unroll
        for (int o = RL / 2; o > 0; o >>= 1) s[f] += __shfl_xor_sync(0xffffffffu, s[f], o, RL);
    if (act && lane == 0)
#pragma unroll
        for (int f = 0; f < B; ++f) bc[(size_t)I * B + f] = s[f];
}

// x_i = Binv_i b_i (the coarsest level, block diagonal)
template <int B>
__device__ __forceinline__ void solve_row(int i, const float* __restrict__ binv, const float* __restrict__ b,
                                          float* __restrict__ x) {
    float v[B];
#pragma unroll
    for (int f = 0; f < B; ++f) v[f] = b[(size_t)i * B + f];
    const float* bi = binv + (size_t)i * B * B;
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        float s = 0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) s += bi[f1 * B + f2] * v[f2];
        x[(size_t)i * B + f1] = s;
    }
}

template <int B, class XF>
__global__ void __launch_bounds__(256) k_mgb_post(int n, const int* __restrict__ bptr, const int* __restrict__ bcol,
                                                  const float* __restrict__ val, const float* __restrict__ binv,
                                                  const float* __restrict__ b, XF xf, float* __restrict__ out) {
    constexpr int GN = 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / GN;
    post_row<B, GN>(i < n ? i : 0, i < n, t % GN, bptr, bcol, val, binv, b, xf, out);
}

template <int B>
__global__ void k_mgb_smooth0(int n, const int* __restrict__ bptr, const float* __restrict__ binv,
                              const float* __restrict__ b, float* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) smooth0_row<B>(i, bptr, binv, b, x);
}

template <int B, class XF>
__global__ void __launch_bounds__(256) k_mgb_resid(int n, const int* __restrict__ bptr, const int* __restrict__ bcol,
                                                   const float* __restrict__ val, const float* __restrict__ b, XF xf,
                                                   float* __restrict__ r) {
    constexpr int GN = 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / GN;
    resid_row<B, GN>(i < n ? i : 0, i < n, t % GN, bptr, bcol, val, b, xf, r);
}

template <int B>
__global__ void k_mgb_restrict(int nc, const int* __restrict__ mem_ptr, const int* __restrict__ mem,
                               const float* __restrict__ r, float* __restrict__ bc) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = t / RL;
    restrict_row<B>(I < nc ? I : 0, I < nc, t % RL, mem_ptr, mem, r, bc);
}

template <int B>
__global__ void k_mgb_solve(int n, const float* __restrict__ binv, const float* __restrict__ b,
                            float* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) solve_row<B>(i, binv, b, x);
}

// The small coarse levels (at most TAIL_MAX nodes and TAIL_BYTES of blocks each) in one thread
// block: restrictions, coarsest solve and the two sweeps of every level on the way up, with a
// block barrier between the phases, instead of three launches per level whose run time is
// launch latency.  Larger levels stay with the whole GPU: one block streams only a few hundred
// GB/s.
constexpr int TAIL_MAX = 2048;
constexpr size_t TAIL_BYTES = 256 << 10;
constexpr int TAIL_LEVELS = 12;
constexpr int TAIL_THREADS = 1024;

struct TailLevel {
    int n;
    const int *bptr, *bcol;
    const float *val, *binv;
    float *b, *x, *xb;
    const int* agg;                // node -> aggregate of the next tail level
    const int *mem_ptr, *mem;      // members of the next tail level's aggregates
};

struct TailArgs {
    int T;
    int exact_last;
    TailLevel lv[TAIL_LEVELS];
};

// Cycle shape by block size: V(0,2) in 2D, V(1,1) in 3D (measured on the GPU: V(0,2) took
// C4 from 294 to 328 instance-steps/s and C1 from 75 to 92 steps/s, but raised C3's Krylov
// iterations by 13% and cost it 5%).
template <int B>
constexpr bool pre_smooth() {
    return B == 4;
}

template <int B>
__global__ void __launch_bounds__(TAIL_THREADS) k_mg_tail(TailArgs a) {
    constexpr int GN = 4;
    constexpr bool PRE = pre_smooth<B>();
    const int tid = threadIdx.x;
    for (int t = 0; t + 1 < a.T; ++t) {
        const TailLevel& L = a.lv[t];
        const TailLevel& C = a.lv[t + 1];
        if (PRE) {  // x = omega Binv b; r = b - A x into xb (free until the way up)
            for (int i = tid; i < L.n; i += TAIL_THREADS) smooth0_row<B>(i, L.bptr, L.binv, L.b, L.x);
            __syncthreads();
            for (int base = 0; base < L.n; base += TAIL_THREADS / GN) {
                const int i = base + tid / GN;
                resid_row<B, GN>(i < L.n ? i : 0, i < L.n, tid % GN, L.bptr, L.bcol, L.val, L.b, XB<B>{L.x}, L.xb);
            }
            __syncthreads();
        }
        for (int base = 0; base < C.n; base += TAIL_THREADS / RL) {
            const int I = base + tid / RL;
            restrict_row<B>(I < C.n ? I : 0, I < C.n, tid % RL, L.mem_ptr, L.mem, PRE ? L.xb : L.b, C.b);
        }
        __syncthreads();
    }
    {
        const TailLevel& Z = a.lv[a.T - 1];
        if (a.exact_last) {
            for (int i = tid; i < Z.n; i += TAIL_THREADS) solve_row<B>(i, Z.binv, Z.b, Z.xb);
        } else {  // four sweeps from zero, ping-pong xb -> x -> xb ...; the result goes to xb
            for (int i = tid; i < Z.n * B; i += TAIL_THREADS) Z.xb[i] = 0.0f;
            for (int sweep = 0; sweep < 4; ++sweep) {
                __syncthreads();
                const float* from = sweep % 2 == 0 ? Z.xb : Z.x;
                float* to = sweep % 2 == 0 ? Z.x : Z.xb;
                for (int base = 0; base < Z.n; base += TAIL_THREADS / GN) {
                    const int i = base + tid / GN;
                    post_row<B, GN>(i < Z.n ? i : 0, i < Z.n, tid % GN, Z.bptr, Z.bcol, Z.val, Z.binv, Z.b,
                                    XB<B>{from}, to);
                }
            }
        }
    }
    __syncthreads();
    for (int t = a.T - 2; t >= 0; --t) {
        const TailLevel& L = a.lv[t];
        const TailLevel& C = a.lv[t + 1];
        if (PRE) {
            for (int base = 0; base < L.n; base += TAIL_THREADS / GN) {
                const int i = base + tid / GN;
                post_row<B, GN>(i < L.n ? i : 0, i < L.n, tid % GN, L.bptr, L.bcol, L.val, L.binv, L.b,
                                XPC<B, false>{L.x, 0, L.agg, C.xb}, L.xb);
            }
        } else {
            for (int base = 0; base < L.n; base += TAIL_THREADS / GN) {
                const int i = base + tid / GN;
                post_row<B, GN>(i < L.n ? i : 0, i < L.n, tid % GN, L.bptr, L.bcol, L.val, L.binv, L.b,
                                PC<B>{L.agg, C.xb}, L.x);
            }
            __syncthreads();
            for (int base = 0; base < L.n; base += TAIL_THREADS / GN) {
                const int i = base + tid / GN;
                post_row<B, GN>(i < L.n ? i : 0, i < L.n, tid % GN, L.bptr, L.bcol, L.val, L.binv, L.b,
                                XB<B>{L.x}, L.xb);
            }
        }
        __syncthreads();
    }
}

// ---- numeric setup ------------------------------------------------------------------------------

template <int B>
__global__ void k_mg_galerkin(int nnzb, const int* __restrict__ gptr, const int* __restrict__ glist,
                              const float* __restrict__ fval, float* __restrict__ cval) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nnzb * B * B) return;
    const int k = (int)(t / (B * B)), e = (int)(t % (B * B));
    float s = 0;
    for (int q = gptr[k]; q < gptr[k + 1]; ++q) s += fval[(size_t)glist[q] * B * B + e];
    cval[t] = s;
}

// Inverse of each diagonal block, Gauss-Jordan with partial pivoting in FP64, stored in FP32.
// A singular block falls back to the inverse of its diagonal.
template <int B>
__global__ void k_mg_binv(int n, const int* __restrict__ bdiag, const float* __restrict__ val,
                          float* __restrict__ binv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* blk = val + (size_t)bdiag[i] * B * B;
    double a[B][2 * B], dg[B];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            a[f1][f2] = blk[f1 * B + f2];
            a[f1][B + f2] = f1 == f2 ? 1.0 : 0.0;
        }
        dg[f1] = a[f1][f1];
    }
    bool ok = true;
#pragma unroll
    for (int kk = 0; kk < B; ++kk) {
        int piv = kk;
        double best = fabs(a[kk][kk]);
#pragma unroll
        for (int r = kk + 1; r < B; ++r)
            if (fabs(a[r][kk]) > best) {
                best = fabs(a[r][kk]);
                piv = r;
            }
        if (best == 0.0) ok = false;
        if (piv != kk) {
#pragma unroll
            for (int j = 0; j < 2 * B; ++j) {
                const double tmp = a[kk][j];
                a[kk][j] = a[piv][j];
                a[piv][j] = tmp;
            }
        }
        const double inv = ok ? 1.0 / a[kk][kk] : 0.0;
#pragma unroll
        for (int j = 0; j < 2 * B; ++j) a[kk][j] *= inv;
#pragma unroll
        for (int r = 0; r < B; ++r) {
            if (r == kk) continue;
            const double f = a[r][kk];
#pragma unroll
            for (int j = 0; j < 2 * B; ++j) a[r][j] -= f * a[kk][j];
        }
    }
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            double v = a[f1][B + f2];
            if (!ok) v = f1 == f2 ? (dg[f1] != 0.0 ? 1.0 / dg[f1] : 1.0) : 0.0;
            binv[(size_t)i * B * B + f1 * B + f2] = (float)v;
        }
}

// ---- host: hierarchy ------------------------------------------------------------------------------

// Greedy aggregation of a graph given as CSR adjacency without self loops.  agg[i] = aggregate
// of node i or -1 (no neighbours).  Returns the number of aggregates.
int aggregate(int n, const std::vector<int>& aptr, const std::vector<int>& aidx, std::vector<int>& agg) {
    constexpr int UNSEEN = -1, LONE = -2;
    agg.assign(n, UNSEEN);
    int na = 0;
    for (int i = 0; i < n; ++i) {
        if (agg[i] != UNSEEN) continue;
        const int b = aptr[i], e = aptr[i + 1];
        if (b == e) {
            agg[i] = LONE;
            continue;
        }
        bool fresh = true;
        for (int k = b; k < e && fresh; ++k) fresh = agg[aidx[k]] == UNSEEN;
        if (!fresh) continue;
        agg[i] = na;
        for (int k = b; k < e; ++k) agg[aidx[k]] = na;
        ++na;
    }
    for (int i = 0; i < n; ++i) {
        if (agg[i] != UNSEEN) continue;
        int to = -1;
        for (int k = aptr[i]; k < aptr[i + 1] && to < 0; ++k)
            if (agg[aidx[k]] >= 0) to = agg[aidx[k]];
        agg[i] = to >= 0 ? to : na++;
    }
    for (int i = 0; i < n; ++i)
        if (agg[i] == LONE) agg[i] = -1;
    return na;
}

template <class T>
int upload(pfg_ctx* c, DBuf& buf, const std::vector<T>& h) {
    int rc = ensure(c, buf, sizeof(T) * std::max<size_t>(h.size(), 1));
    if (rc) return rc;
    if (!h.empty()) PFG_CUDA(c, cudaMemcpyAsync(buf.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, c->stream));
    return PFG_OK;
}

}  // namespace

void mg_release(pfg_ctx* c) {
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (MgLevel& l : c->mg) {
        DBuf* bufs[] = {&l.agg, &l.mem_ptr, &l.mem, &l.bptr, &l.bcol, &l.bdiag, &l.gptr,
                        &l.glist, &l.val, &l.binv, &l.x, &l.xb, &l.b};
        for (DBuf* b : bufs) {
            c->bytes_in_use -= std::min(c->bytes_in_use, b->cap);
            release(*b);
        }
    }
    c->mg.clear();
    c->n_mg = 0;
}

// Builds the coarse levels of the current mesh (host aggregation, device patterns and lists).
// Device buffers of earlier meshes are reused (grow-only).
int mg_setup(pfg_ctx* c) {
    c->n_mg = 0;
    const int N = c->N, B = c->dim + 1;
    int rc;
    if ((rc = ensure(c, c->mg_x0, sizeof(float) * (size_t)B * N))) return rc;
    // level-0 graph: the node adjacency without self (device lists, sorted)
    std::vector<int> ptr0(N + 1), idx0(c->P);
    PFG_CUDA(c, cudaMemcpyAsync(ptr0.data(), c->nbr_ptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(idx0.data(), c->nbr.p, sizeof(int) * (size_t)c->P, cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    // fine level description: block rows (with self) and block columns
    std::vector<int> fptr = ptr0, fcol = idx0;
    int fn = N;
    for (int lev = 1; lev <= 16; ++lev) {
        // adjacency without self
        std::vector<int> aptr(fn + 1, 0), aidx;
        aidx.reserve(fcol.size());
        for (int i = 0; i < fn; ++i) {
            for (int k = fptr[i]; k < fptr[i + 1]; ++k)
                if (fcol[k] != i) aidx.push_back(fcol[k]);
            aptr[i + 1] = (int)aidx.size();
        }
        if (aidx.empty()) break;  // the finer level is block diagonal: it is the coarsest
        std::vector<int> agg;
        const int nc = aggregate(fn, aptr, aidx, agg);
        if (nc >= fn) break;
        // members
        std::vector<int> mptr(nc + 1, 0), mem;
        for (int i = 0; i < fn; ++i)
            if (agg[i] >= 0) mptr[agg[i] + 1]++;
        for (int I = 0; I < nc; ++I) mptr[I + 1] += mptr[I];
        mem.resize(mptr[nc]);
        {
            std::vector<int> fill(mptr.begin(), mptr.end() - 1);
            for (int i = 0; i < fn; ++i)
                if (agg[i] >= 0) mem[fill[agg[i]]++] = i;
        }
        // coarse block pattern: aggregates adjacent through any member pair, with self
        std::vector<int> cptr(nc + 1, 0), ccol;
        {
            std::vector<int> tmp;
            for (int I = 0; I < nc; ++I) {
                tmp.clear();
                tmp.push_back(I);
                for (int q = mptr[I]; q < mptr[I + 1]; ++q) {
                    const int i = mem[q];
                    for (int k = fptr[i]; k < fptr[i + 1]; ++k) {
                        const int J = agg[fcol[k]];
                        if (J >= 0) tmp.push_back(J);
                    }
                }
                std::sort(tmp.begin(), tmp.end());
                tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
                ccol.insert(ccol.end(), tmp.begin(), tmp.end());
                cptr[I + 1] = (int)ccol.size();
            }
        }
        const int nnzb = (int)ccol.size();
        std::vector<int> cdiag(nc);
        for (int I = 0; I < nc; ++I)
            cdiag[I] = (int)(std::lower_bound(ccol.begin() + cptr[I], ccol.begin() + cptr[I + 1], I) - ccol.begin());
        // Galerkin gather lists: fine block k (row i, column fcol[k]) -> coarse block
        std::vector<int> target(fcol.size(), -1), gptr(nnzb + 1, 0), glist;
        for (int i = 0; i < fn; ++i) {
            const int I = agg[i];
            if (I < 0) continue;
            for (int k = fptr[i]; k < fptr[i + 1]; ++k) {
                const int J = agg[fcol[k]];
                if (J < 0) continue;
                const int kc = (int)(std::lower_bound(ccol.begin() + cptr[I], ccol.begin() + cptr[I + 1], J) - ccol.begin());
                target[k] = kc;
                gptr[kc + 1]++;
            }
        }
        for (int k = 0; k < nnzb; ++k) gptr[k + 1] += gptr[k];
        glist.resize(gptr[nnzb]);
        {
            std::vector<int> fill(gptr.begin(), gptr.end() - 1);
            for (size_t k = 0; k < target.size(); ++k)
                if (target[k] >= 0) glist[fill[target[k]]++] = (int)k;
        }
        if ((int)c->mg.size() < lev) c->mg.emplace_back();
        MgLevel& L = c->mg[lev - 1];
        L.n = nc;
        L.nnzb = nnzb;
        c->n_mg = lev;
        if ((rc = upload(c, L.agg, agg)) || (rc = upload(c, L.mem_ptr, mptr)) || (rc = upload(c, L.mem, mem)) ||
            (rc = upload(c, L.bptr, cptr)) || (rc = upload(c, L.bcol, ccol)) || (rc = upload(c, L.bdiag, cdiag)) ||
            (rc = upload(c, L.gptr, gptr)) || (rc = upload(c, L.glist, glist)) ||
            (rc = ensure(c, L.val, sizeof(float) * (size_t)std::max(nnzb, 1) * B * B)) ||
            (rc = ensure(c, L.binv, sizeof(float) * (size_t)nc * B * B)) ||
            (rc = ensure(c, L.x, sizeof(float) * (size_t)nc * B)) || (rc = ensure(c, L.xb, sizeof(float) * (size_t)nc * B)) ||
            (rc = ensure(c, L.b, sizeof(float) * (size_t)nc * B)))
            return rc;
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));  // host vectors go out of scope
        fptr.swap(cptr);
        fcol.swap(ccol);
        fn = nc;
    }
    return PFG_OK;
}

// Coarse values and block inverses of every level from the current FP32 level-0 matrix.
int mg_numeric(pfg_ctx* c) {
    for (int l = 0; l < c->n_mg; ++l) {
        MgLevel& L = c->mg[l];
        const long long nt = (long long)L.nnzb * (c->dim + 1) * (c->dim + 1);
        const int grid = div_up(nt, BLOCK);
        {
            // level-0 blocks are the node-pair blocks of the FP32 system; glist holds pair ids
            const float* fv = l == 0 ? ptr<float>(c->val32) : ptr<float>(c->mg[l - 1].val);
            if (c->dim == 2)
                k_mg_galerkin<3><<<grid, BLOCK, 0, c->stream>>>(L.nnzb, ptr<int>(L.gptr), ptr<int>(L.glist), fv,
                                                                ptr<float>(L.val));
            else
                k_mg_galerkin<4><<<grid, BLOCK, 0, c->stream>>>(L.nnzb, ptr<int>(L.gptr), ptr<int>(L.glist), fv,
                                                                ptr<float>(L.val));
        }
        if (c->dim == 2)
            k_mg_binv<3><<<div_up(L.n, BLOCK), BLOCK, 0, c->stream>>>(L.n, ptr<int>(L.bdiag), ptr<float>(L.val),
                                                                      ptr<float>(L.binv));
        else
            k_mg_binv<4><<<div_up(L.n, BLOCK), BLOCK, 0, c->stream>>>(L.n, ptr<int>(L.bdiag), ptr<float>(L.val),
                                                                      ptr<float>(L.binv));
    }
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

namespace {

// One cycle.  V(0,2) (2D): restrict the right-hand side down to the coarsest level, solve it
// exactly, and on the way up apply at every level the prolonged correction followed by two
// damped block-Jacobi sweeps (the first reads the prolonged correction directly).  V(1,1)
// (3D): one sweep from zero and the residual on the way down, the prolonged correction and one
// sweep on the way up.  Both read the level's matrix twice per level.
// GN0: lanes per node of the level-0 sweeps (the tuned mg_lanes)
template <int DIM, int GN0>
void vcycle(pfg_ctx* c, const float* b0, float* out0) {
    constexpr int B = DIM + 1;
    constexpr int GNB = 4;
    const int N = c->N;
    cudaStream_t s = c->stream;
    const float* binv0 = ptr<float>(c->binv32);
    float* x0 = ptr<float>(c->mg_x0);
    const int* nptr = ptr<int>(c->nbr_ptr);
    const int* nbr = ptr<int>(c->nbr);
    const uint16_t* v0 = ptr<uint16_t>(c->val16);  // level-0 sweeps read the bfloat16 blocks
    const int L = c->n_mg;
    const int g0l = div_up((long long)N * GN0, 256);
    // levels lt.. are small enough for the single-block tail
    int lt = L;
    while (lt > 0 && c->mg[lt - 1].n <= TAIL_MAX && (size_t)c->mg[lt - 1].nnzb * B * B * sizeof(float) <= TAIL_BYTES &&
           L - (lt - 1) <= TAIL_LEVELS)
        --lt;
    constexpr bool PRE = pre_smooth<B>();
    const int g0 = div_up(N, BLOCK);
    // down: restrict the right-hand side (V(0,2)) or the residual of one sweep (V(1,1), kept in
    // out0 / xb until the way up)
    {
        MgLevel& L1 = c->mg[0];
        if (PRE) {
            k_mg0_smooth0<DIM><<<g0, BLOCK, 0, s>>>(N, nptr, binv0, b0, x0);
            k_mg0_resid<DIM, GN0><<<g0l, 256, 0, s>>>(N, nptr, nbr, v0, b0, X0<B>{x0, N}, out0);
        }
        k_mg0_restrict<DIM><<<div_up((long long)L1.n * RL, BLOCK), BLOCK, 0, s>>>(
            L1.n, ptr<int>(L1.mem_ptr), ptr<int>(L1.mem), N, PRE ? out0 : b0, ptr<float>(L1.b));
    }
    const int ldown = lt < L ? lt : L - 1;  // levels below this one are handled below
    for (int l = 0; l < ldown; ++l) {
        MgLevel& A = c->mg[l];
        MgLevel& C = c->mg[l + 1];
        if (PRE) {
            k_mgb_smooth0<B><<<div_up(A.n, BLOCK), BLOCK, 0, s>>>(A.n, ptr<int>(A.bptr), ptr<float>(A.binv),
                                                                  ptr<float>(A.b), ptr<float>(A.x));
            k_mgb_resid<B><<<div_up((long long)A.n * GNB, 256), 256, 0, s>>>(
                A.n, ptr<int>(A.bptr), ptr<int>(A.bcol), ptr<float>(A.val), ptr<float>(A.b), XB<B>{ptr<float>(A.x)},
                ptr<float>(A.xb));
        }
        k_mgb_restrict<B><<<div_up((long long)C.n * RL, BLOCK), BLOCK, 0, s>>>(C.n, ptr<int>(C.mem_ptr), ptr<int>(C.mem),
                                                                               ptr<float>(PRE ? A.xb : A.b),
                                                                               ptr<float>(C.b));
    }
    MgLevel& Z = c->mg[L - 1];
    if (lt < L) {
        TailArgs ta{};
        ta.T = L - lt;
        ta.exact_last = Z.nnzb == Z.n;
        for (int t = 0; t < ta.T; ++t) {
            MgLevel& A = c->mg[lt + t];
            TailLevel& tl = ta.lv[t];
            tl.n = A.n;
            tl.bptr = ptr<int>(A.bptr);
            tl.bcol = ptr<int>(A.bcol);
            tl.val = ptr<float>(A.val);
            tl.binv = ptr<float>(A.binv);
            tl.b = ptr<float>(A.b);
            tl.x = ptr<float>(A.x);
            tl.xb = ptr<float>(A.xb);
            if (t + 1 < ta.T) {
                MgLevel& C = c->mg[lt + t + 1];
                tl.agg = ptr<int>(C.agg);
                tl.mem_ptr = ptr<int>(C.mem_ptr);
                tl.mem = ptr<int>(C.mem);
            }
        }
        k_mg_tail<B><<<1, TAIL_THREADS, 0, s>>>(ta);
    } else if (Z.nnzb == Z.n) {  // coarsest: exact block solve when block diagonal
        k_mgb_solve<B><<<div_up(Z.n, BLOCK), BLOCK, 0, s>>>(Z.n, ptr<float>(Z.binv), ptr<float>(Z.b), ptr<float>(Z.xb));
    } else {  // else four sweeps from zero, ending in xb
        const int gl = div_up((long long)Z.n * GNB, 256);
        cudaMemsetAsync(Z.xb.p, 0, sizeof(float) * (size_t)Z.n * B, s);
        for (int sweep = 0; sweep < 4; ++sweep) {
            const float* from = ptr<float>(sweep % 2 == 0 ? Z.xb : Z.x);
            float* to = ptr<float>(sweep % 2 == 0 ? Z.x : Z.xb);
            k_mgb_post<B><<<gl, 256, 0, s>>>(Z.n, ptr<int>(Z.bptr), ptr<int>(Z.bcol), ptr<float>(Z.val), ptr<float>(Z.binv),
                                             ptr<float>(Z.b), XB<B>{from}, to);
        }
    }
    // up: prolonged correction and the sweeps of every level
    for (int l = ldown - 1; l >= 0; --l) {
        MgLevel& A = c->mg[l];
        MgLevel& C = c->mg[l + 1];
        const int gl = div_up((long long)A.n * GNB, 256);
        if (PRE) {
            k_mgb_post<B><<<gl, 256, 0, s>>>(A.n, ptr<int>(A.bptr), ptr<int>(A.bcol), ptr<float>(A.val),
                                             ptr<float>(A.binv), ptr<float>(A.b),
                                             XPC<B, false>{ptr<float>(A.x), 0, ptr<int>(C.agg), ptr<float>(C.xb)},
                                             ptr<float>(A.xb));
        } else {
            k_mgb_post<B><<<gl, 256, 0, s>>>(A.n, ptr<int>(A.bptr), ptr<int>(A.bcol), ptr<float>(A.val),
                                             ptr<float>(A.binv), ptr<float>(A.b), PC<B>{ptr<int>(C.agg), ptr<float>(C.xb)},
                                             ptr<float>(A.x));
            k_mgb_post<B><<<gl, 256, 0, s>>>(A.n, ptr<int>(A.bptr), ptr<int>(A.bcol), ptr<float>(A.val),
                                             ptr<float>(A.binv), ptr<float>(A.b), XB<B>{ptr<float>(A.x)},
                                             ptr<float>(A.xb));
        }
    }
    const int* agg0 = ptr<int>(c->mg[0].agg);
    const float* xc0 = ptr<float>(c->mg[0].xb);
    if (PRE) {
        k_mg0_post<DIM, GN0><<<g0l, 256, 0, s>>>(N, nptr, nbr, v0, binv0, b0, XPC<B, true>{x0, N, agg0, xc0}, out0);
    } else {
        k_mg0_post<DIM, GN0><<<g0l, 256, 0, s>>>(N, nptr, nbr, v0, binv0, b0, PC<B>{agg0, xc0}, x0);
        k_mg0_post<DIM, GN0><<<g0l, 256, 0, s>>>(N, nptr, nbr, v0, binv0, b0, X0<B>{x0, N}, out0);
    }
}

}  // namespace

// out = M^-1 b for the FP32 scaled system (one V-cycle), both field-major R-vectors.
void mg_apply(pfg_ctx* c, const float* b, float* out) {
    const int g = c->tune.mg_lanes;
    if (c->dim == 2) {
        if (g == 2) vcycle<2, 2>(c, b, out);
        else if (g == 8) vcycle<2, 8>(c, b, out);
        else vcycle<2, 4>(c, b, out);
    } else {
        if (g == 4) vcycle<3, 4>(c, b, out);
        else if (g == 16) vcycle<3, 16>(c, b, out);
        else vcycle<3, 8>(c, b, out);
    }
}

}  // namespace pfg
