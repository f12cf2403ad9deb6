// Mixed-precision incompressible PSPG step: FP32 Krylov iterations steered by FP64 iterative
// refinement.
//
// The reference solves A(q) q = b(q) with a direct FP64 LU at every Picard iteration
// (MomContEquationPSPG.inl:281-291).  Here A and b are assembled once per Picard iteration in
// FP64 (same gather and element order as the FP64 path) together with an FP32 rounding of A,
// and one linear solve is
//     x <- x + BiCGSTAB_fp32(A32, r),  r = b - A x in FP64,  until ||r|| <= max(rel_tol ||b||, abs_tol),
// the classic mixed-precision iterative refinement: its fixed point is the FP64 system's
// solution, so the Picard iterates agree with the FP64 path to the refinement tolerance.  (An
// FP32-assembled matrix alone is not enough: rounding the C1 system to FP32 already moves its
// solution by ~7e-7 relative, and FP32 element arithmetic by ~7e-6.)  The residual evaluated
// right after a re-assembly is, at the same time, the Picard "Ax_f" residual (:366-371) and
// the first refinement residual of the next solve.
//
// Everything runs over "instances": independent meshes stored back to back in one node /
// element numbering (one instance for a single mesh).  Node-wise kernels run on segments of
// NB nodes that never straddle two instances, so every dot product and norm is reduced per
// instance, deterministically, by the last segment of that instance to finish.  Instances
// carry their own rho, mu, dt, Picard counters and Krylov scalars; converged or failed
// instances drop out of the launches while the others keep iterating.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"
#include "pfg_blocks.cuh"
#include "pfg_df.cuh"
#include "pfg_pspg_common.cuh"

namespace pfg {

namespace {

constexpr int NB = 64;           // nodes per segment (= threads of the node kernels)
constexpr int SPMV_BLOCK = 256;  // threads of the segment SpMV kernels

// per-instance int fields
// I_MODE: precision of the correction solves (0 FP32, 1 FP64); I_ROLL: undo the last sweep
// I_M64: the FP64 CSR values of the instance are current for this assembly
// I_LOOSE: the last correction solve ran at a loosened tolerance; I_TIGHT: loosening is off
// for the rest of this linear solve
enum : int {
    I_B0 = 0, I_B1, I_N0, I_N1, I_ACTIVE, I_STATUS, I_IT, I_KIT, I_TICKET, I_MODE, I_ROLL, I_M64, I_LOOSE, I_TIGHT,
    I_COUNT = 14
};
// correction-solve precision of an instance
enum : int { MODE_FP32 = 0, MODE_FP64 = 2 };
// per-instance double fields
enum : int { D_RHO = 0, D_MU, D_DT, D_RR, D_BB, D_RES, D_PAD0, D_PAD1, D_COUNT = 8 };
// per-instance Krylov scalars (one FP32 and one FP64 set)
enum : int { M_RHO = 0, M_RHO_OLD, M_ALPHA, M_OMEGA, M_RR, M_TOL2, M_DONE, M_ITERS, M_RR0, M_COUNT = 10 };
// FP32 Krylov vectors
// W_Z: the FP32 correction of an FP32 solve, added to the FP64 iterate once per sweep
enum : int { W_R = 0, W_RHAT, W_P, W_V, W_S, W_T, W_PHAT, W_SHAT, W_Z, W_COUNT };
// device counters
enum : int { C_NEED = 0, C_ACTIVE = 1, C_NEED64 = 2, C_ROLLBACK = 3 };

struct Mx {
    const int* seg;   // [3 * n_seg]: instance, first node, end node
    int* ii;          // [I_COUNT * n_inst]
    double* id;       // [D_COUNT * n_inst]
    float* sc;        // [M_COUNT * n_inst]
    double* sc64;     // [M_COUNT * n_inst]
    double* part;     // [4 * n_seg]
    int* cnt;         // [4]
    const int* node_inst;
};

struct MxConst {
    double refSize, sumw;
    PspgTables t;
    // double-float copies of the tables, refSize, sum_g w_g, 1/pi, gravity and the Boussinesq
    // factors 1 + alpha Tr and alpha; FP32 copies for the FP32 assembly
    DF mm_df[4][4], s_df[4], ref_df, hsum_df, inv_pi_df, g_df[3], bq_c0, bq_alpha;
    float mm32[4][4], s32[4], ref32;
    // p1: the tables have the P1 structure M_ij = m0 (1 + delta_ij), s_j = s (exact Gauss
    // rules), which the node kernel's right-hand side uses to sum velocities per element once
    bool p1;
    DF m0_df;
    BoussArgs bq;
    double rtol, atol, eta, min_res;
    int max_iter;
};

Mx mx_ptrs(pfg_ctx* c) {
    Mx m;
    m.seg = ptr<int>(c->mx_seg);
    m.ii = ptr<int>(c->mx_ii);
    m.id = ptr<double>(c->mx_id);
    m.sc = ptr<float>(c->mx_sc);
    m.sc64 = reinterpret_cast<double*>(ptr<char>(c->mx_sc) + 256 * (((size_t)c->n_inst * M_COUNT * sizeof(float) + 255) / 256));
    m.part = ptr<double>(c->mx_part);
    m.cnt = ptr<int>(c->mx_cnt);
    m.node_inst = ptr<int>(c->node_inst);
    return m;
}

MxConst mx_const(pfg_ctx* c) {
    const GaussConst g = gauss_const(c->dim);
    MxConst k{};
    k.refSize = g.refSize;
    k.sumw = g.sumw;
    for (int i = 0; i < 4; ++i) {
        k.t.s[i] = g.s[i];
        for (int j = 0; j < 4; ++j) k.t.MM[i][j] = g.MM[i][j];
    }
    for (int f = 0; f < 3; ++f) k.t.g[f] = c->prm.gravity[f];
    auto split = [](double d) { const float h = (float)d; return DF{h, (float)(d - (double)h)}; };
    for (int i = 0; i < 4; ++i) {
        k.s_df[i] = split(g.s[i]);
        for (int j = 0; j < 4; ++j) k.mm_df[i][j] = split(g.MM[i][j]);
    }
    k.ref_df = split(g.refSize);
    k.hsum_df = split(g.sumw);
    k.inv_pi_df = split(1.0 / M_PI);
    for (int f = 0; f < 3; ++f) k.g_df[f] = split(c->prm.gravity[f]);
    k.bq = boussinesq_args(c);
    k.bq_c0 = split(1 + k.bq.alpha * k.bq.Tr);
    k.bq_alpha = split(k.bq.alpha);
    for (int i = 0; i < 4; ++i) {
        k.s32[i] = (float)g.s[i];
        for (int j = 0; j < 4; ++j) k.mm32[i][j] = (float)g.MM[i][j];
    }
    k.ref32 = (float)g.refSize;
    const int npe = c->dim + 1;
    const double m0 = g.MM[0][1], s0 = g.s[0];
    // (the reference's 3D Gauss points carry 15 digits, so its tables have this structure to
    // ~1e-15 relative: the regrouped sums differ from the table sums by that much)
    k.p1 = m0 > 0 && s0 > 0;
    for (int i = 0; i < npe; ++i) {
        k.p1 = k.p1 && std::fabs(g.s[i] - s0) <= 1e-12 * s0;
        for (int j = 0; j < npe; ++j) k.p1 = k.p1 && std::fabs(g.MM[i][j] - (i == j ? 2.0 : 1.0) * m0) <= 1e-12 * m0;
    }
    k.m0_df = split(m0);
    k.rtol = c->prm.krylov_rel_tol;
    k.atol = c->prm.krylov_abs_tol;
    k.eta = c->prm.inner_rel_tol > 0 ? c->prm.inner_rel_tol : 1e-4;
    k.min_res = c->prm.picard_min_res;
    k.max_iter = c->prm.picard_max_iter;
    return k;
}

// Block sum in the solve's own precision (FP32 sums for the FP32 solves keep the FP64 pipe,
// 1/64 of the FP32 rate on GB300, out of the Krylov kernels).  sh: 32 values of scratch.
template <int NT, class T>
__device__ __forceinline__ T block_sum_t(T v, double* shd) {
    if constexpr (sizeof(T) == 8) {
        return block_sum<NT>(v, shd);
    } else {
        float* sh = reinterpret_cast<float*>(shd);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) sh[wid] = v;
        __syncthreads();
        v = 0;
        if (wid == 0) {
            v = lane < NT / 32 ? sh[lane] : 0.0f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        }
        __syncthreads();
        return v;
    }
}

// Per-instance deterministic reduction of NV values: each segment block writes its partials,
// the last block of the instance to arrive sums the partials of the instance's blocks in
// block order.  Returns true in the last block (totals valid in thread 0).
template <int NT, int NV, class T>
__device__ __forceinline__ bool inst_reduce(T (&v)[NV], int b, int b0, int b1, T* part, unsigned* ticket, double* sh) {
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = block_sum_t<NT, T>(v[i], sh);
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) part[(size_t)b * NV + i] = v[i];
        __threadfence();
        last = atomicAdd(ticket, 1u) == (unsigned)(b1 - b0 - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        T s = 0;
        for (int k = b0 + threadIdx.x; k < b1; k += NT) s += __ldcg(part + (size_t)k * NV + i);
        v[i] = block_sum_t<NT, T>(s, sh);
    }
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// ---- assembly --------------------------------------------------------------------------------
//
// Per Picard iteration (MomContEquationPSPG.inl:6-235 at the current iterate):
//   k_mx_prep_df element: geometry (Element.cpp:15-135), tau (:237-259) and the K factor in
//                double-float on the FP32 pipe (k_mx_prep: the same in FP64, for Bingham
//                fluids), stored as double-float in two FP32 planes (high parts, low parts);
//   k_mx_vprep   node: double-float copies of the previous velocities (and temperatures);
//   k_mx_node    node: its own (d+1)^2 block, its right-hand side in double-float, the node
//                boundary conditions, the row scales, the block inverses, the scaled diagonal
//                block of the FP32 system and ||b||^2 per instance;
//   k_mx_asm32_rows  node pair: the off-diagonal blocks of the scaled FP32 system from the
//                pair's element list, the element records of a block's rows staged in shared
//                memory (k_mx_asm32 reads them from global memory; k_mx_asm32_items is the
//                item-parallel form; the tuner picks among the three).
// The FP32 system only steers the correction solves; the refinement residual below is
// evaluated matrix-free in double-float, so it alone decides the solution.  The FP64 CSR
// values are assembled (k_mx_pairs, double-float) only for instances whose correction solves
// fell back to FP64.

// Per-instance coefficients as double-float pairs: rho, 1/dt, sum_g w_g / rho, rho/dt,
// 4 mu / rho and mu sum_g w_g (the Newtonian K factor).
enum : int { F_RHO = 0, F_INVDT = 2, F_LSUM = 4, F_CM = 6, F_MU4R = 8, F_KSUM = 10, F_COUNT = 12 };

__device__ __forceinline__ DF inst_df(const float* f32, int inst, int which) {
    return DF{f32[inst * F_COUNT + which], f32[inst * F_COUNT + which + 1]};
}

// Element data, double-float, element-major at the element's slot s (elements ordered by their
// smallest node): the 16 high parts in ah[16 s ..], the low parts in al[16 s ..], so a kernel
// that gathers an element reads two 32-byte sectors of high parts (FP32 arithmetic), plus two
// of low parts (double-float), and the elements of consecutive nodes share sectors and L2
// lines.  High and low parts are kept apart so that the FP32 gathers' L2 footprint is the high
// parts alone.
constexpr int ED_AOS = 16;
// row-staged pair assembly: pairs per block and element records staged in shared memory
constexpr int STAGE_PAIRS = 128;
constexpr int STAGE_RECORDS = 320;
constexpr int STAGE_ITEMS = 768;
struct EdPlanes {
    const float* ah;
    const float* al;
    int E;
    __device__ __forceinline__ DF gdf(int v, int s) const {
        return DF{__ldg(ah + (size_t)s * ED_AOS + v), __ldg(al + (size_t)s * ED_AOS + v)};
    }
    __device__ __forceinline__ float gf(int v, int s) const { return __ldg(ah + (size_t)s * ED_AOS + v); }
};

// Stores element e's values v (high and low parts) element-major at the element's slot.
template <int NV>
__device__ __forceinline__ void ed_store(float* __restrict__ ea, int E, int slot, const DF (&v)[NV]) {
    static_assert(NV <= ED_AOS, "element record holds 16 values");
    float rh[ED_AOS], rl[ED_AOS];
#pragma unroll
    for (int k = 0; k < ED_AOS; ++k) {
        rh[k] = k < NV ? v[k < NV ? k : 0].h : 0.0f;
        rl[k] = k < NV ? v[k < NV ? k : 0].l : 0.0f;
    }
    float4* dh = reinterpret_cast<float4*>(ea + (size_t)slot * ED_AOS);
    float4* dl = reinterpret_cast<float4*>(ea + (size_t)E * ED_AOS + (size_t)slot * ED_AOS);
#pragma unroll
    for (int k = 0; k < ED_AOS / 4; ++k) {
        dh[k] = make_float4(rh[4 * k], rh[4 * k + 1], rh[4 * k + 2], rh[4 * k + 3]);
        dl[k] = make_float4(rl[4 * k], rl[4 * k + 1], rl[4 * k + 2], rl[4 * k + 3]);
    }
}

__device__ __forceinline__ DF df_fma(DF a, DF b, DF c) { return df_add(df_mul(a, b), c); }

// Sums over the element's nodes of the previous velocities, V_f = sum_j v_jf in double-float,
// stored element-major at the element's slot as two float4 (high parts, then low parts; one
// 32-byte sector): with the P1 tables the right-hand side's mass and continuity terms of a node
// need only these sums.
template <int DIM>
__device__ __forceinline__ void elem_vsum(const DF* __restrict__ vp, int N, const int (&nd)[DIM + 1], int e,
                                          float4* __restrict__ vsum) {
    DF V[DIM];
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        V[f] = vp[(size_t)f * N + nd[0]];
#pragma unroll
        for (int j = 1; j <= DIM; ++j) V[f] = df_add(V[f], vp[(size_t)f * N + nd[j]]);
    }
    vsum[2 * (size_t)e] = make_float4(V[0].h, V[1].h, DIM == 3 ? V[DIM - 1].h : 0.0f, 0.0f);
    vsum[2 * (size_t)e + 1] = make_float4(V[0].l, V[1].l, DIM == 3 ? V[DIM - 1].l : 0.0f, 0.0f);
}

// Geometry (Element.cpp:15-135) and tau (MomContEquationPSPG.inl:237-259) of the elements of
// active instances in FP64, with the Bingham K factor: [detJ, tau, gradN, ksum] stored as
// double-float planes.
template <int DIM>
__global__ void k_mx_prep(int E, int N, const int* __restrict__ conn, const double* __restrict__ pos,
                          const double* __restrict__ q_iter, Mx m, double refSize, ViscArgs va,
                          float* __restrict__ ea, const DF* __restrict__ vp, float4* __restrict__ vsum,
                          const int* __restrict__ el_slot) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[DIM + 1];
    load_nodes<DIM>(conn, E, e, nd);
    const int inst = m.node_inst[nd[0]];
    if (!m.ii[inst * I_COUNT + I_ACTIVE]) return;
    const int slot = el_slot[e];
    elem_vsum<DIM>(vp, N, nd, slot, vsum);
    const double rho = m.id[inst * D_COUNT + D_RHO], mu = m.id[inst * D_COUNT + D_MU];
    const double dt = m.id[inst * D_COUNT + D_DT];
    Geom<DIM> g;
    compute_geom<DIM>(pos, N, nd, g);
    double G[DIM][DIM + 1];
    grad_n<DIM>(g, G);
    const double h = sqrt(refSize * g.detJ / M_PI);
    double U = 0;
#pragma unroll
    for (int k = 0; k <= DIM; ++k) {
        double nodeU = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const double v = q_iter[(size_t)d * N + nd[k]];
            nodeU += v * v;
        }
        U += sqrt(nodeU);
    }
    U /= (DIM + 1);
    const double a = 2 / dt, b = 2 * U / h, c = 4 * mu / (h * h * rho);
    const double tau = 1 / sqrt(a * a + b * b + 9 * c * c);
    double v[ed_count<DIM>()];
    v[0] = g.detJ;
    v[1] = tau;
#pragma unroll
    for (int f = 0; f < DIM; ++f)
#pragma unroll
        for (int i = 0; i <= DIM; ++i) v[2 + f * (DIM + 1) + i] = G[f][i];
    v[ed_ksum<DIM>()] = k_sum<DIM>(va, mu, G, q_iter, N, nd);
    DF dv[ed_count<DIM>()];
#pragma unroll
    for (int k = 0; k < ed_count<DIM>(); ++k) dv[k] = df_from(v[k]);
    ed_store<ed_count<DIM>()>(ea, E, slot, dv);
}

// Double-float copies of the positions and the iterate's velocities (inputs of k_mx_prep_df).
template <int DIM>
__global__ void k_mx_gprep(int N, const double* __restrict__ pos, const double* __restrict__ q_iter, Mx m,
                           DF* __restrict__ gdf) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    if (!m.ii[m.node_inst[n] * I_COUNT + I_ACTIVE]) return;
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        gdf[(size_t)f * N + n] = df_from(pos[(size_t)f * N + n]);
        gdf[(size_t)(DIM + f) * N + n] = df_from(q_iter[(size_t)f * N + n]);
    }
}

// k_mx_prep in double-float on the FP32 pipe for Newtonian fluids (the FP64 element prep is
// bound by the FP64 pipe, 1/64 of the FP32 rate on GB300): the same quantities from the same
// closed forms (Element.cpp:15-135, MomContEquationPSPG.inl:237-259), each operation an
// error-free or double-float one, so the element data agree with the FP64 ones to ~1e-14.
template <int DIM>
__global__ void k_mx_prep_df(int E, int N, const int* __restrict__ conn, const DF* __restrict__ gdf,
                             const float* __restrict__ f32, Mx m, DF ref_df, DF inv_pi, float* __restrict__ ea,
                             const DF* __restrict__ vp, float4* __restrict__ vsum, const int* __restrict__ el_slot) {
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    const int inst = m.node_inst[nd[0]];
    if (!m.ii[inst * I_COUNT + I_ACTIVE]) return;
    const int slot = el_slot[e];
    elem_vsum<DIM>(vp, N, nd, slot, vsum);
    DF X[NPE][DIM];
#pragma unroll
    for (int k = 0; k < NPE; ++k)
#pragma unroll
        for (int f = 0; f < DIM; ++f) X[k][f] = gdf[(size_t)f * N + nd[k]];
    DF J[DIM][DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int c = 0; c < DIM; ++c) J[r][c] = df_sub(X[c + 1][r], X[0][r]);
    DF det, cof[DIM][DIM];  // invJ = cof / det
    if constexpr (DIM == 2) {
        det = df_sub(df_mul(J[0][0], J[1][1]), df_mul(J[1][0], J[0][1]));
        cof[0][0] = J[1][1];
        cof[0][1] = df_neg(J[0][1]);
        cof[1][0] = df_neg(J[1][0]);
        cof[1][1] = J[0][0];
    } else {
        det = df_add(df_add(df_mul(df_mul(J[0][0], J[1][1]), J[2][2]), df_mul(df_mul(J[0][1], J[1][2]), J[2][0])),
                     df_mul(df_mul(J[0][2], J[1][0]), J[2][1]));
        det = df_sub(det, df_add(df_add(df_mul(df_mul(J[2][0], J[1][1]), J[0][2]),
                                        df_mul(df_mul(J[2][1], J[1][2]), J[0][0])),
                                 df_mul(df_mul(J[2][2], J[1][0]), J[0][1])));
        auto c2 = [&](int a, int b, int c, int d) { return df_sub(df_mul(J[a][b], J[c][d]), df_mul(J[a][d], J[c][b])); };
        cof[0][0] = c2(1, 1, 2, 2);
        cof[0][1] = c2(2, 1, 0, 2);
        cof[0][2] = c2(0, 1, 1, 2);
        cof[1][0] = c2(2, 0, 1, 2);
        cof[1][1] = c2(0, 0, 2, 2);
        cof[1][2] = c2(1, 0, 0, 2);
        cof[2][0] = c2(1, 0, 2, 1);
        cof[2][1] = c2(2, 0, 0, 1);
        cof[2][2] = c2(0, 0, 1, 1);
    }
    const DF inv_det = df_div(DF{1.0f, 0.0f}, det);
    DF G[DIM][NPE];
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        DF sum{0.0f, 0.0f};
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
            G[f][k + 1] = df_mul(cof[k][f], inv_det);
            sum = df_add(sum, G[f][k + 1]);
        }
        G[f][0] = df_neg(sum);
    }
    // tau (m_computeTauPSPG): h = sqrt(refSize detJ / pi), U = mean nodal |v| of the iterate
    const DF h = df_sqrt(df_mul(df_mul(ref_df, det), inv_pi));
    DF U{0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < NPE; ++k) {
        DF u2{0.0f, 0.0f};
#pragma unroll
        for (int f = 0; f < DIM; ++f) {
            const DF v = gdf[(size_t)(DIM + f) * N + nd[k]];
            u2 = df_add(u2, df_mul(v, v));
        }
        U = df_add(U, df_sqrt(u2));
    }
    U = df_div(U, DF{(float)NPE, 0.0f});
    const DF inv_dt = inst_df(f32, inst, F_INVDT);
    const DF a = df_add(inv_dt, inv_dt);
    const DF b = df_div(df_add(U, U), h);
    const DF c = df_div(inst_df(f32, inst, F_MU4R), df_mul(h, h));
    const DF nine{9.0f, 0.0f};
    const DF tau = df_div(DF{1.0f, 0.0f}, df_sqrt(df_add(df_add(df_mul(a, a), df_mul(b, b)), df_mul(nine, df_mul(c, c)))));
    DF dv[ed_count<DIM>()];
    dv[0] = det;
    dv[1] = tau;
#pragma unroll
    for (int f = 0; f < DIM; ++f)
#pragma unroll
        for (int i = 0; i < NPE; ++i) dv[2 + f * NPE + i] = G[f][i];
    dv[ed_ksum<DIM>()] = inst_df(f32, inst, F_KSUM);
    ed_store<ed_count<DIM>()>(ea, E, slot, dv);
}

// Double-float copies of the previous velocities and (Boussinesq) the temperatures.
template <int DIM>
__global__ void k_mx_vprep(int N, const double* __restrict__ q_prev, const double* __restrict__ T, Mx m,
                           DF* __restrict__ vp, DF* __restrict__ tdf) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    if (!m.ii[m.node_inst[n] * I_COUNT + I_ACTIVE]) return;
#pragma unroll
    for (int f = 0; f < DIM; ++f) vp[(size_t)f * N + n] = df_from(q_prev[(size_t)f * N + n]);
    if (T) tdf[n] = df_from(T[n]);
}

// One element's share of block (i, j) of the system before boundary conditions, added to acc:
// the expressions of pspg_pair_block in double-float.
template <int DIM>
__device__ __forceinline__ void pair_item_df(const EdPlanes& ed, int e, int i, int j, DF rho, DF inv_dt, DF l_sum,
                                             const MxConst& k, DF (&acc)[DIM + 1][DIM + 1]) {
    constexpr int NPE = DIM + 1;
    const DF detJ = ed.gdf(0, e);
    const DF tau = ed.gdf(1, e);
    const DF ae = df_mul(detJ, k.ref_df);
    DF gi[DIM], gj[DIM];
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        gi[f] = ed.gdf(2 + f * NPE + i, e);
        gj[f] = ed.gdf(2 + f * NPE + j, e);
    }
    DF dot = df_mul(gi[0], gj[0]);
#pragma unroll
    for (int f = 1; f < DIM; ++f) dot = df_add(dot, df_mul(gi[f], gj[f]));
    const DF mij = df_mul(inv_dt, df_mul(df_mul(rho, k.mm_df[i][j]), ae));
    const DF kf = df_mul(ae, ed.gdf(ed_ksum<DIM>(), e));
#pragma unroll
    for (int f1 = 0; f1 < DIM; ++f1) {
#pragma unroll
        for (int f2 = 0; f2 < DIM; ++f2) {
            const DF g2 = df_mul(gi[f2], gj[f1]);
            const DF kv = df_mul(kf, f1 == f2 ? df_add(dot, g2) : g2);
            acc[f1][f2] = df_add(acc[f1][f2], f1 == f2 ? df_add(mij, kv) : kv);
        }
        acc[f1][DIM] = df_add(acc[f1][DIM], df_neg(df_mul(df_mul(ae, k.s_df[j]), gi[f1])));
    }
    const DF ctau = df_mul(tau, inv_dt);
#pragma unroll
    for (int f2 = 0; f2 < DIM; ++f2) {
        const DF c1 = df_mul(ctau, df_mul(df_mul(ae, gi[f2]), k.s_df[j]));
        const DF c2 = df_mul(df_mul(ae, k.s_df[i]), gj[f2]);
        acc[DIM][f2] = df_add(acc[DIM][f2], df_add(c1, c2));
    }
    acc[DIM][DIM] = df_add(acc[DIM][DIM], df_mul(tau, df_mul(df_mul(ae, l_sum), dot)));
}

// Inverse of a (d+1)x(d+1) block by Gauss-Jordan elimination with partial pivoting in the
// block's own precision; a singular block falls back to the inverse of its diagonal.
template <int B, class T>
__device__ __forceinline__ void block_inverse(const T (&a0)[B][B], T (&inv)[B][B]) {
    T a[B][2 * B];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            a[f1][f2] = a0[f1][f2];
            a[f1][B + f2] = (f1 == f2) ? T(1) : T(0);
        }
    bool ok = true;
#pragma unroll
    for (int kk = 0; kk < B; ++kk) {
        int piv = kk;
        T best = fabs(a[kk][kk]);
#pragma unroll
        for (int i = kk + 1; i < B; ++i)
            if (fabs(a[i][kk]) > best) {
                best = fabs(a[i][kk]);
                piv = i;
            }
        if (best == T(0)) ok = false;
        // row swap through compile-time indices (keeps the block in registers)
#pragma unroll
        for (int i = kk + 1; i < B; ++i)
            if (i == piv) {
#pragma unroll
                for (int j = 0; j < 2 * B; ++j) {
                    const T t = a[kk][j];
                    a[kk][j] = a[i][j];
                    a[i][j] = t;
                }
            }
        const T inv_p = ok ? T(1) / a[kk][kk] : T(0);
#pragma unroll
        for (int j = 0; j < 2 * B; ++j) a[kk][j] *= inv_p;
#pragma unroll
        for (int i = 0; i < B; ++i) {
            if (i == kk) continue;
            const T f = a[i][kk];
#pragma unroll
            for (int j = 0; j < 2 * B; ++j) a[i][j] -= f * a[kk][j];
        }
    }
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2)
            inv[f1][f2] = ok ? a[f1][B + f2]
                             : ((f1 == f2) ? (a0[f1][f1] != T(0) ? T(1) / a0[f1][f1] : T(1)) : T(0));
}

__device__ __forceinline__ int self_rank(const int* __restrict__ nbr, int b0, int b1, int n) {
    int lo = b0, hi = b1 - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (nbr[mid] < n) lo = mid + 1;
        else hi = mid;
    }
    return lo - b0;
}

template <int B>
__device__ __forceinline__ void store_block32(float* __restrict__ blk, uint16_t* __restrict__ blk16, int p,
                                              const float (&out)[B * B]) {
    if constexpr (B == 4) {
        float4* d4 = reinterpret_cast<float4*>(blk + (size_t)p * 16);
#pragma unroll
        for (int r = 0; r < 4; ++r) d4[r] = make_float4(out[4 * r], out[4 * r + 1], out[4 * r + 2], out[4 * r + 3]);
    } else {
        float* dst = blk + (size_t)p * B * B;
#pragma unroll
        for (int e = 0; e < B * B; ++e) dst[e] = out[e];
    }
    if (blk16) {
        uint16_t h[B * 4];
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
            for (int f2 = 0; f2 < 4; ++f2)
                h[f1 * 4 + f2] = f2 < B ? __bfloat16_as_ushort(__float2bfloat16_rn(out[f1 * B + f2])) : (uint16_t)0;
        uint2* d2 = reinterpret_cast<uint2*>(blk16 + (size_t)p * bf16_stride<B>());
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
            d2[f1] = make_uint2((uint32_t)h[f1 * 4] | ((uint32_t)h[f1 * 4 + 1] << 16),
                                (uint32_t)h[f1 * 4 + 2] | ((uint32_t)h[f1 * 4 + 3] << 16));
    }
}

// Node kernel, one block per segment, one thread per node: the node's diagonal block (in the
// FP32 system's arithmetic: FP32, or double-float with DFA) and right-hand side (double-float)
// in element order, with the expressions of pspg_pair_block and pspg_node_rhs; then
// m_applyBCPSPG's node conditions (:189-232; identity rows :108-128, the Dirichlet columns of
// the node's own block zeroed), the row scales S = |a_rr|^-1/2, the FP32 inverse of the scaled
// diagonal block (the block-Jacobi smoother), the scaled diagonal block of the FP32 system and
// ||b||^2 of each instance (the relative tolerance of its linear solves).
//
// Right-hand side with the P1 tables (M_ij = m0 (1 + delta_ij), s_j = s) and no Boussinesq
// factors: for node i of element e with a_e = detJ refSize, tau_e and the element's velocity
// sums V_e (k_mx_prep*),
//   b_f = rho s g_f sum_e a_e + (rho m0 / dt) (sum_e a_e V_ef + v_if sum_e a_e)
//   b_p = hsum sum_f g_f sum_e tau_e a_e g_if + (s / dt) sum_e tau_e a_e (g_i . V_e)
// which is the element sum of F_i + (M/dt) v_prev and tau H_i + (tau/dt) C v_prev
// (MomContEquationPSPG.inl:48-96) regrouped; otherwise the element expressions term by term.
template <int DIM, bool DFA>
__global__ void __launch_bounds__(NB) k_mx_node(Mx m, int N, int E, const int* __restrict__ ne_ptr,
                                                const int* __restrict__ ne_elem, const int* __restrict__ ne_slot,
                                                const uint8_t* __restrict__ ne_loc, const int* __restrict__ conn,
                                                EdPlanes ed, const uint8_t* __restrict__ flags,
                                                const DF* __restrict__ vp, const float4* __restrict__ vsum,
                                                const DF* __restrict__ tdf,
                                                const double* __restrict__ q_prev, const double* __restrict__ vbc,
                                                const double* __restrict__ fst, const int* __restrict__ nbr_ptr,
                                                const int* __restrict__ nbr, const float* __restrict__ f32, MxConst k,
                                                double* __restrict__ rhs, double* __restrict__ scale,
                                                float* __restrict__ scale32, float* __restrict__ binv32,
                                                float* __restrict__ blk, uint16_t* __restrict__ blk16) {
    constexpr int B = DIM + 1, NPE = DIM + 1;
    __shared__ double sh[32];
    const int sb = blockIdx.x;
    const int inst = m.seg[3 * sb];
    int* ii = m.ii + inst * I_COUNT;
    if (!ii[I_ACTIVE]) return;
    const int n = m.seg[3 * sb + 1] + threadIdx.x;
    const bool act = n < m.seg[3 * sb + 2];
    const bool p1 = k.p1 && !tdf;
    double bb = 0;
    if (act) {
        if (n == ii[I_N0]) ii[I_M64] = 0;  // the FP64 CSR values (if any) predate this assembly
        const uint8_t fl = flags[n];
        const DF rho = inst_df(f32, inst, F_RHO), inv_dt = inst_df(f32, inst, F_INVDT);
        const DF l_sum = inst_df(f32, inst, F_LSUM);
        DF A[DFA ? B : 1][DFA ? B : 1], bv[DIM], bp = DF{0.0f, 0.0f};
        float A32[B][B];
#pragma unroll
        for (int a = 0; a < B; ++a)
#pragma unroll
            for (int b = 0; b < B; ++b) {
                if constexpr (DFA) A[a][b] = DF{0.0f, 0.0f};
                A32[a][b] = 0.0f;
            }
        const float cm32 = f32[inst * F_COUNT + F_CM], ct32 = f32[inst * F_COUNT + F_INVDT];
        const float l32 = f32[inst * F_COUNT + F_LSUM];
        // P1 accumulators: sum a_e, sum a_e V_e, sum tau_e a_e g_i, sum tau_e a_e (g_i . V_e)
        DF sae{0.0f, 0.0f}, av[DIM], tg[DIM], tc{0.0f, 0.0f};
#pragma unroll
        for (int f = 0; f < DIM; ++f) bv[f] = av[f] = tg[f] = DF{0.0f, 0.0f};
        const int q_begin = ne_ptr[n], q_end = ne_ptr[n + 1];
        if (!DFA && p1) {
            // the default path, software-pipelined: the next incidence's element data are loaded
            // before this incidence's arithmetic (the same operations as the loop below)
            struct Inc {
                DF ae, tau, gi[DIM];
                float ks;
                float4 vh, vl;
                int i;
            };
            auto load = [&](int q, Inc& t) {
                const int e = ne_slot[q];
                t.i = ne_loc[q];
                t.ae = ed.gdf(0, e);
                t.tau = ed.gdf(1, e);
#pragma unroll
                for (int f = 0; f < DIM; ++f) t.gi[f] = ed.gdf(2 + f * NPE + t.i, e);
                t.ks = ed.gf(ed_ksum<DIM>(), e);
                t.vh = __ldg(vsum + 2 * (size_t)e);
                t.vl = __ldg(vsum + 2 * (size_t)e + 1);
            };
            Inc nxt;
            if (q_begin < q_end) load(q_begin, nxt);
            for (int q = q_begin; q < q_end; ++q) {
                const Inc cur = nxt;
                if (q + 1 < q_end) load(q + 1, nxt);
                const int i = cur.i;
                const DF ae = df_mul(cur.ae, k.ref_df);
                const DF tau = cur.tau;
                const float a32 = ae.h, t32 = tau.h, kf = a32 * cur.ks;
                float g[DIM], dot = 0.0f;
#pragma unroll
                for (int f = 0; f < DIM; ++f) {
                    g[f] = cur.gi[f].h;
                    dot += g[f] * g[f];
                }
                const float mii = cm32 * k.mm32[i][i] * a32, as = a32 * k.s32[i];
#pragma unroll
                for (int f1 = 0; f1 < DIM; ++f1) {
#pragma unroll
                    for (int f2 = 0; f2 < DIM; ++f2) A32[f1][f2] += kf * ((f1 == f2 ? dot : 0.0f) + g[f2] * g[f1]);
                    A32[f1][f1] += mii;
                    A32[f1][DIM] -= as * g[f1];
                    A32[DIM][f1] += (t32 * ct32 + 1.0f) * as * g[f1];
                }
                A32[DIM][DIM] += t32 * a32 * l32 * dot;
                const DF V[3] = {DF{cur.vh.x, cur.vl.x}, DF{cur.vh.y, cur.vl.y}, DF{cur.vh.z, cur.vl.z}};
                const DF ta = df_mul(tau, ae);
                DF gv = df_mul(cur.gi[0], V[0]);
#pragma unroll
                for (int f = 1; f < DIM; ++f) gv = df_add(gv, df_mul(cur.gi[f], V[f]));
                sae = df_add(sae, ae);
#pragma unroll
                for (int f = 0; f < DIM; ++f) {
                    av[f] = df_add(av[f], df_mul(ae, V[f]));
                    tg[f] = df_add(tg[f], df_mul(ta, cur.gi[f]));
                }
                tc = df_add(tc, df_mul(ta, gv));
            }
        }
        for (int q = (!DFA && p1) ? q_end : q_begin; q < q_end; ++q) {
            const int e = ne_slot[q];  // element-major data are stored by slot
            const int i = ne_loc[q];
            const DF ae = df_mul(ed.gdf(0, e), k.ref_df);
            const DF tau = ed.gdf(1, e);
            DF gi[DIM];
#pragma unroll
            for (int f = 0; f < DIM; ++f) gi[f] = ed.gdf(2 + f * NPE + i, e);
            if constexpr (DFA) {
                pair_item_df<DIM>(ed, e, i, i, rho, inv_dt, l_sum, k, A);
            } else {  // pspg_pair_block's (i, i) share in FP32
                const float a32 = ae.h, t32 = tau.h, kf = a32 * ed.gf(ed_ksum<DIM>(), e);
                float g[DIM], dot = 0.0f;
#pragma unroll
                for (int f = 0; f < DIM; ++f) {
                    g[f] = gi[f].h;
                    dot += g[f] * g[f];
                }
                const float mii = cm32 * k.mm32[i][i] * a32, as = a32 * k.s32[i];
#pragma unroll
                for (int f1 = 0; f1 < DIM; ++f1) {
#pragma unroll
                    for (int f2 = 0; f2 < DIM; ++f2) A32[f1][f2] += kf * ((f1 == f2 ? dot : 0.0f) + g[f2] * g[f1]);
                    A32[f1][f1] += mii;
                    A32[f1][DIM] -= as * g[f1];
                    A32[DIM][f1] += (t32 * ct32 + 1.0f) * as * g[f1];
                }
                A32[DIM][DIM] += t32 * a32 * l32 * dot;
            }
            if (p1) {
                const float4 vh = __ldg(vsum + 2 * (size_t)e), vl = __ldg(vsum + 2 * (size_t)e + 1);
                const DF V[3] = {DF{vh.x, vl.x}, DF{vh.y, vl.y}, DF{vh.z, vl.z}};
                const DF ta = df_mul(tau, ae);
                DF gv = df_mul(gi[0], V[0]);
#pragma unroll
                for (int f = 1; f < DIM; ++f) gv = df_add(gv, df_mul(gi[f], V[f]));
                sae = df_add(sae, ae);
#pragma unroll
                for (int f = 0; f < DIM; ++f) {
                    av[f] = df_add(av[f], df_mul(ae, V[f]));
                    tg[f] = df_add(tg[f], df_mul(ta, gi[f]));
                }
                tc = df_add(tc, df_mul(ta, gv));
                continue;
            }
            int nd[NPE];
            load_nodes<DIM>(conn, E, ne_elem[q], nd);
            DF fs = k.s_df[i], hs = k.hsum_df;
            if (tdf) {  // Boussinesq factors (MomContEquation.inl:164-199)
                DF mt{0.0f, 0.0f}, st{0.0f, 0.0f};
#pragma unroll
                for (int j = 0; j < NPE; ++j) {
                    const DF Tj = tdf[nd[j]];
                    mt = df_add(mt, df_mul(k.mm_df[i][j], Tj));
                    st = df_add(st, df_mul(k.s_df[j], Tj));
                }
                fs = df_sub(df_mul(k.bq_c0, k.s_df[i]), df_mul(k.bq_alpha, mt));
                hs = df_sub(df_mul(k.bq_c0, k.hsum_df), df_mul(k.bq_alpha, st));
            }
            // momentum rows: F + (M/dt) v_prev; continuity row: tau H + (tau/dt) C v_prev
            DF mrow[NPE];
#pragma unroll
            for (int j = 0; j < NPE; ++j) mrow[j] = df_mul(inv_dt, df_mul(df_mul(rho, k.mm_df[i][j]), ae));
            DF cv{0.0f, 0.0f}, gdot{0.0f, 0.0f};
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                DF mv{0.0f, 0.0f};
                const DF ag = df_mul(ae, gi[f]);
#pragma unroll
                for (int j = 0; j < NPE; ++j) {
                    const DF vj = vp[(size_t)f * N + nd[j]];
                    mv = df_add(mv, df_mul(mrow[j], vj));
                    cv = df_add(cv, df_mul(df_mul(ag, k.s_df[j]), vj));
                }
                const DF F = df_mul(ae, df_mul(df_mul(rho, fs), k.g_df[f]));
                bv[f] = df_add(bv[f], df_add(F, mv));
                gdot = df_add(gdot, df_mul(gi[f], k.g_df[f]));
            }
            const DF H = df_mul(tau, df_mul(df_mul(ae, hs), gdot));
            bp = df_add(bp, df_add(H, df_mul(df_mul(tau, inv_dt), cv)));
        }
        if (p1) {
            const DF cm = df_mul(df_mul(rho, k.m0_df), inv_dt), rs = df_mul(rho, k.s_df[0]);
            DF hg{0.0f, 0.0f};
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                const DF mv = df_mul(cm, df_add(av[f], df_mul(sae, vp[(size_t)f * N + n])));
                bv[f] = df_add(df_mul(df_mul(rs, k.g_df[f]), sae), mv);
                hg = df_add(hg, df_mul(k.g_df[f], tg[f]));
            }
            bp = df_add(df_mul(k.hsum_df, hg), df_mul(df_mul(k.s_df[0], inv_dt), tc));
        }
        // right-hand side with the node conditions (m_applyBCPSPG :186-232)
        const bool free_n = fl & F_FREE, bound = fl & F_BOUND, dir = bound && (fl & F_DIRICHLET);
        double b[B];
#pragma unroll
        for (int f = 0; f < DIM; ++f) b[f] = df_to(bv[f]) + (fst ? fst[(size_t)f * N + n] : 0.0);
        b[DIM] = df_to(bp);
        if (free_n) {
            b[DIM] = 0.0;
            if (!bound) {
                const double dt = m.id[inst * D_COUNT + D_DT];
#pragma unroll
                for (int f = 0; f < DIM; ++f) b[f] = q_prev[(size_t)f * N + n] + dt * k.t.g[f];
            }
        }
        if (dir)
#pragma unroll
            for (int f = 0; f < DIM; ++f) b[f] = vbc[(size_t)f * N + n];
#pragma unroll
        for (int f = 0; f < B; ++f) {
            rhs[(size_t)f * N + n] = b[f];
            bb += b[f] * b[f];
        }
        // the node's own block with its identity rows and zeroed Dirichlet columns
        float a[B][B];
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) {
                float v;
                if constexpr (DFA) v = (float)df_to(A[f1][f2]);
                else v = A32[f1][f2];
                if (free_n || (bound && f1 < DIM)) v = (f1 == f2) ? 1.0f : 0.0f;
                else if (dir && f2 < DIM && f1 != f2) v = 0.0f;
                a[f1][f2] = v;
            }
        // S = |a_rr|^-1/2, correctly rounded in FP32 (the FP64 scale of the refinement is its
        // exact copy, so both precisions scale by the same numbers; no FP64 root or division)
        float s[B];
#pragma unroll
        for (int f = 0; f < B; ++f) {
            const float d = fabsf(a[f][f]);
            s[f] = d > 0.0f ? __frsqrt_rn(d) : 1.0f;
            scale[(size_t)f * N + n] = (double)s[f];
            scale32[(size_t)f * N + n] = s[f];
        }
        float sas[B][B], inv[B][B];
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) sas[f1][f2] = s[f1] * a[f1][f2] * s[f2];
        block_inverse<B>(sas, inv);
        float out[B * B];
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) {
                binv32[(size_t)(f1 * B + f2) * N + n] = inv[f1][f2];
                out[f1 * B + f2] = sas[f1][f2];
            }
        const int b0 = nbr_ptr[n];
        store_block32<B>(blk, blk16, b0 + self_rank(nbr, b0, nbr_ptr[n + 1], n), out);
    }
    double v[1] = {bb};
    if (!inst_reduce<NB, 1, double>(v, sb, ii[I_B0], ii[I_B1], m.part, reinterpret_cast<unsigned*>(ii + I_TICKET), sh))
        return;
    if (threadIdx.x == 0) m.id[inst * D_COUNT + D_BB] = v[0];
}

// One pair element item's FP32 contribution to the pair's (d+1)^2 block: element area ae, PSPG
// tau, viscosity sum ks, shape gradients gi / gj of the pair's nodes (local indices i, j).
template <int DIM>
__device__ __forceinline__ void pair_item32(int i, int j, float ae_ref, float tau, float ks, const float (&gi)[DIM],
                                            const float (&gj)[DIM], float cm, float inv_dt, float l_sum,
                                            const MxConst& k, float (&a)[DIM + 1][DIM + 1]) {
    const float ae = ae_ref * k.ref32;
    const float kf = ae * ks;
    float dot = gi[0] * gj[0];
#pragma unroll
    for (int f = 1; f < DIM; ++f) dot += gi[f] * gj[f];
    const float mij = cm * k.mm32[i][j] * ae;
    const float asj = ae * k.s32[j], asi = ae * k.s32[i];
    const float ct = tau * inv_dt;
#pragma unroll
    for (int f1 = 0; f1 < DIM; ++f1) {
#pragma unroll
        for (int f2 = 0; f2 < DIM; ++f2) a[f1][f2] += kf * ((f1 == f2 ? dot : 0.0f) + gi[f2] * gj[f1]);
        a[f1][f1] += mij;
        a[f1][DIM] -= asj * gi[f1];
        a[DIM][f1] += ct * asj * gi[f1] + asi * gj[f1];
    }
    a[DIM][DIM] += tau * ae * l_sum * dot;
}

// The row / column BCs and scales of an off-diagonal block, stored with its bfloat16 copy.
template <int DIM>
__device__ __forceinline__ void pair_finish32(int p, uint8_t fn, uint8_t fm, const float (&sn)[DIM + 1],
                                              const float (&sm)[DIM + 1], const float (&a)[DIM + 1][DIM + 1],
                                              float* __restrict__ blk, uint16_t* __restrict__ blk16) {
    constexpr int B = DIM + 1;
    const bool bound = fn & F_BOUND;
    const bool mdir = (fm & F_BOUND) && (fm & F_DIRICHLET);
    float out[B * B];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            float v = a[f1][f2];
            if ((fn & F_FREE) || (bound && f1 < DIM) || (mdir && f2 < DIM)) v = 0.0f;
            out[f1 * B + f2] = sn[f1] * v * sm[f2];
        }
    store_block32<B>(blk, blk16, p, out);
}

// Off-diagonal blocks of the scaled FP32 system, one thread per node pair p = (n, m), m != n:
// the pair's elements in ascending order (FP32 arithmetic with the element formulas of
// pspg_pair_block, or with DFA double-float arithmetic rounded once), the identity rows of
// bound nodes, the zeroed Dirichlet columns (:216-229) and the row / column scales; written as
// one (d+1)^2 block (and its bfloat16 copy).
template <int DIM, bool DFA>
__global__ void __launch_bounds__(BLOCK) k_mx_asm32(int P, int N, const int* __restrict__ pair_node,
                                                    const int* __restrict__ nbr, const int* __restrict__ pe_ptr,
                                                    const int* __restrict__ pe_item, EdPlanes ed,
                                                    const uint8_t* __restrict__ flags,
                                                    const float* __restrict__ scale32, const float* __restrict__ f32,
                                                    Mx m, MxConst k, float* __restrict__ blk,
                                                    uint16_t* __restrict__ blk16) {
    constexpr int B = DIM + 1, NPE = DIM + 1;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int n = pair_node[p];
    const int mm = nbr[p];
    if (mm == n) return;  // diagonal blocks: k_mx_node
    const int inst = m.node_inst[n];
    if (!m.ii[inst * I_COUNT + I_ACTIVE]) return;
    const uint8_t fn = flags[n], fm = flags[mm];
    float a[B][B];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) a[f1][f2] = 0.0f;
    if (DFA && !(fn & F_FREE)) {
        const DF rho = inst_df(f32, inst, F_RHO), inv_dt = inst_df(f32, inst, F_INVDT);
        const DF l_sum = inst_df(f32, inst, F_LSUM);
        DF acc[B][B];
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) acc[f1][f2] = DF{0.0f, 0.0f};
        const int k1 = pe_ptr[p + 1];
        for (int kk = pe_ptr[p]; kk < k1; ++kk) {
            const int it = __ldg(pe_item + kk);
            pair_item_df<DIM>(ed, it >> 4, (it >> 2) & 3, it & 3, rho, inv_dt, l_sum, k, acc);
        }
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) a[f1][f2] = acc[f1][f2].h + acc[f1][f2].l;
    } else if (!(fn & F_FREE)) {
        const float cm = f32[inst * F_COUNT + F_CM], inv_dt = f32[inst * F_COUNT + F_INVDT];
        const float l_sum = f32[inst * F_COUNT + F_LSUM];
        const int k0 = pe_ptr[p], k1 = pe_ptr[p + 1];
        // the element data of the next item are loaded before this item's arithmetic (two
        // items' gathers in flight per thread)
        struct Item {
            float ae, tau, ks, gi[DIM], gj[DIM];
            int i, j;
        };
        auto load = [&](int kk, Item& t) {
            const int it = __ldg(pe_item + kk);
            const int e = it >> 4;
            t.i = (it >> 2) & 3;
            t.j = it & 3;
            t.ae = ed.gf(0, e);
            t.tau = ed.gf(1, e);
            t.ks = ed.gf(ed_ksum<DIM>(), e);
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                t.gi[f] = ed.gf(2 + f * NPE + t.i, e);
                t.gj[f] = ed.gf(2 + f * NPE + t.j, e);
            }
        };
        Item nxt;
        if (k0 < k1) load(k0, nxt);
        for (int kk = k0; kk < k1; ++kk) {
            const Item cur = nxt;
            if (kk + 1 < k1) load(kk + 1, nxt);
            pair_item32<DIM>(cur.i, cur.j, cur.ae, cur.tau, cur.ks, cur.gi, cur.gj, cm, inv_dt, l_sum, k, a);
        }
    }
    float sn[B], sm[B];
#pragma unroll
    for (int f = 0; f < B; ++f) {
        sn[f] = scale32[(size_t)f * N + n];
        sm[f] = scale32[(size_t)f * N + mm];
    }
    pair_finish32<DIM>(p, fn, fm, sn, sm, a, blk, blk16);
}

// Row-staged pair assembly (the FP32 default): a block takes 128 consecutive node pairs, which
// belong to a run of consecutive rows.  Their element records (contiguous in the node-element
// incidence arrays) and their item lists (contiguous in pe_pos) are first copied into shared
// memory with independent loads; then every thread sums its pair's items from there (same
// items, order and arithmetic as k_mx_asm32, so the blocks are the same).  A block whose rows
// hold more records or items than fit reads them from global memory instead.
template <int DIM>
__global__ void __launch_bounds__(STAGE_PAIRS) k_mx_asm32_rows(int P, int N, const int* __restrict__ pair_node,
                                                               const int* __restrict__ nbr,
                                                               const int* __restrict__ pe_ptr,
                                                               const int* __restrict__ pe_pos,
                                                               const int* __restrict__ ne_ptr,
                                                               const int* __restrict__ ne_slot, EdPlanes ed,
                                                               const uint8_t* __restrict__ flags,
                                                               const float* __restrict__ scale32,
                                                               const float* __restrict__ f32, Mx m, MxConst k,
                                                               float* __restrict__ blk, uint16_t* __restrict__ blk16) {
    constexpr int B = DIM + 1, NPE = DIM + 1;
    // records at an odd stride (17 floats): the threads of a warp read the same field of
    // different records from different banks
    constexpr int RS = ED_AOS + 1;
    __shared__ float srec[STAGE_RECORDS * RS];
    __shared__ int sitem[STAGE_ITEMS];
    const int p0 = blockIdx.x * STAGE_PAIRS;
    const int pe = min(p0 + STAGE_PAIRS, P);
    const int nf = pair_node[p0], nl = pair_node[pe - 1];
    {  // a block inside one instance that no longer iterates (a batch's converged instance)
        const int i_f = m.node_inst[nf];
        if (i_f == m.node_inst[nl] && !m.ii[i_f * I_COUNT + I_ACTIVE]) return;
    }
    const int q0 = ne_ptr[nf], nrec = ne_ptr[nl + 1] - q0;
    const int i0 = pe_ptr[p0], nit = pe_ptr[pe] - i0;
    const bool rec_staged = nrec <= STAGE_RECORDS, it_staged = nit <= STAGE_ITEMS;
    // every global load of the block is issued before the barrier: the staging copies (four
    // in flight per thread) and each thread's own pair data
    if (rec_staged) {
        const float4* src = reinterpret_cast<const float4*>(ed.ah);
#pragma unroll 4
        for (int t = threadIdx.x; t < nrec * (ED_AOS / 4); t += STAGE_PAIRS) {
            const int r = t / (ED_AOS / 4), c = t % (ED_AOS / 4);
            const float4 v = __ldg(src + (size_t)__ldg(ne_slot + q0 + r) * (ED_AOS / 4) + c);
            float* d = srec + r * RS + 4 * c;
            d[0] = v.x;
            d[1] = v.y;
            d[2] = v.z;
            d[3] = v.w;
        }
    }
    if (it_staged)
#pragma unroll 4
        for (int t = threadIdx.x; t < nit; t += STAGE_PAIRS) sitem[t] = __ldg(pe_pos + i0 + t);
    const int p = p0 + threadIdx.x;
    const bool live = p < pe;
    int n = 0, mm = 0, inst = 0, kb = 0, ke = 0, base = 0, active = 0;
    uint8_t fn = F_FREE, fm = 0;
    float sn[B], sm[B], cm = 0.0f, inv_dt = 0.0f, l_sum = 0.0f;
    if (live) {
        n = pair_node[p];
        mm = nbr[p];
        kb = pe_ptr[p];
        ke = pe_ptr[p + 1];
        inst = m.node_inst[n];
        fn = flags[n];
        fm = flags[mm];
        base = ne_ptr[n] - q0;
#pragma unroll
        for (int f = 0; f < B; ++f) {
            sn[f] = scale32[(size_t)f * N + n];
            sm[f] = scale32[(size_t)f * N + mm];
        }
        active = m.ii[inst * I_COUNT + I_ACTIVE];
        cm = f32[inst * F_COUNT + F_CM];
        inv_dt = f32[inst * F_COUNT + F_INVDT];
        l_sum = f32[inst * F_COUNT + F_LSUM];
    }
    __syncthreads();
    if (!live || mm == n || !active) return;  // diagonal blocks: k_mx_node
    float a[B][B];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) a[f1][f2] = 0.0f;
    if (!(fn & F_FREE)) {
        for (int kk = kb; kk < ke; ++kk) {
            const int it = it_staged ? sitem[kk - i0] : __ldg(pe_pos + kk);
            const int r = base + (it >> 4), i = (it >> 2) & 3, j = it & 3;
            float ae, tau, ks, gi[DIM], gj[DIM];
            if (rec_staged) {
                const float* rec = srec + r * RS;
                ae = rec[0];
                tau = rec[1];
                ks = rec[ed_ksum<DIM>()];
#pragma unroll
                for (int f = 0; f < DIM; ++f) {
                    gi[f] = rec[2 + f * NPE + i];
                    gj[f] = rec[2 + f * NPE + j];
                }
            } else {
                const int e = __ldg(ne_slot + q0 + r);
                ae = ed.gf(0, e);
                tau = ed.gf(1, e);
                ks = ed.gf(ed_ksum<DIM>(), e);
#pragma unroll
                for (int f = 0; f < DIM; ++f) {
                    gi[f] = ed.gf(2 + f * NPE + i, e);
                    gj[f] = ed.gf(2 + f * NPE + j, e);
                }
            }
            pair_item32<DIM>(i, j, ae, tau, ks, gi, gj, cm, inv_dt, l_sum, k, a);
        }
    }
    pair_finish32<DIM>(p, fn, fm, sn, sm, a, blk, blk16);
}

// Off-diagonal blocks of the scaled FP32 system, item-parallel (the FP32 assembly's default):
// block c evaluates the pair element items [ASM_ITEMS c, ASM_ITEMS (c + 1)) one per thread
// (each item's (d+1)^2 FP32 contribution, the element formulas of k_mx_asm32, into shared
// memory), then the thread holding a pair's first item sums the pair's contributions in
// ascending item order (its items past the block's window evaluated by that thread directly)
// and applies the identity rows, the zeroed Dirichlet columns and the scales of k_mx_asm32.
// Every gather is issued at once per thread instead of one chain per pair.
constexpr int ASM_ITEMS = 256;

// One item's block contribution.  Every operation is an explicitly rounded intrinsic, so the
// inlined copies (shared-memory phase and the owner's items past the window) give the same
// bits: a pair's block then does not depend on where the block windows fall, and an instance
// assembled in a batch equals the instance assembled alone.
template <int DIM>
__device__ __forceinline__ void item_block32(int it, const EdPlanes& ed, const MxConst& k, float cm, float inv_dt,
                                             float l_sum, float (&c)[(DIM + 1) * (DIM + 1)]) {
    constexpr int B = DIM + 1, NPE = DIM + 1;
    const int e = it >> 4, i = (it >> 2) & 3, j = it & 3;
    const float ae = __fmul_rn(ed.gf(0, e), k.ref32);
    const float tau = ed.gf(1, e);
    const float kf = __fmul_rn(ae, ed.gf(ed_ksum<DIM>(), e));
    float gi[DIM], gj[DIM];
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        gi[f] = ed.gf(2 + f * NPE + i, e);
        gj[f] = ed.gf(2 + f * NPE + j, e);
    }
    float dot = __fmul_rn(gi[0], gj[0]);
#pragma unroll
    for (int f = 1; f < DIM; ++f) dot = __fmaf_rn(gi[f], gj[f], dot);
    const float mij = __fmul_rn(__fmul_rn(cm, k.mm32[i][j]), ae);
    const float asj = __fmul_rn(ae, k.s32[j]), asi = __fmul_rn(ae, k.s32[i]);
    const float cta = __fmul_rn(__fmul_rn(tau, inv_dt), asj);
#pragma unroll
    for (int f1 = 0; f1 < DIM; ++f1) {
#pragma unroll
        for (int f2 = 0; f2 < DIM; ++f2) {
            const float g2 = f1 == f2 ? __fmaf_rn(gi[f2], gj[f1], dot) : __fmul_rn(gi[f2], gj[f1]);
            c[f1 * B + f2] = __fmaf_rn(kf, g2, f1 == f2 ? mij : 0.0f);
        }
        c[f1 * B + DIM] = -__fmul_rn(asj, gi[f1]);
        c[DIM * B + f1] = __fmaf_rn(cta, gi[f1], __fmul_rn(asi, gj[f1]));
    }
    c[DIM * B + DIM] = __fmul_rn(__fmul_rn(__fmul_rn(tau, ae), l_sum), dot);
}

template <int DIM>
__global__ void __launch_bounds__(ASM_ITEMS) k_mx_asm32_items(long long n_items, int N,
                                                              const int* __restrict__ pair_node,
                                                              const int* __restrict__ nbr,
                                                              const int* __restrict__ pe_ptr,
                                                              const int* __restrict__ pe_item,
                                                              const int* __restrict__ pe_pair, EdPlanes ed,
                                                              const uint8_t* __restrict__ flags,
                                                              const float* __restrict__ scale32,
                                                              const float* __restrict__ f32, Mx m, MxConst k,
                                                              float* __restrict__ blk, uint16_t* __restrict__ blk16) {
    constexpr int B = DIM + 1, BB = B * B;
    __shared__ float sc[ASM_ITEMS][BB + 1];
    const long long w0 = (long long)blockIdx.x * ASM_ITEMS;
    const long long w1 = min(w0 + ASM_ITEMS, n_items);
    const int t = threadIdx.x;
    const long long it = w0 + t;
    int p = -1, n = 0, inst = 0;
    bool active = false;
    float cm = 0.0f, inv_dt = 0.0f, l_sum = 0.0f;
    if (it < w1) {
        p = pe_pair[it];
        n = pair_node[p];
        inst = m.node_inst[n];
        active = m.ii[inst * I_COUNT + I_ACTIVE] != 0;
        if (active && !(flags[n] & F_FREE)) {
            cm = f32[inst * F_COUNT + F_CM];
            inv_dt = f32[inst * F_COUNT + F_INVDT];
            l_sum = f32[inst * F_COUNT + F_LSUM];
            float c[BB];
            item_block32<DIM>(__ldg(pe_item + it), ed, k, cm, inv_dt, l_sum, c);
#pragma unroll
            for (int q = 0; q < BB; ++q) sc[t][q] = c[q];
        }
    }
    __syncthreads();
    if (p < 0 || !active) return;
    const int i0 = pe_ptr[p];
    if (it != i0) return;  // the pair's first item owns it
    const int i1 = pe_ptr[p + 1];
    const int mm = nbr[p];
    const uint8_t fn = flags[n], fm = flags[mm];
    float a[BB];
#pragma unroll
    for (int q = 0; q < BB; ++q) a[q] = 0.0f;
    if (!(fn & F_FREE)) {
        const int in_win = (int)min((long long)i1, w1) - i0;
        for (int r = 0; r < in_win; ++r)
#pragma unroll
            for (int q = 0; q < BB; ++q) a[q] = __fadd_rn(a[q], sc[t + r][q]);
        for (long long r = w1; r < i1; ++r) {  // items past the window
            float c[BB];
            item_block32<DIM>(__ldg(pe_item + r), ed, k, cm, inv_dt, l_sum, c);
#pragma unroll
            for (int q = 0; q < BB; ++q) a[q] = __fadd_rn(a[q], c[q]);
        }
    }
    const bool bound = fn & F_BOUND;
    const bool mdir = (fm & F_BOUND) && (fm & F_DIRICHLET);
    float sn[B], sm[B];
#pragma unroll
    for (int f = 0; f < B; ++f) {
        sn[f] = scale32[(size_t)f * N + n];
        sm[f] = scale32[(size_t)f * N + mm];
    }
    float out[BB];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            float v = a[f1 * B + f2];
            if ((fn & F_FREE) || (bound && f1 < DIM) || (mdir && f2 < DIM)) v = 0.0f;
            out[f1 * B + f2] = sn[f1] * v * sm[f2];
        }
    store_block32<B>(blk, blk16, p, out);
}

// FP64 CSR values of the instances whose correction solves run in FP64 (and whose values are
// not yet current for this assembly), one thread per node pair: the gather and Dirichlet
// elimination of the FP64 path, each element's share in double-float (pair_item_df).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_mx_pairs(int P, int N, int E, const int* __restrict__ pair_node,
                                                    const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                                                    const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                                                    const int* __restrict__ ne_slot,
                                                    const uint8_t* __restrict__ ne_loc, const int* __restrict__ conn,
                                                    EdPlanes ed, const uint8_t* __restrict__ flags,
                                                    const int* __restrict__ row_ptr, double* __restrict__ val,
                                                    const double* __restrict__ vbc, const float* __restrict__ f32,
                                                    Mx m, MxConst k) {
    constexpr int NPE = DIM + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P) return;
    const int n = pair_node[t];
    const int inst = m.node_inst[n];
    const int* ii = m.ii + inst * I_COUNT;
    if (!ii[I_ACTIVE] || ii[I_MODE] != MODE_FP64 || ii[I_M64]) return;
    const int b0 = nbr_ptr[n];
    const int deg = nbr_ptr[n + 1] - b0;
    const int rank = t - b0;
    const int mm = nbr[t];
    const uint8_t fn = flags[n];
    if (fn & F_FREE) {
#pragma unroll
        for (int f = 0; f <= DIM; ++f) val[row_ptr[n + f * N]] = 1.0;
        return;
    }
    const DF rho = inst_df(f32, inst, F_RHO), inv_dt = inst_df(f32, inst, F_INVDT);
    const DF l_sum = inst_df(f32, inst, F_LSUM);
    DF acc[NPE][NPE];
#pragma unroll
    for (int a = 0; a < NPE; ++a)
#pragma unroll
        for (int b = 0; b < NPE; ++b) acc[a][b] = DF{0.0f, 0.0f};
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        int j = -1;
#pragma unroll
        for (int jj = 0; jj < NPE; ++jj)
            if (__ldg(conn + (size_t)jj * E + e) == mm) j = jj;
        if (j >= 0) pair_item_df<DIM>(ed, ne_slot[q], ne_loc[q], j, rho, inv_dt, l_sum, k, acc);
    }
    double out[NPE][NPE];
#pragma unroll
    for (int a = 0; a < NPE; ++a)
#pragma unroll
        for (int b = 0; b < NPE; ++b) out[a][b] = df_to(acc[a][b]);
    pspg_write_block<DIM>(n, mm, N, deg, rank, fn, flags[mm], row_ptr, out, true, vbc, nullptr, val, nullptr);
}

// FP64 inverses of the diagonal blocks of the FP64 CSR values (block-Jacobi of the FP64
// correction solves), for the instances k_mx_pairs just assembled: identity rows (free nodes,
// velocity rows of bound nodes) hold their single diagonal entry.
template <int DIM>
__global__ void k_mx_binv64(int N, const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                            const int* __restrict__ row_ptr, const double* __restrict__ val,
                            const uint8_t* __restrict__ flags, Mx m, double* __restrict__ binv) {
    constexpr int B = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int* ii = m.ii + m.node_inst[n] * I_COUNT;
    if (!ii[I_ACTIVE] || ii[I_MODE] != MODE_FP64 || ii[I_M64]) return;
    const uint8_t fl = flags[n];
    const int b0 = nbr_ptr[n], deg = nbr_ptr[n + 1] - b0;
    const int rank = self_rank(nbr, b0, nbr_ptr[n + 1], n);
    double a[B][B], inv[B][B];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        const bool single = (fl & F_FREE) || ((fl & F_BOUND) && f1 < DIM);
        const int rp = row_ptr[n + (size_t)f1 * N];
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2)
            a[f1][f2] = single ? (f1 == f2 ? val[rp] : 0.0) : val[rp + f2 * deg + rank];
    }
    block_inverse<B>(a, inv);
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) binv[(size_t)(f1 * B + f2) * N + n] = inv[f1][f2];
}

__global__ void k_mx_mark_csr64(int n_inst, Mx m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_inst) return;
    int* ii = m.ii + i * I_COUNT;
    if (ii[I_ACTIVE] && ii[I_MODE] == MODE_FP64) ii[I_M64] = 1;
}

// ---- refinement residual, matrix-free in double-float ----------------------------------------
//
// r = b - A x with A applied element by element from the double-float element data (no FP64
// matrix): k_mx_xdf makes a double-float copy of x with the Dirichlet values in the Dirichlet
// velocity columns (b - A x over the full matrix at those values equals the eliminated system's
// residual, :216-229); k_mx_res_elem evaluates each element's A_e x for its d+1 element rows
// from element-level gradients (grad u, grad p, sums of s_j u_j) and writes one record per
// element node; k_mx_res_node sums its node's records in ascending element order and forms
// r = b - A x (identity rows: r = b - x).  Right after a re-assembly this is also the Picard
// "Ax_f" residual (:366-371).

template <int DIM>
__global__ void k_mx_xdf(int N, const double* __restrict__ x, const double* __restrict__ vbc,
                         const uint8_t* __restrict__ flags, Mx m, DF* __restrict__ xdf) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    if (!m.ii[m.node_inst[n] * I_COUNT + I_ACTIVE]) return;
    const uint8_t fl = flags[n];
    const bool dir = (fl & F_BOUND) && (fl & F_DIRICHLET);
#pragma unroll
    for (int f = 0; f <= DIM; ++f) {
        const size_t r = (size_t)f * N + n;
        xdf[r] = df_from(dir && f < DIM ? vbc[r] : x[r]);
    }
}

constexpr int RES_ELEM_BLOCK = 64;  // ~136 registers a thread: small blocks keep more warps resident

// A_e x for every element row of the element's nodes (momentum rows of bound nodes are
// identity rows and get 0): record (e, i) holds d+1 double-float values, 32 bytes.
template <int DIM>
__global__ void __launch_bounds__(RES_ELEM_BLOCK) k_mx_res_elem(int E, int N, const int* __restrict__ conn_s,
                                                                EdPlanes ed, const uint8_t* __restrict__ flags,
                                                                const DF* __restrict__ xdf, const float* __restrict__ f32,
                                                                Mx m, MxConst k, float4* __restrict__ rec) {
    constexpr int NPE = DIM + 1;
    // one thread per element slot: slot-ordered connectivity, element data and records are
    // read and written coalesced
    const int es = blockIdx.x * blockDim.x + threadIdx.x;
    if (es >= E) return;
    const int e = es;  // records are kept by slot as well
    int nd[NPE];
    load_nodes<DIM>(conn_s, E, es, nd);
    const int inst = m.node_inst[nd[0]];
    if (!m.ii[inst * I_COUNT + I_ACTIVE]) return;
    const DF inv_dt = inst_df(f32, inst, F_INVDT), l_sum = inst_df(f32, inst, F_LSUM);
    const DF cm = inst_df(f32, inst, F_CM);
    const DF ae = df_mul(ed.gdf(0, es), k.ref_df);
    const DF tau = ed.gdf(1, es);
    const DF kf = df_mul(ae, ed.gdf(ed_ksum<DIM>(), es));
    DF G[DIM][NPE];
#pragma unroll
    for (int f = 0; f < DIM; ++f)
#pragma unroll
        for (int j = 0; j < NPE; ++j) G[f][j] = ed.gdf(2 + f * NPE + j, es);
    DF u[NPE][DIM], p[NPE];
#pragma unroll
    for (int j = 0; j < NPE; ++j) {
#pragma unroll
        for (int f = 0; f < DIM; ++f) u[j][f] = xdf[(size_t)f * N + nd[j]];
        p[j] = xdf[(size_t)DIM * N + nd[j]];
    }
    // element-level sums: Gu[a][b] = sum_j dN_j/dx_b u_j[a], grad p, s-weighted sums
    DF Gu[DIM][DIM], gp[DIM], Su[DIM], Sp{0.0f, 0.0f};
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
#pragma unroll
        for (int b = 0; b < DIM; ++b) {
            DF s = df_mul(G[b][0], u[0][a]);
#pragma unroll
            for (int j = 1; j < NPE; ++j) s = df_fma(G[b][j], u[j][a], s);
            Gu[a][b] = s;
        }
        DF s = df_mul(G[a][0], p[0]);
#pragma unroll
        for (int j = 1; j < NPE; ++j) s = df_fma(G[a][j], p[j], s);
        gp[a] = s;
        DF t = df_mul(k.s_df[0], u[0][a]);
#pragma unroll
        for (int j = 1; j < NPE; ++j) t = df_fma(k.s_df[j], u[j][a], t);
        Su[a] = t;
    }
#pragma unroll
    for (int j = 0; j < NPE; ++j) Sp = df_fma(k.s_df[j], p[j], Sp);
    DF div = Gu[0][0];
#pragma unroll
    for (int a = 1; a < DIM; ++a) div = df_add(div, Gu[a][a]);
    DF sym[DIM][DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
        for (int b = 0; b < DIM; ++b) sym[a][b] = df_add(Gu[a][b], Gu[b][a]);
    const DF cma = df_mul(cm, ae);
    const DF cta = df_mul(df_mul(tau, inv_dt), ae);
    const DF tla = df_mul(df_mul(tau, ae), l_sum);
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        DF out[4];
        // continuity row: (tau/dt) C u + D u + tau L p
        DF gs = df_mul(G[0][i], Su[0]), gq = df_mul(G[0][i], gp[0]);
#pragma unroll
        for (int f = 1; f < DIM; ++f) {
            gs = df_fma(G[f][i], Su[f], gs);
            gq = df_fma(G[f][i], gp[f], gq);
        }
        out[DIM] = df_add(df_add(df_mul(cta, gs), df_mul(df_mul(ae, k.s_df[i]), div)), df_mul(tla, gq));
        if (flags[nd[i]] & F_BOUND) {
#pragma unroll
            for (int a = 0; a < DIM; ++a) out[a] = DF{0.0f, 0.0f};
        } else {
            // momentum rows: (M/dt) u + K u - D^T p
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                DF mu_ = df_mul(k.mm_df[i][0], u[0][a]);
#pragma unroll
                for (int j = 1; j < NPE; ++j) mu_ = df_fma(k.mm_df[i][j], u[j][a], mu_);
                DF ks = df_mul(G[0][i], sym[a][0]);
#pragma unroll
                for (int c = 1; c < DIM; ++c) ks = df_fma(G[c][i], sym[a][c], ks);
                out[a] = df_sub(df_add(df_mul(cma, mu_), df_mul(kf, ks)), df_mul(df_mul(ae, G[a][i]), Sp));
            }
        }
        if constexpr (DIM == 2) out[3] = DF{0.0f, 0.0f};
        float4* r = rec + ((size_t)e * NPE + i) * 2;
        r[0] = make_float4(out[0].h, out[0].l, out[1].h, out[1].l);
        r[1] = make_float4(out[2].h, out[2].l, out[3].h, out[3].l);
    }
}

// r = b - A x of the segment's nodes from the element records, then the seeds of the
// instance's next correction solve and its Picard / refinement bookkeeping.  `kind`:
//   RES_SWEEP   after a correction sweep: an FP32 sweep that did not shrink ||r|| tenfold moves
//               the instance to FP64 mode (and, if ||r|| grew, asks the host to undo it);
//   RES_PICARD  after a re-assembly: decides the instance's Picard iteration count,
//               convergence and failure (PicardAlgo.cpp:48-90);
//   RES_START   first residual of a step, or after an undo.
enum : int { RES_SWEEP = 0, RES_PICARD = 1, RES_START = 2 };

template <int DIM>
__global__ void __launch_bounds__(NB) k_mx_res_node(Mx m, int N, const int* __restrict__ ne_ptr,
                                                    const int* __restrict__ ne_slot, const uint8_t* __restrict__ ne_loc,
                                                    const float4* __restrict__ rec, const uint8_t* __restrict__ flags,
                                                    const double* __restrict__ b, const double* __restrict__ x,
                                                    const double* __restrict__ scale, MxConst k,
                                                    float* __restrict__ W, double* __restrict__ W64, size_t ld,
                                                    int kind) {
    constexpr int B = DIM + 1, NPE = DIM + 1;
    __shared__ double sh[32];
    const int blk = blockIdx.x;
    const int inst = m.seg[3 * blk];
    int* ii = m.ii + inst * I_COUNT;
    if (!ii[I_ACTIVE]) return;
    const bool fp64 = ii[I_MODE] == MODE_FP64;
    const int n = m.seg[3 * blk + 1] + threadIdx.x;
    double rr = 0, rs = 0;
    if (n < m.seg[3 * blk + 2]) {
        const uint8_t fl = flags[n];
        const bool ident_v = fl & (F_BOUND | F_FREE), ident_p = fl & F_FREE;
        DF ax[4] = {DF{0.0f, 0.0f}, DF{0.0f, 0.0f}, DF{0.0f, 0.0f}, DF{0.0f, 0.0f}};
        if (!ident_p) {
            for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
                const float4* r = rec + ((size_t)__ldg(ne_slot + q) * NPE + __ldg(ne_loc + q)) * 2;
                const float4 r0 = __ldg(r), r1 = __ldg(r + 1);
                ax[0] = df_add(ax[0], DF{r0.x, r0.y});
                ax[1] = df_add(ax[1], DF{r0.z, r0.w});
                ax[2] = df_add(ax[2], DF{r1.x, r1.y});
                if constexpr (DIM == 3) ax[3] = df_add(ax[3], DF{r1.z, r1.w});
            }
        }
#pragma unroll
        for (int f = 0; f < B; ++f) {
            const size_t r = (size_t)f * N + n;
            const double bv = b[r];
            double rv;
            if ((f < DIM && ident_v) || (f == DIM && ident_p))
                rv = bv - x[r];
            else
                rv = df_to(df_sub(df_from(bv), ax[f]));
            if (fp64) {
                W64[W_R * ld + r] = rv;
                W64[W_RHAT * ld + r] = rv;
                W64[W_P * ld + r] = 0.0;
                W64[W_V * ld + r] = 0.0;
                rs += rv * rv;
            } else {
                const double sv = scale[r] * rv;
                const float r32 = (float)sv;
                W[W_R * ld + r] = r32;
                W[W_RHAT * ld + r] = r32;
                W[W_P * ld + r] = 0.0f;
                W[W_V * ld + r] = 0.0f;
                rs += sv * sv;
            }
            rr += rv * rv;
        }
    }
    double v[2] = {rr, rs};
    if (!inst_reduce<NB, 2, double>(v, blk, ii[I_B0], ii[I_B1], m.part, reinterpret_cast<unsigned*>(ii + I_TICKET), sh))
        return;
    if (threadIdx.x != 0) return;
    double* idd = m.id + inst * D_COUNT;
    rr = v[0];
    rs = v[1];
    const double bb = idd[D_BB];
    const double rr_prev = idd[D_RR];
    idd[D_RR] = rr;
    bool active = true;
    if (kind == RES_PICARD) {
        const double res = sqrt(rr);
        idd[D_RES] = res;
        const int it = ++ii[I_IT];
        if (res <= k.min_res) {
            ii[I_STATUS] = 1;
            active = false;
        } else if (isnan(res) || it > k.max_iter) {
            ii[I_STATUS] = 2;
            active = false;
        }
        if (!active) ii[I_ACTIVE] = 0;
    }
    const double tol = fmax(k.rtol * sqrt(bb), k.atol);
    bool need = active && rr > tol * tol;
    const int mode = ii[I_MODE];  // the mode this pass seeded for
    if (kind != RES_SWEEP) {  // a new linear solve
        ii[I_LOOSE] = 0;
        ii[I_TIGHT] = 0;
    }
    if (kind == RES_SWEEP && mode == MODE_FP32 && need && !(rr <= 0.01 * rr_prev)) {
        if (ii[I_LOOSE] && rr <= rr_prev) {
            // a loosened sweep that fell short: the rest of this solve runs at eta
            ii[I_TIGHT] = 1;
        } else {
            // an FP32 sweep that did not shrink ||r|| tenfold: FP64 from now on (and, if ||r||
            // grew, the sweep is undone and the residual recomputed after)
            ii[I_MODE] = MODE_FP64;
            if (!(rr <= rr_prev)) {
                ii[I_ROLL] = 1;
                idd[D_RR] = rr_prev;
                atomicAdd(m.cnt + C_ROLLBACK, 1);
                need = false;
            }
        }
    }
    const int nmode = ii[I_MODE];
    float* sc = m.sc + inst * M_COUNT;
    double* sc64 = m.sc64 + inst * M_COUNT;
    // seeds written this pass are valid unless the instance just crossed into FP64
    const bool need32 = need && nmode != MODE_FP64;
    const bool need64 = need && nmode == MODE_FP64 && fp64;
    // The correction solve's relative tolerance: eta, loosened for a sweep that needs less than
    // that to meet the outer test (the last sweep of a solve): 0.2 of the remaining reduction
    // tol / ||r||, at most 0.01.  A loosened sweep that misses the target and the tenfold test
    // (the FP32 operator's own error adds to its reduction) turns loosening off for the rest of
    // the solve instead of moving the instance to FP64.
    const double eta =
        need && rr > 0.0 && !ii[I_TIGHT] ? fmax(k.eta, fmin(0.01, 0.2 * tol / sqrt(rr))) : k.eta;
    ii[I_LOOSE] = eta > k.eta;
    sc[M_RHO] = (float)rs;
    sc[M_RHO_OLD] = 1.0f;
    sc[M_ALPHA] = 1.0f;
    sc[M_OMEGA] = 1.0f;
    sc[M_RR] = (float)rs;
    sc[M_RR0] = (float)rs;
    sc[M_TOL2] = (float)(eta * eta * rs);
    sc[M_ITERS] = 0.0f;
    sc[M_DONE] = need32 ? 0.0f : 1.0f;
    sc64[M_RHO] = rs;
    sc64[M_RHO_OLD] = 1.0;
    sc64[M_ALPHA] = 1.0;
    sc64[M_OMEGA] = 1.0;
    sc64[M_RR] = rs;
    sc64[M_RR0] = rs;
    sc64[M_TOL2] = eta * eta * rs;
    sc64[M_ITERS] = 0.0;
    sc64[M_DONE] = need64 ? 0.0 : 1.0;
    if (need32) atomicAdd(m.cnt + C_NEED, 1);
    if (need64) atomicAdd(m.cnt + C_NEED64, 1);
    // an instance that just moved to FP64 without an undo needs an FP64 seed: the host
    // re-evaluates the residual
    if (need && nmode == MODE_FP64 && !fp64) atomicAdd(m.cnt + C_ROLLBACK, 1);
    if (active) atomicAdd(m.cnt + C_ACTIVE, 1);
}

// ---- BiCGSTAB correction solves on segments (FP32 on S A S, or FP64 on A) --------------------
//
// One kernel set, instantiated for T = float (the scaled FP32 system, the mixed form's default)
// and T = double (the unscaled FP64 system, taken by an instance whose FP32 correction solves
// stop contracting).  Each precision has its own vectors, block inverses and per-instance
// scalars; an instance runs in exactly one of them, the other set's kernels skip it.

template <class T, int DIM>
__device__ __forceinline__ void block_apply_t(int n, int N, const T* __restrict__ binv, const T (&y)[DIM + 1],
                                              T* __restrict__ z) {
    constexpr int B = DIM + 1;
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        T s = 0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) s += binv[(size_t)(f1 * B + f2) * N + n] * y[f2];
        z[(size_t)f1 * N + n] = s;
    }
}

// Row r of the matrix times y over G lanes (valid on lane 0 of the group).
template <class T, int G>
__device__ __forceinline__ T row_dot_t(int r, bool act, const int* __restrict__ rp, const int* __restrict__ col,
                                       const T* __restrict__ val, const T* __restrict__ y, int lane) {
    const int b = act ? rp[r] : 0, e = act ? rp[r + 1] : 0;
    T s = 0;
    // four independent column/value loads in flight per lane before the dependent gathers
    int kk = b + lane;
    for (; kk + 3 * G < e; kk += 4 * G) {
        const int c0 = __ldg(col + kk), c1 = __ldg(col + kk + G), c2 = __ldg(col + kk + 2 * G),
                  c3 = __ldg(col + kk + 3 * G);
        const T v0 = __ldg(val + kk), v1 = __ldg(val + kk + G), v2 = __ldg(val + kk + 2 * G),
                v3 = __ldg(val + kk + 3 * G);
        const T y0 = __ldg(y + c0), y1 = __ldg(y + c1), y2 = __ldg(y + c2), y3 = __ldg(y + c3);
        s += v0 * y0;
        s += v1 * y1;
        s += v2 * y2;
        s += v3 * y3;
    }
    for (; kk < e; kk += G) s += __ldg(val + kk) * __ldg(y + __ldg(col + kk));
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    return s;
}

// p = r + beta (p - omega v); phat = Binv p
template <class T, int DIM>
__global__ void __launch_bounds__(NB) k_mx_up_p(Mx m, const int* __restrict__ list, T* __restrict__ scb, int N,
                                                T* __restrict__ W, size_t ld,
                                                const T* __restrict__ binv) {
    const int b = list ? list[blockIdx.x] : blockIdx.x;  // segment
    const T* sc = scb + m.seg[3 * b] * M_COUNT;
    if (sc[M_DONE] != 0) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    if (n >= m.seg[3 * b + 2]) return;
    const T beta = (sc[M_RHO] / sc[M_RHO_OLD]) * (sc[M_ALPHA] / sc[M_OMEGA]);
    const T om = sc[M_OMEGA];
    T p[DIM + 1];
#pragma unroll
    for (int f = 0; f <= DIM; ++f) {
        const size_t r = (size_t)f * N + n;
        p[f] = W[W_R * ld + r] + beta * (W[W_P * ld + r] - om * W[W_V * ld + r]);
        W[W_P * ld + r] = p[f];
    }
    block_apply_t<T, DIM>(n, N, binv, p, W + W_PHAT * ld);
}

// s = r - alpha v; shat = Binv s
template <class T, int DIM>
__global__ void __launch_bounds__(NB) k_mx_up_s(Mx m, const int* __restrict__ list, T* __restrict__ scb, int N,
                                                T* __restrict__ W, size_t ld,
                                                const T* __restrict__ binv) {
    const int b = list ? list[blockIdx.x] : blockIdx.x;  // segment
    const T* sc = scb + m.seg[3 * b] * M_COUNT;
    if (sc[M_DONE] != 0) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    if (n >= m.seg[3 * b + 2]) return;
    const T al = sc[M_ALPHA];
    T s[DIM + 1];
#pragma unroll
    for (int f = 0; f <= DIM; ++f) {
        const size_t r = (size_t)f * N + n;
        s[f] = W[W_R * ld + r] - al * W[W_V * ld + r];
        W[W_S * ld + r] = s[f];
    }
    block_apply_t<T, DIM>(n, N, binv, s, W + W_SHAT * ld);
}

// FP64 row products of node n (field-major CSR: column (m, f2) of row (n, f1) at
// row_ptr(n, f1) + f2 deg(n) + rank(m); identity rows hold their diagonal only).
template <int DIM, int GN>
__device__ __forceinline__ void node_rows_f64(int n, bool act, int N, const int* __restrict__ rp,
                                              const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                                              const double* __restrict__ val, const double* __restrict__ x,
                                              int lane, double (&y)[DIM + 1]) {
    constexpr int B = DIM + 1;
    int rowp[B];
    bool full[B];
#pragma unroll
    for (int f = 0; f < B; ++f) {
        y[f] = 0;
        rowp[f] = act ? rp[n + f * N] : 0;
        full[f] = act && (rp[n + f * N + 1] - rowp[f] > 1);
    }
    const int b0 = act ? nbr_ptr[n] : 0;
    const int deg = act ? nbr_ptr[n + 1] - b0 : 0;
    for (int k = lane; k < deg; k += GN) {
        const int mn = __ldg(nbr + b0 + k);
        double xm[B];
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) xm[f2] = __ldg(x + (size_t)f2 * N + mn);
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1) {
            if (!full[f1]) continue;
            double acc = 0;
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) acc += __ldg(val + rowp[f1] + f2 * deg + k) * xm[f2];
            y[f1] += acc;
        }
    }
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
#pragma unroll
        for (int o = GN / 2; o > 0; o >>= 1) y[f1] += __shfl_xor_sync(0xffffffffu, y[f1], o, GN);
        if (act && !full[f1]) y[f1] = val[rowp[f1]] * x[(size_t)f1 * N + n];
    }
}

// out = A in over the rows of the segment's nodes (all fields); dots for alpha or omega.
// MODE 0: v = A phat, alpha = rho / (rhat . v).  MODE 1: t = A shat, omega = (t.s)/(t.t).
// Node-row product: the d+1 rows of node n share n's neighbour list, so a group of GN lanes
// walks n's neighbours once (one index and d+1 input values per neighbour) and accumulates
// all d+1 rows.  One pass: NB x GN threads per segment.  FP32 reads the node-pair blocks of
// the scaled system, FP64 the field-major CSR of A.
template <class T, int DIM, int MODE, int GN>
__global__ void __launch_bounds__(NB * GN) k_mx_spmv(Mx m, const int* __restrict__ list,
                                                                  T* __restrict__ scb, int cnt_slot, int N,
                                                                  const int* __restrict__ rp,
                                                                  const int* __restrict__ nbr_ptr,
                                                                  const int* __restrict__ nbr,
                                                                  const T* __restrict__ val, T* __restrict__ W,
                                                                  size_t ld) {
    constexpr int B = DIM + 1;
    constexpr int NT = NB * GN;
    __shared__ double sh[32];
    const int b = list ? list[blockIdx.x] : blockIdx.x;  // segment
    const int inst = m.seg[3 * b];
    T* sc = scb + inst * M_COUNT;
    if (sc[M_DONE] != 0) return;
    const int n0 = m.seg[3 * b + 1], cnt = m.seg[3 * b + 2] - n0;
    const int lane = threadIdx.x % GN;
    const T* in = W + (MODE == 0 ? W_PHAT : W_SHAT) * ld;
    T* out = W + (MODE == 0 ? W_V : W_T) * ld;
    T d0 = 0, d1 = 0;
    const int ln = threadIdx.x / GN;
    const bool act = ln < cnt;
    const int n = n0 + (act ? ln : 0);
    T y[B];
    if constexpr (sizeof(T) == 4)
        block_row_f32<DIM, GN>(n, act, N, nbr_ptr, nbr, val, in, lane, y);
    else
        node_rows_f64<DIM, GN>(n, act, N, rp, nbr_ptr, nbr, val, in, lane, y);
    if (act && lane == 0) {
#pragma unroll
        for (int f1 = 0; f1 < B; ++f1) {
            const size_t r = (size_t)f1 * N + n;
            out[r] = y[f1];
            if (MODE == 0) {
                d0 += W[W_RHAT * ld + r] * y[f1];
            } else {
                d0 += y[f1] * W[W_S * ld + r];
                d1 += y[f1] * y[f1];
            }
        }
    }
    const int* ii = m.ii + inst * I_COUNT;
    T v[2] = {d0, d1};
    if (!inst_reduce<NT, 2, T>(v, b, ii[I_B0], ii[I_B1], reinterpret_cast<T*>(m.part),
                                       reinterpret_cast<unsigned*>(m.ii + inst * I_COUNT + I_TICKET), sh))
        return;
    if (threadIdx.x != 0) return;
    if (MODE == 0) {
        const T al = sc[M_RHO] / v[0];
        if (v[0] == 0 || !isfinite(v[0]) || !isfinite(al)) {  // breakdown: end this correction solve
            sc[M_DONE] = 2;
            atomicSub(m.cnt + cnt_slot, 1);
        } else {
            sc[M_ALPHA] = al;
        }
    } else {
        // omega = 0 ends the solve after the half step x += alpha phat (see k_mx_up_x)
        const T om = (v[1] == 0 || !isfinite(v[1])) ? T(0) : v[0] / v[1];
        sc[M_OMEGA] = isfinite(om) ? om : T(0);
    }
}

// FP32: z += alpha phat + omega shat (the correction, added to x as S z after the solve);
// FP64: x += alpha phat + omega shat.  r = s - omega t; rho = rhat.r; rr = r.r
template <class T, int DIM>
__global__ void __launch_bounds__(NB) k_mx_up_x(Mx m, const int* __restrict__ list, T* __restrict__ scb, int cnt_slot,
                                                int N, double* __restrict__ x,
                                                const double* __restrict__ scale, T* __restrict__ W, size_t ld) {
    __shared__ double sh[32];
    const int b = list ? list[blockIdx.x] : blockIdx.x;  // segment
    const int inst = m.seg[3 * b];
    T* sc = scb + inst * M_COUNT;
    if (sc[M_DONE] != 0) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    const T al = sc[M_ALPHA], om = sc[M_OMEGA];
    T rh = 0, rr = 0;
    if (n < m.seg[3 * b + 2]) {
#pragma unroll
        for (int f = 0; f <= DIM; ++f) {
            const size_t r = (size_t)f * N + n;
            if constexpr (sizeof(T) == 4)
                W[W_Z * ld + r] += al * W[W_PHAT * ld + r] + om * W[W_SHAT * ld + r];
            else
                x[r] += al * W[W_PHAT * ld + r] + om * W[W_SHAT * ld + r];
            const T rv = W[W_S * ld + r] - om * W[W_T * ld + r];
            W[W_R * ld + r] = rv;
            rh += W[W_RHAT * ld + r] * rv;
            rr += rv * rv;
        }
    }
    int* ii = m.ii + inst * I_COUNT;
    T v[2] = {rh, rr};
    if (!inst_reduce<NB, 2, T>(v, b, ii[I_B0], ii[I_B1], reinterpret_cast<T*>(m.part),
                               reinterpret_cast<unsigned*>(ii + I_TICKET), sh))
        return;
    if (threadIdx.x != 0) return;
    sc[M_RHO_OLD] = sc[M_RHO];
    sc[M_RHO] = v[0];
    sc[M_RR] = v[1];
    sc[M_ITERS] += 1;
    ii[I_KIT] += 1;
    T done = 0;
    if (!isfinite(v[1]))
        done = 2;
    else if (v[1] <= sc[M_TOL2])
        done = 1;
    else if (v[0] == 0 || om == 0)  // breakdown
        done = 2;
    if (done != 0) {
        sc[M_DONE] = done;
        atomicSub(m.cnt + cnt_slot, 1);
    }
}

// x += S z and z = 0 over every node: the FP32 solves' corrections (z stays 0 for instances
// solving in FP64)
template <int DIM>
__global__ void k_mx_apply_z(int N, const double* __restrict__ scale, float* __restrict__ z, double* __restrict__ x) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
#pragma unroll
    for (int f = 0; f <= DIM; ++f) {
        const size_t r = (size_t)f * N + n;
        const float zv = z[r];
        if (zv != 0.0f) {
            x[r] += scale[r] * (double)zv;
            z[r] = 0.0f;
        }
    }
}

// x = x_save for instances whose last FP32 correction sweep made the residual grow
template <int DIM>
__global__ void k_mx_rollback(int N, const double* __restrict__ xs, Mx m, double* __restrict__ x) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    if (!m.ii[m.node_inst[n] * I_COUNT + I_ROLL]) return;
#pragma unroll
    for (int f = 0; f <= DIM; ++f) x[(size_t)f * N + n] = xs[(size_t)f * N + n];
}

__global__ void k_mx_clear_roll(int n_inst, Mx m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_inst) m.ii[i * I_COUNT + I_ROLL] = 0;
}

// ---- node updates ---------------------------------------------------------------------------

// x = x_save + dt v for non-fixed nodes of active instances (Mesh.cpp:1246-1256)
template <int DIM>
__global__ void k_mx_positions(int N, const uint8_t* __restrict__ flags, const double* __restrict__ save,
                               const double* __restrict__ q, Mx m, double* __restrict__ pos) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int inst = m.node_inst[n];
    if (!m.ii[inst * I_COUNT + I_ACTIVE]) return;
    if (flags[n] & F_FIXED) return;
    const double dt = m.id[inst * D_COUNT + D_DT];
#pragma unroll
    for (int d = 0; d < DIM; ++d) pos[(size_t)d * N + n] = save[(size_t)d * N + n] + q[(size_t)d * N + n] * dt;
}

// Failed instances: positions and states revert to the saved node list (Mesh::restoreNodesList)
template <int DIM>
__global__ void k_mx_restore(int N, const double* __restrict__ save, const double* __restrict__ qprev, Mx m,
                             double* __restrict__ pos, double* __restrict__ q) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int inst = m.node_inst[n];
    if (m.ii[inst * I_COUNT + I_STATUS] != 2) return;
#pragma unroll
    for (int d = 0; d < DIM; ++d) pos[(size_t)d * N + n] = save[(size_t)d * N + n];
#pragma unroll
    for (int f = 0; f <= DIM; ++f) q[(size_t)f * N + n] = qprev[(size_t)f * N + n];
}

// ---- host side ---------------------------------------------------------------------------------

struct Counters {
    int need32, active, need64, redo;
};

int read_counters(pfg_ctx* c, Counters* k) {
    PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, c->mx_cnt.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    const int* h = reinterpret_cast<const int*>(c->h_scalars);
    k->need32 = h[C_NEED];
    k->active = h[C_ACTIVE];
    k->need64 = h[C_NEED64];
    k->redo = h[C_ROLLBACK];
    return PFG_OK;
}

// sum_g mu w_g in the order of k_sum's loop (the Newtonian K factor)
double ksum_newtonian(int dim, double mu) {
    const GaussConst g = gauss_const(dim);
    double s = 0;
    for (int q = 0; q < g.n; ++q) s += mu * g.w[q];
    return s;
}

EdPlanes ed_planes(pfg_ctx* c) {
    float* a = ptr<float>(c->mx_ed_aos);
    return EdPlanes{a, a + (size_t)ED_AOS * c->E, c->E};
}

// A, b at the iterate q_iter: element data, node blocks and right-hand side, FP32 pair blocks
// (and the multigrid's coarse blocks).
template <int DIM>
int mx_assemble(pfg_ctx* c, const double* q_iter, const MxConst& k) {
    const int N = c->N, E = c->E;
    Mx m = mx_ptrs(c);
    const EdPlanes ed = ed_planes(c);
    const bool dfa = c->prm.assembly == PFG_ASM_DOUBLE_FLOAT;
    DF* tdf = k.bq.T ? ptr<DF>(c->mx_tdf) : nullptr;
    float4* vsum = ptr<float4>(c->mx_vsum);
    prof_begin(c, PH_PSPG_ELEM);
    k_mx_vprep<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, ptr<double>(c->q_prev), k.bq.T, m,
                                                               ptr<DF>(c->mx_vpdf), tdf);
    if (E > 0) {
        if (c->prm.tau0 > 0) {  // Bingham viscosity from the iterate's strain rates: FP64 element prep
            k_mx_prep<DIM><<<div_up(E, c->tune.elem_block), c->tune.elem_block, 0, c->stream>>>(
                E, N, ptr<int>(c->conn), ptr<double>(c->pos), q_iter, m, k.refSize, visc_args(c),
                const_cast<float*>(ed.ah), ptr<DF>(c->mx_vpdf), vsum, ptr<int>(c->el_slot));
        } else {
            k_mx_gprep<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, ptr<double>(c->pos), q_iter, m,
                                                                       ptr<DF>(c->mx_gdf));
            k_mx_prep_df<DIM><<<div_up(E, c->tune.elem_block), c->tune.elem_block, 0, c->stream>>>(
                E, N, ptr<int>(c->conn), ptr<DF>(c->mx_gdf), ptr<float>(c->mx_f32), m, k.ref_df, k.inv_pi_df,
                const_cast<float*>(ed.ah), ptr<DF>(c->mx_vpdf), vsum, ptr<int>(c->el_slot));
        }
    }
    prof_end(c, PH_PSPG_ELEM);
    PFG_CHECK_LAUNCH(c);
    prof_begin(c, PH_PSPG_RHS);
    const FstArgs fa = fst_args(c);
    if (fa.nodes)
        k_fst<DIM, double><<<div_up(fa.n_nodes, BLOCK), BLOCK, 0, c->stream>>>(
            fa, E, ptr<int>(c->conn), PosF64{ptr<double>(c->pos), N}, N, ptr<double>(c->fst_force));
    uint16_t* v16 = c->n_mg > 0 ? ptr<uint16_t>(c->val16) : nullptr;
    auto node_kernel = dfa ? k_mx_node<DIM, true> : k_mx_node<DIM, false>;
    node_kernel<<<c->n_seg, NB, 0, c->stream>>>(
        m, N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem), ptr<int>(c->ne_slot), ptr<uint8_t>(c->ne_loc),
        ptr<int>(c->conn), ed, ptr<uint8_t>(c->flags), ptr<DF>(c->mx_vpdf), vsum, tdf, ptr<double>(c->q_prev), ptr<double>(c->vbc),
        fst_force<double>(c), ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<float>(c->mx_f32), k, ptr<double>(c->rhs),
        ptr<double>(c->mx_scale), ptr<float>(c->mx_scale32), ptr<float>(c->binv32), ptr<float>(c->val32), v16);
    prof_end(c, PH_PSPG_RHS);
    PFG_CHECK_LAUNCH(c);
    prof_begin(c, PH_PSPG_PAIRS);
    if (!dfa && c->tune.pair_block == STAGE_PAIRS) {
        // the row-staged FP32 pair kernel (default)
        k_mx_asm32_rows<DIM><<<div_up(c->P, STAGE_PAIRS), STAGE_PAIRS, 0, c->stream>>>(
            c->P, N, ptr<int>(c->pair_node), ptr<int>(c->nbr), ptr<int>(c->pe_ptr), ptr<int>(c->pe_pos),
            ptr<int>(c->ne_ptr), ptr<int>(c->ne_slot), ed, ptr<uint8_t>(c->flags), ptr<float>(c->mx_scale32),
            ptr<float>(c->mx_f32), m, k, ptr<float>(c->val32), v16);
    } else if (dfa || c->tune.pair_block != ASM_ITEMS) {
        // double-float pair arithmetic, or the pair-parallel kernel reading global memory
        auto pair_kernel = dfa ? k_mx_asm32<DIM, true> : k_mx_asm32<DIM, false>;
        const int pb = dfa ? BLOCK : c->tune.pair_block;
        pair_kernel<<<div_up(c->P, pb), pb, 0, c->stream>>>(
            c->P, N, ptr<int>(c->pair_node), ptr<int>(c->nbr), ptr<int>(c->pe_ptr), ptr<int>(c->pe_item), ed,
            ptr<uint8_t>(c->flags), ptr<float>(c->mx_scale32), ptr<float>(c->mx_f32), m, k, ptr<float>(c->val32), v16);
    } else if (c->n_items > 0) {
        k_mx_asm32_items<DIM><<<(int)((c->n_items + ASM_ITEMS - 1) / ASM_ITEMS), ASM_ITEMS, 0, c->stream>>>(
            c->n_items, N, ptr<int>(c->pair_node), ptr<int>(c->nbr), ptr<int>(c->pe_ptr), ptr<int>(c->pe_item),
            ptr<int>(c->pe_pair), ed, ptr<uint8_t>(c->flags), ptr<float>(c->mx_scale32), ptr<float>(c->mx_f32), m, k,
            ptr<float>(c->val32), v16);
    }
    prof_end(c, PH_PSPG_PAIRS);
    PFG_CHECK_LAUNCH(c);
    if (c->n_mg > 0) {
        prof_begin(c, PH_MG_SETUP);
        int rc = mg_numeric(c);
        prof_end(c, PH_MG_SETUP);
        if (rc) return rc;
    }
    return PFG_OK;
}

// FP64 CSR values for the instances in FP64 mode that lack them for this assembly (the FP64
// correction solves' products); the kernel does nothing for the other instances.
template <int DIM>
int mx_csr64(pfg_ctx* c, const MxConst& k) {
    Mx m = mx_ptrs(c);
    prof_begin(c, PH_PSPG_PAIRS);
    k_mx_pairs<DIM><<<div_up(c->P, BLOCK), BLOCK, 0, c->stream>>>(
        c->P, c->N, c->E, ptr<int>(c->pair_node), ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<int>(c->ne_ptr),
        ptr<int>(c->ne_elem), ptr<int>(c->ne_slot), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn), ed_planes(c),
        ptr<uint8_t>(c->flags),
        ptr<int>(c->row_ptr), ptr<double>(c->val), ptr<double>(c->vbc), ptr<float>(c->mx_f32), m, k);
    k_mx_binv64<DIM><<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(c->N, ptr<int>(c->nbr_ptr), ptr<int>(c->nbr),
                                                                   ptr<int>(c->row_ptr), ptr<double>(c->val),
                                                                   ptr<uint8_t>(c->flags), m, ptr<double>(c->binv));
    k_mx_mark_csr64<<<div_up(c->n_inst, BLOCK), BLOCK, 0, c->stream>>>(c->n_inst, m);
    prof_end(c, PH_PSPG_PAIRS);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

template <int DIM>
int mx_residual(pfg_ctx* c, const MxConst& k, int kind, Counters* cnt) {
    Mx m = mx_ptrs(c);
    const int N = c->N, E = c->E;
    PFG_CUDA(c, cudaMemsetAsync(c->mx_cnt.p, 0, 4 * sizeof(int), c->stream));
    prof_begin(c, PH_RESIDUAL);
    k_mx_xdf<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, ptr<double>(c->q), ptr<double>(c->vbc),
                                                             ptr<uint8_t>(c->flags), m, ptr<DF>(c->mx_xdf));
    if (E > 0)
        k_mx_res_elem<DIM><<<div_up(E, c->tune.res_block), c->tune.res_block, 0, c->stream>>>(
            E, N, ptr<int>(c->conn_s), ed_planes(c), ptr<uint8_t>(c->flags), ptr<DF>(c->mx_xdf), ptr<float>(c->mx_f32),
            m, k, ptr<float4>(c->mx_rec));
    k_mx_res_node<DIM><<<c->n_seg, NB, 0, c->stream>>>(
        m, N, ptr<int>(c->ne_ptr), ptr<int>(c->ne_slot), ptr<uint8_t>(c->ne_loc), ptr<float4>(c->mx_rec),
        ptr<uint8_t>(c->flags), ptr<double>(c->rhs), ptr<double>(c->q), ptr<double>(c->mx_scale), k,
        ptr<float>(c->kv32), ptr<double>(c->kv), (size_t)c->R, kind);
    prof_end(c, PH_RESIDUAL);
    PFG_CHECK_LAUNCH(c);
    return read_counters(c, cnt);
}

// FP64 correction solves preconditioned by the FP32 multigrid of the scaled system:
// M^-1 v = S (S A S)^-1_MG (S v).  k_mx_to_mg writes FP32(S v), k_mx_from_mg v_hat = S out.
template <int DIM>
__global__ void __launch_bounds__(NB) k_mx_to_mg(Mx m, const int* __restrict__ list, const double* __restrict__ scb,
                                                 int N, const double* __restrict__ v, const double* __restrict__ scale,
                                                 float* __restrict__ out) {
    const int b = list ? list[blockIdx.x] : blockIdx.x;
    if (scb[m.seg[3 * b] * M_COUNT + M_DONE] != 0) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    if (n >= m.seg[3 * b + 2]) return;
#pragma unroll
    for (int f = 0; f <= DIM; ++f) {
        const size_t r = (size_t)f * N + n;
        out[r] = (float)(scale[r] * v[r]);
    }
}

template <int DIM>
__global__ void __launch_bounds__(NB) k_mx_from_mg(Mx m, const int* __restrict__ list, const double* __restrict__ scb,
                                                   int N, const float* __restrict__ in, const double* __restrict__ scale,
                                                   double* __restrict__ vhat) {
    const int b = list ? list[blockIdx.x] : blockIdx.x;
    if (scb[m.seg[3 * b] * M_COUNT + M_DONE] != 0) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    if (n >= m.seg[3 * b + 2]) return;
#pragma unroll
    for (int f = 0; f <= DIM; ++f) {
        const size_t r = (size_t)f * N + n;
        vhat[r] = scale[r] * (double)in[r];
    }
}

// The five kernels of one BiCGSTAB iteration in precision T, over `grid` segments (all of them,
// or the compacted list of segments whose instance is still iterating).  With the multigrid
// on, its V-cycle replaces the node-block Jacobi apply in both precisions.
template <class T, int DIM>
struct KSet {
    Mx m;
    const int* list;
    T* scb;
    int slot, N;
    size_t ld;
    T* W;
    const T* binv;
    const T* val;
    const double* scale;
    const int* rp;
    const int* col;
    const int* nptr;
    const int* nbr;
    double* x;

    // vhat = M^-1 v by the multigrid (the block-Jacobi vhat of the update kernel is overwritten)
    void precondition(pfg_ctx* c, int grid, T* v, T* vhat) const {
        if (c->n_mg == 0) return;
        prof_begin(c, PH_MG_CYCLE);
        if constexpr (sizeof(T) == 4) {
            mg_apply(c, v, vhat);
        } else {
            float* in = ptr<float>(c->mg_in64);
            float* out = in + ld;
            const double* sc = ptr<double>(c->mx_scale);
            k_mx_to_mg<DIM><<<grid, NB, 0, c->stream>>>(m, list, scb, N, v, sc, in);
            mg_apply(c, in, out);
            k_mx_from_mg<DIM><<<grid, NB, 0, c->stream>>>(m, list, scb, N, out, sc, vhat);
        }
        prof_end(c, PH_MG_CYCLE);
    }

    void up_p(pfg_ctx* c, int grid) const { k_mx_up_p<T, DIM><<<grid, NB, 0, c->stream>>>(m, list, scb, N, W, ld, binv); }
    void up_s(pfg_ctx* c, int grid) const { k_mx_up_s<T, DIM><<<grid, NB, 0, c->stream>>>(m, list, scb, N, W, ld, binv); }
    void up_x(pfg_ctx* c, int grid) const {
        k_mx_up_x<T, DIM><<<grid, NB, 0, c->stream>>>(m, list, scb, slot, N, x, scale, W, ld);
    }
    // The FP32 products are the timed "Krylov SpMV" phase (with the node pairs they read); the
    // FP64 fallback's stay in the iteration phase only.
    template <int MODE>
    void spmv(pfg_ctx* c, int grid) const {
        constexpr bool F32 = sizeof(T) == 4;
        if (F32) {
            prof_begin(c, PH_KRYLOV_SPMV);
            if (c->prof) c->spmv_pairs += c->spmv_list_pairs;
        }
        // lanes per node: the tuned choice (node_lanes<DIM>() by default)
        const int gn = c->tune.spmv_lanes;
        if (gn == node_lanes<DIM>() / 2)
            k_mx_spmv<T, DIM, MODE, node_lanes<DIM>() / 2><<<grid, NB * gn, 0, c->stream>>>(m, list, scb, slot, N, rp,
                                                                                          nptr, nbr, val, W, ld);
        else if (gn == 2 * node_lanes<DIM>())
            k_mx_spmv<T, DIM, MODE, 2 * node_lanes<DIM>()><<<grid, NB * gn, 0, c->stream>>>(m, list, scb, slot, N, rp,
                                                                                          nptr, nbr, val, W, ld);
        else
            k_mx_spmv<T, DIM, MODE, node_lanes<DIM>()><<<grid, NB * node_lanes<DIM>(), 0, c->stream>>>(
                m, list, scb, slot, N, rp, nptr, nbr, val, W, ld);
        if (F32) prof_end(c, PH_KRYLOV_SPMV);
    }

    void iterate(pfg_ctx* c, int grid) const {
        prof_begin(c, PH_KRYLOV_ITER);
        up_p(c, grid);
        precondition(c, grid, W + W_P * ld, W + W_PHAT * ld);
        spmv<0>(c, grid);
        up_s(c, grid);
        precondition(c, grid, W + W_S * ld, W + W_SHAT * ld);
        spmv<1>(c, grid);
        up_x(c, grid);
        prof_end(c, PH_KRYLOV_ITER);
    }
};

// One BiCGSTAB iteration of a batch whose instances iterate in both precisions (na segments
// in FP32, nb in FP64).  With the multigrid on, one V-cycle serves both: the FP64 instances'
// scaled vectors are written into their (unused) rows of the FP32 workspace, so the cycle over
// all nodes preconditions every instance at once.
template <int DIM>
void iterate_batch(pfg_ctx* c, const KSet<float, DIM>& a, int na, const KSet<double, DIM>& b, int nb) {
    auto shared_cycle = [&](int src, int dst) {
        if (c->n_mg == 0) return;
        prof_begin(c, PH_MG_CYCLE);
        const double* sc = ptr<double>(c->mx_scale);
        float* in = a.W + src * a.ld;
        float* out = a.W + dst * a.ld;
        if (nb) k_mx_to_mg<DIM><<<nb, NB, 0, c->stream>>>(b.m, b.list, b.scb, b.N, b.W + src * b.ld, sc, in);
        mg_apply(c, in, out);
        if (nb) k_mx_from_mg<DIM><<<nb, NB, 0, c->stream>>>(b.m, b.list, b.scb, b.N, out, sc, b.W + dst * b.ld);
        prof_end(c, PH_MG_CYCLE);
    };
    prof_begin(c, PH_KRYLOV_ITER);
    if (na) a.up_p(c, na);
    if (nb) b.up_p(c, nb);
    shared_cycle(W_P, W_PHAT);
    if (na) a.template spmv<0>(c, na);
    if (nb) b.template spmv<0>(c, nb);
    if (na) a.up_s(c, na);
    if (nb) b.up_s(c, nb);
    shared_cycle(W_S, W_SHAT);
    if (na) a.template spmv<1>(c, na);
    if (nb) b.template spmv<1>(c, nb);
    if (na) a.up_x(c, na);
    if (nb) b.up_x(c, nb);
    prof_end(c, PH_KRYLOV_ITER);
}

template <class T, int DIM>
KSet<T, DIM> kset(pfg_ctx* c, const int* list) {
    constexpr bool F32 = sizeof(T) == 4;
    KSet<T, DIM> k;
    k.m = mx_ptrs(c);
    k.list = list;
    k.scb = F32 ? reinterpret_cast<T*>(k.m.sc) : reinterpret_cast<T*>(k.m.sc64);
    k.slot = F32 ? C_NEED : C_NEED64;
    k.N = c->N;
    k.ld = (size_t)c->R;
    k.W = F32 ? reinterpret_cast<T*>(c->kv32.p) : reinterpret_cast<T*>(c->kv.p);
    k.binv = F32 ? reinterpret_cast<const T*>(c->binv32.p) : reinterpret_cast<const T*>(c->binv.p);
    k.val = F32 ? reinterpret_cast<const T*>(c->val32.p) : reinterpret_cast<const T*>(c->val.p);
    k.scale = F32 ? ptr<double>(c->mx_scale) : nullptr;
    k.rp = ptr<int>(c->row_ptr);
    k.col = ptr<int>(c->col);
    k.nptr = ptr<int>(c->nbr_ptr);
    k.nbr = ptr<int>(c->nbr);
    k.x = ptr<double>(c->q);
    return k;
}

// Correction solves in precision T of a single mesh, until done or the iteration cap is
// reached: chunks of 8 iterations replayed from a CUDA graph, the running-solve counter polled
// after 1, 1, 2, 2, 4, 4, ... chunks (a finished solve skips the extra iterations in every
// kernel).  x (the FP64 iterate) is updated in place.
template <class T, int DIM>
int mx_inner(pfg_ctx* c, Counters* cnt) {
    constexpr bool F32 = sizeof(T) == 4;
    const KSet<T, DIM> ks = kset<T, DIM>(c, nullptr);
    cudaGraphExec_t& graph = c->mx_graph[F32 ? 0 : 1];
    const int max_it = std::max(1, c->prm.krylov_max_iter);
    const int chunk = 8;
    int done_it = 0;
    int polls = 0;
    int* need = F32 ? &cnt->need32 : &cnt->need64;
    while (*need > 0 && done_it < max_it) {
        const int reps = std::min(1 << (polls / 2), 4);
        const int n = std::min(chunk * reps, max_it - done_it);
        ++polls;
        if (n == chunk * reps && !c->prof) {
            if (!graph) {
                cudaGraph_t g = nullptr;
                PFG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                for (int it = 0; it < chunk; ++it) ks.iterate(c, c->n_seg);
                cudaError_t e = cudaStreamEndCapture(c->stream, &g);
                if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
                e = cudaGraphInstantiate(&graph, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    graph = nullptr;
                    return cuda_fail(c, e, "cudaGraphInstantiate");
                }
            }
            for (int r = 0; r < reps; ++r) PFG_CUDA(c, cudaGraphLaunch(graph, c->stream));
        } else {
            for (int it = 0; it < n; ++it) ks.iterate(c, c->n_seg);
        }
        PFG_CHECK_LAUNCH(c);
        done_it += n;
        int rc = read_counters(c, cnt);
        if (rc) return rc;
    }
    return PFG_OK;
}

// Correction solves of a batch: FP32 and FP64 instances iterate in the same loop, and after
// every chunk of 8 iterations the kernels are relaunched over the compacted list of segments
// whose instance is still iterating (finished instances cost nothing afterwards).
template <int DIM>
int mx_inner_batch(pfg_ctx* c, Counters* cnt) {
    const int K = c->n_inst;
    int* d_list32 = ptr<int>(c->mx_list);
    int* d_list64 = d_list32 + c->n_seg;
    const KSet<float, DIM> k32 = kset<float, DIM>(c, d_list32);
    const KSet<double, DIM> k64 = kset<double, DIM>(c, d_list64);
    std::vector<float> done32((size_t)K * M_COUNT);
    std::vector<double> done64((size_t)K * M_COUNT);
    std::vector<int> l32, l64;
    l32.reserve(c->n_seg);
    l64.reserve(c->n_seg);
    const std::vector<int>& hi = c->h_mx_ii;
    auto rebuild = [&]() -> int {
        const Mx m = mx_ptrs(c);
        PFG_CUDA(c, cudaMemcpyAsync(done32.data(), m.sc, sizeof(float) * done32.size(), cudaMemcpyDeviceToHost,
                                    c->stream));
        PFG_CUDA(c, cudaMemcpyAsync(done64.data(), m.sc64, sizeof(double) * done64.size(), cudaMemcpyDeviceToHost,
                                    c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        std::vector<int> n32, n64;
        n32.reserve(c->n_seg);
        n64.reserve(c->n_seg);
        c->spmv_list_pairs = 0;
        for (int i = 0; i < K; ++i) {
            const int b0 = hi[(size_t)i * I_COUNT + I_B0], b1 = hi[(size_t)i * I_COUNT + I_B1];
            if (done32[(size_t)i * M_COUNT + M_DONE] == 0.0f) {
                for (int b = b0; b < b1; ++b) n32.push_back(b);
                c->spmv_list_pairs += c->h_inst_pairs[i];
            }
            if (done64[(size_t)i * M_COUNT + M_DONE] == 0.0)
                for (int b = b0; b < b1; ++b) n64.push_back(b);
        }
        if (n32 != l32 && !n32.empty())
            PFG_CUDA(c, cudaMemcpyAsync(d_list32, n32.data(), sizeof(int) * n32.size(), cudaMemcpyHostToDevice,
                                        c->stream));
        if (n64 != l64 && !n64.empty())
            PFG_CUDA(c, cudaMemcpyAsync(d_list64, n64.data(), sizeof(int) * n64.size(), cudaMemcpyHostToDevice,
                                        c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        l32.swap(n32);
        l64.swap(n64);
        return PFG_OK;
    };
    int rc;
    if ((rc = rebuild())) return rc;
    const int max_it = std::max(1, c->prm.krylov_max_iter);
    const int chunk = 8;
    int done_it = 0;
    while ((!l32.empty() || !l64.empty()) && done_it < max_it) {
        const int n = std::min(chunk, max_it - done_it);
        for (int it = 0; it < n; ++it) iterate_batch<DIM>(c, k32, (int)l32.size(), k64, (int)l64.size());
        PFG_CHECK_LAUNCH(c);
        done_it += n;
        if ((rc = rebuild())) return rc;
    }
    return read_counters(c, cnt);
}

// One linear solve of every active instance by iterative refinement: correction sweeps in
// each instance's precision, FP64 residual after each; an FP32 sweep that made things worse
// is undone and the instance continues in FP64.
template <int DIM>
int mx_refine(pfg_ctx* c, const MxConst& k, Counters* cnt) {
    const int max_ref = c->prm.refine_max_iter > 0 ? c->prm.refine_max_iter : 30;
    int rc;
    for (int sweep = 0; sweep < max_ref && (cnt->need32 > 0 || cnt->need64 > 0); ++sweep) {
        PFG_CUDA(c, cudaMemcpyAsync(c->q_iter_prev.p, c->q.p, sizeof(double) * c->R, cudaMemcpyDeviceToDevice,
                                    c->stream));
        if (cnt->need64 > 0 && (rc = mx_csr64<DIM>(c, k))) return rc;
        if (c->n_inst > 1) {
            if ((rc = mx_inner_batch<DIM>(c, cnt))) return rc;
        } else {
            if (cnt->need32 > 0 && (rc = mx_inner<float, DIM>(c, cnt))) return rc;
            if (cnt->need64 > 0 && (rc = mx_inner<double, DIM>(c, cnt))) return rc;
        }
        k_mx_apply_z<DIM><<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(
            c->N, ptr<double>(c->mx_scale), ptr<float>(c->kv32) + (size_t)W_Z * c->R, ptr<double>(c->q));
        PFG_CHECK_LAUNCH(c);
        if ((rc = mx_residual<DIM>(c, k, RES_SWEEP, cnt))) return rc;
        if (cnt->redo > 0) {
            k_mx_rollback<DIM><<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(c->N, ptr<double>(c->q_iter_prev),
                                                                            mx_ptrs(c), ptr<double>(c->q));
            k_mx_clear_roll<<<div_up(c->n_inst, BLOCK), BLOCK, 0, c->stream>>>(c->n_inst, mx_ptrs(c));
            PFG_CHECK_LAUNCH(c);
            if ((rc = mx_residual<DIM>(c, k, RES_START, cnt))) return rc;
        }
    }
    return PFG_OK;
}

template <int DIM>
int mx_picard(pfg_ctx* c, const double* dts, pfg_step_status* st) {
    const int K = c->n_inst;
    const size_t R = c->R;
    int rc;
    // per-instance tables: counters reset, dt of this step, all instances active (the
    // correction-solve precision of each instance carries over from its previous steps)
    std::vector<int>& hi = c->h_mx_ii;
    std::vector<double>& hd = c->h_mx_id;
    for (int i = 0; i < K; ++i) {
        int* r = hi.data() + (size_t)i * I_COUNT;
        r[I_ACTIVE] = 1;
        r[I_STATUS] = 0;
        r[I_IT] = 0;
        r[I_KIT] = 0;
        r[I_TICKET] = 0;
        r[I_ROLL] = 0;
        hd[(size_t)i * D_COUNT + D_DT] = dts[i];
    }
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_ii.p, hi.data(), sizeof(int) * hi.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_id.p, hd.data(), sizeof(double) * hd.size(), cudaMemcpyHostToDevice, c->stream));
    // per-instance coefficients as double-float pairs (high parts = the FP32 kernels' values)
    {
        const double sumw = gauss_const(c->dim).sumw;
        std::vector<float>& hf = c->h_mx_f32;
        hf.assign((size_t)K * F_COUNT, 0.0f);
        auto put = [&](int i, int which, double v) {
            const float h = (float)v;
            hf[(size_t)i * F_COUNT + which] = h;
            hf[(size_t)i * F_COUNT + which + 1] = (float)(v - (double)h);
        };
        for (int i = 0; i < K; ++i) {
            const double rho = hd[(size_t)i * D_COUNT + D_RHO], mu = hd[(size_t)i * D_COUNT + D_MU];
            put(i, F_RHO, rho);
            put(i, F_INVDT, 1.0 / dts[i]);
            put(i, F_LSUM, sumw / rho);
            put(i, F_CM, rho / dts[i]);
            put(i, F_MU4R, 4 * mu / rho);
            put(i, F_KSUM, ksum_newtonian(c->dim, mu));
        }
        PFG_CUDA(c, cudaMemcpyAsync(c->mx_f32.p, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice,
                                    c->stream));
    }
    // prepare: save the node list, qPrev = states, build A and b at the current geometry
    PFG_CUDA(c, cudaMemcpyAsync(c->pos_save.p, c->pos.p, sizeof(double) * c->dim * c->N, cudaMemcpyDeviceToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->q_prev.p, c->q.p, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
    const MxConst k = mx_const(c);
    if ((rc = mx_assemble<DIM>(c, ptr<double>(c->q_prev), k))) return rc;
    Counters cnt{};
    if ((rc = mx_residual<DIM>(c, k, RES_START, &cnt))) return rc;
    while (true) {
        if ((rc = mx_refine<DIM>(c, k, &cnt))) return rc;
        // Picard update: positions, re-assembly, residual check
        k_mx_positions<DIM><<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(
            c->N, ptr<uint8_t>(c->flags), ptr<double>(c->pos_save), ptr<double>(c->q), mx_ptrs(c), ptr<double>(c->pos));
        PFG_CHECK_LAUNCH(c);
        if ((rc = mx_assemble<DIM>(c, ptr<double>(c->q), k))) return rc;
        if ((rc = mx_residual<DIM>(c, k, RES_PICARD, &cnt))) return rc;
        if (cnt.active == 0) break;
        if (cnt.redo > 0 && (rc = mx_residual<DIM>(c, k, RES_START, &cnt))) return rc;
    }
    k_mx_restore<DIM><<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(
        c->N, ptr<double>(c->pos_save), ptr<double>(c->q_prev), mx_ptrs(c), ptr<double>(c->pos), ptr<double>(c->q));
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaMemcpyAsync(hi.data(), c->mx_ii.p, sizeof(int) * hi.size(), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(hd.data(), c->mx_id.p, sizeof(double) * hd.size(), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int i = 0; i < K; ++i) {
        const int* r = hi.data() + (size_t)i * I_COUNT;
        pfg_step_status& s = st[i];
        std::memset(&s, 0, sizeof(s));
        s.converged = r[I_STATUS] == 1 ? 1 : 0;
        s.picard_iterations = r[I_IT];
        s.krylov_iterations = r[I_KIT];
        s.residual = hd[(size_t)i * D_COUNT + D_RES];
        s.dt = dts[i];
        s.fp64_solves = r[I_MODE] == MODE_FP64 ? 1 : 0;
    }
    return PFG_OK;
}

}  // namespace

int mx_alloc(pfg_ctx* c) {
    const size_t R = std::max(c->R, 1), N = std::max(c->N, 1), E = std::max(c->E, 1);
    int rc;
    const size_t npe = c->dim + 1;
    if ((rc = ensure(c, c->val32, sizeof(float) * (size_t)std::max(c->P, 1) * (c->dim + 1) * (c->dim + 1))) ||
        (rc = ensure(c, c->mx_scale32, sizeof(float) * R)) || (rc = ensure(c, c->mx_xdf, sizeof(DF) * R)) ||
        (rc = ensure(c, c->mx_vpdf, sizeof(DF) * (size_t)c->dim * N)) ||
        (rc = ensure(c, c->mx_gdf, sizeof(DF) * 2 * (size_t)c->dim * N)) ||
        (rc = ensure(c, c->mx_tdf, sizeof(DF) * (c->prm.boussinesq ? N : 1))) ||
        (rc = ensure(c, c->mx_rec, 32 * npe * E)) ||
        (rc = ensure(c, c->mx_ed_aos, sizeof(float) * 2 * ED_AOS * E)) ||
        (rc = ensure(c, c->mx_vsum, 2 * sizeof(float4) * E)) ||
        (rc = ensure(c, c->kv32, sizeof(float) * W_COUNT * R)) || (rc = ensure(c, c->mx_scale, sizeof(double) * R)) ||
        (rc = ensure(c, c->binv32, sizeof(float) * (size_t)(c->dim + 1) * (c->dim + 1) * N)) ||
        (rc = ensure(c, c->mx_cnt, 64)) || (rc = ensure(c, c->node_inst, sizeof(int) * N)))
        return rc;
    PFG_CUDA(c, cudaMemsetAsync(ptr<float>(c->kv32) + (size_t)W_Z * R, 0, sizeof(float) * R, c->stream));
    c->n_mg = 0;
    if (c->prm.preconditioner == PFG_PC_MULTIGRID) {
        if ((rc = mg_setup(c)) || (rc = ensure(c, c->mg_in64, sizeof(float) * 2 * R)) ||
            (rc = ensure(c, c->val16, sizeof(uint16_t) * (size_t)std::max(c->P, 1) * (c->dim + 1) * 4)))
            return rc;
        // the cycle runs over every node: keep the rows of instances not in FP64 mode finite
        PFG_CUDA(c, cudaMemsetAsync(c->mg_in64.p, 0, sizeof(float) * 2 * R, c->stream));
    }
    // one instance covering the whole mesh until pfg_set_instances says otherwise
    const int off[2] = {0, c->N};
    const double rho = c->prm.rho, mu = c->prm.mu;
    return mx_set_instances(c, 1, off, &rho, &mu);
}

void mx_release_graph(pfg_ctx* c) {
    for (auto& g : c->mx_graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

int mx_set_instances(pfg_ctx* c, int n_inst, const int* node_off, const double* rho, const double* mu) {
    const int N = c->N;
    mx_release_graph(c);
    // segments of at most NB nodes inside each instance
    std::vector<int> seg;
    std::vector<int> node_inst(N);
    c->h_mx_ii.assign((size_t)n_inst * I_COUNT, 0);
    c->h_mx_id.assign((size_t)n_inst * D_COUNT, 0.0);
    for (int i = 0; i < n_inst; ++i) {
        const int n0 = node_off[i], n1 = node_off[i + 1];
        int* r = c->h_mx_ii.data() + (size_t)i * I_COUNT;
        r[I_N0] = n0;
        r[I_N1] = n1;
        r[I_B0] = (int)(seg.size() / 3);
        for (int s = n0; s < n1; s += NB) {
            seg.push_back(i);
            seg.push_back(s);
            seg.push_back(std::min(n1, s + NB));
        }
        if (n1 == n0) {  // an empty instance still owns one (empty) segment for its reductions
            seg.push_back(i);
            seg.push_back(n0);
            seg.push_back(n0);
        }
        r[I_B1] = (int)(seg.size() / 3);
        for (int n = n0; n < n1; ++n) node_inst[n] = i;
        double* d = c->h_mx_id.data() + (size_t)i * D_COUNT;
        d[D_RHO] = rho[i];
        d[D_MU] = mu[i];
        d[D_DT] = 1e-3;
    }
    c->n_inst = n_inst;
    c->n_seg = (int)(seg.size() / 3);
    int rc;
    if ((rc = ensure(c, c->mx_seg, sizeof(int) * seg.size())) ||
        (rc = ensure(c, c->mx_ii, sizeof(int) * c->h_mx_ii.size())) ||
        (rc = ensure(c, c->mx_id, sizeof(double) * c->h_mx_id.size())) ||
        (rc = ensure(c, c->mx_sc, 256 * (((size_t)n_inst * M_COUNT * sizeof(float) + 255) / 256) +
                                      sizeof(double) * (size_t)n_inst * M_COUNT)) ||
        (rc = ensure(c, c->mx_part, sizeof(double) * 4 * (size_t)c->n_seg)) ||
        (rc = ensure(c, c->mx_f32, sizeof(float) * F_COUNT * (size_t)n_inst)) ||
        (rc = ensure(c, c->mx_list, sizeof(int) * 2 * (size_t)c->n_seg)))
        return rc;
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_seg.p, seg.data(), sizeof(int) * seg.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->node_inst.p, node_inst.data(), sizeof(int) * (size_t)N, cudaMemcpyHostToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_ii.p, c->h_mx_ii.data(), sizeof(int) * c->h_mx_ii.size(), cudaMemcpyHostToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_id.p, c->h_mx_id.data(), sizeof(double) * c->h_mx_id.size(),
                                cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(c->mx_sc.p, 0, sizeof(float) * (size_t)n_inst * M_COUNT, c->stream));
    // node pairs per instance (the work of its SpMV rows, for the phase counters)
    std::vector<int> nptr((size_t)N + 1);
    PFG_CUDA(c, cudaMemcpyAsync(nptr.data(), c->nbr_ptr.p, sizeof(int) * nptr.size(), cudaMemcpyDeviceToHost,
                                c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->h_inst_pairs.assign(n_inst, 0);
    for (int i = 0; i < n_inst; ++i) c->h_inst_pairs[i] = (long long)nptr[node_off[i + 1]] - nptr[node_off[i]];
    return PFG_OK;
}

int mx_picard_step(pfg_ctx* c, const double* dts, pfg_step_status* st) {
    return c->dim == 2 ? mx_picard<2>(c, dts, st) : mx_picard<3>(c, dts, st);
}

}  // namespace pfg
