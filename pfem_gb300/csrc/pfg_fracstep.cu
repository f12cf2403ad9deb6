// Fractional-step solver of the incompressible equations (solver "FracStep"), plain FP64 form.
//
// Reference: MomContEqIncompNewton with m_setupPicardFracStep (MomContEquationFracStep.inl:
// 463-630), m_buildMatFracStep (:7-197), m_applyBCVAppStep (:199-260), m_buildMatPcorrStep
// (:262-301), m_applyBCPCorrStep (:303-325), m_buildMatVStep (:327-387), m_applyBCVStep
// (:389-413); factors M rho, K mu (Bingham law included), D 1, L 1, F rho (MomContEquation.inl:
// 97-161).  One Picard iteration at the current positions, with the previous step's (v, p):
//   (M/dt + K) v~ = F + M/dt v_prev + gammaFS D^T p_prev      velocity prediction
//   L p = -(rho/dt) D v~ + gammaFS L p_prev                    pressure
//   M dv = dt D^T (p - gammaFS p_prev)                          velocity correction
//   v = v~ + dv, positions = saved + dt v, residual U or U_P (the relative change of the
//   iterate over the non-free nodes, :568-629).
// Identity rows: bound and free nodes in the velocity systems, free nodes in L; the Dirichlet
// velocity columns of the prediction moved to its right-hand side; the columns of bound and
// free nodes in M and of free nodes in L set to the identity column.  Free-surface nodes keep
// their Laplacian rows with a zero right-hand side, as in the reference, which leaves constant
// pressures in the null space of L: each connected group of elements gets a gauge node (its
// smallest free-surface node, else its smallest node) treated as a free node in L (p = 0
// there); with fs_pressure_dirichlet every free-surface node is (the usual PFEM condition).
//
// Layout: the velocity matrix in CSR over the dim N velocity unknowns (row (n, a) holds, in
// field-major blocks, columns (m, b) at row_ptr + b deg(n) + rank of m; one diagonal entry for
// bound and free rows); L and M (one scalar matrix for every velocity component) in the
// node-pair layout of the adjacency (value of pair p = (n, m) at p).  Each value is gathered by
// one thread from the elements the two nodes share, in ascending element order; right-hand
// sides are gathered per node in ascending element order, so no atomics are used.  The three
// SPD systems are solved by Jacobi-preconditioned CG to the context's Krylov tolerances (the
// reference factorises each with SparseLU).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"
#include "pfg_pspg_common.cuh"

namespace pfg {

namespace {

struct FsConst {
    double rho, dt, gfs, refSize;
    double l_sum;  // sum_g w_g (the L factor 1)
    double MM[4][4], s[4], g[3];
};

FsConst fs_const(pfg_ctx* c, double dt) {
    const GaussConst gc = gauss_const(c->dim);
    FsConst k{};
    k.rho = c->prm.rho;
    k.dt = dt;
    k.gfs = c->prm.gamma_fs;
    k.refSize = gc.refSize;
    k.l_sum = 0;
    for (int q = 0; q < gc.n; ++q) k.l_sum += 1.0 * gc.w[q];
    for (int i = 0; i < 4; ++i) {
        k.s[i] = gc.s[i];
        for (int j = 0; j < 4; ++j) k.MM[i][j] = gc.MM[i][j];
    }
    for (int f = 0; f < 3; ++f) k.g[f] = c->prm.gravity[f];
    return k;
}

__device__ __forceinline__ bool v_single(uint8_t fl) { return (fl & F_BOUND) || (fl & F_FREE); }

// velocity CSR: row lengths and columns
__global__ void k_fs_row_len(int N, int dim, const uint8_t* __restrict__ flags, const int* __restrict__ nbr_ptr,
                             int* __restrict__ len) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (long long)dim * N) return;
    const int n = (int)(r % N);
    len[r] = v_single(flags[n]) ? 1 : dim * (nbr_ptr[n + 1] - nbr_ptr[n]);
}

__global__ void k_fs_fill_cols(int N, int dim, const uint8_t* __restrict__ flags, const int* __restrict__ nbr_ptr,
                               const int* __restrict__ nbr, const int* __restrict__ rp, int* __restrict__ col) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (long long)dim * N) return;
    const int n = (int)(r % N);
    if (v_single(flags[n])) {
        col[rp[r]] = (int)r;
        return;
    }
    const int b0 = nbr_ptr[n], deg = nbr_ptr[n + 1] - b0;
    for (int b = 0; b < dim; ++b)
        for (int t = 0; t < deg; ++t) col[rp[r] + b * deg + t] = nbr[b0 + t] + b * N;
}

// Values of pair p = (n, m): the velocity matrix block (M/dt + K, :63-118), L (:120-131) and M
// (:70-76), with the identity rows and columns of the boundary conditions.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_fs_pairs(int P, int N, int E, const int* __restrict__ pair_node,
                                                    const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                                                    const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                                                    const uint8_t* __restrict__ ne_loc, const int* __restrict__ conn,
                                                    const double* __restrict__ ed, const uint8_t* __restrict__ flags,
                                                    const uint8_t* __restrict__ gauge, const int* __restrict__ rpv,
                                                    FsConst k, double* __restrict__ valv, double* __restrict__ vall,
                                                    double* __restrict__ valm) {
    constexpr int NPE = DIM + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P) return;
    const int n = pair_node[t], m = nbr[t];
    const int b0 = nbr_ptr[n], deg = nbr_ptr[n + 1] - b0, rank = t - b0;
    const uint8_t fn = flags[n], fm = flags[m];
    const bool diag = m == n;
    double acc[DIM][DIM], ms = 0, le = 0;
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
        for (int b = 0; b < DIM; ++b) acc[a][b] = 0;
    const double inv_dt = 1 / k.dt;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        int j = -1;
#pragma unroll
        for (int jj = 0; jj < NPE; ++jj)
            if (__ldg(conn + (size_t)jj * E + e) == m) j = jj;
        if (j < 0) continue;
        const int i = ne_loc[q];
        const double ae = ed[e] * k.refSize;
        double gi[DIM], gj[DIM], dot = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f) {
            gi[f] = ed[(size_t)(2 + f * NPE + i) * E + e];
            gj[f] = ed[(size_t)(2 + f * NPE + j) * E + e];
            dot += gi[f] * gj[f];
        }
        const double mij = k.rho * k.MM[i][j] * ae;
        const double kf = ae * ed[(size_t)ed_ksum<DIM>() * E + e];
        // triplet order of one element: M/dt then K for each (d, d2) entry
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) {
                if (a == b) acc[a][b] += mij * inv_dt;
                acc[a][b] += kf * ((a == b ? dot : 0.0) + gi[b] * gj[a]);
            }
        ms += mij;
        le += ae * k.l_sum * dot;
    }
    // velocity prediction matrix
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
        const int rp = rpv[n + (size_t)a * N];
        if (v_single(fn)) {
            if (diag) valv[rp] = 1.0;
            continue;
        }
#pragma unroll
        for (int b = 0; b < DIM; ++b) valv[rp + b * deg + rank] = acc[a][b];
    }
    // pressure Laplacian: free and gauge nodes take identity rows and columns
    const bool lrow = (fn & F_FREE) || gauge[n], lcol = (fm & F_FREE) || gauge[m];
    vall[t] = lrow ? (diag ? 1.0 : 0.0) : ((lcol && !diag) ? 0.0 : (diag && lcol ? 1.0 : le));
    // velocity correction mass: bound and free nodes take identity rows and columns
    const bool mrow = v_single(fn), mcol = v_single(fm);
    valm[t] = mrow ? (diag ? 1.0 : 0.0) : ((mcol && !diag) ? 0.0 : ms);
}

// Right-hand side of the velocity prediction, node n (:133-150 in element order), the surface
// tension (:207-243), the node conditions and the Dirichlet column elimination of the rows of
// n in ascending column order (:245-257).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_fs_rhs_v(int N, int E, const int* __restrict__ ne_ptr,
                                                    const int* __restrict__ ne_elem, const uint8_t* __restrict__ ne_loc,
                                                    const int* __restrict__ conn, const double* __restrict__ ed,
                                                    const uint8_t* __restrict__ flags, const double* __restrict__ qp,
                                                    const double* __restrict__ vbc, const int* __restrict__ nbr_ptr,
                                                    const int* __restrict__ nbr, const int* __restrict__ rpv,
                                                    double* __restrict__ valv, const double* __restrict__ fst,
                                                    FsConst k, double* __restrict__ bv) {
    constexpr int NPE = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const uint8_t fl = flags[n];
    const double inv_dt = 1 / k.dt;
    double b[DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a) b[a] = 0;
    if (!v_single(fl)) {
        for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
            const int e = ne_elem[q];
            const int i = ne_loc[q];
            int nd[NPE];
            load_nodes<DIM>(conn, E, e, nd);
            const double ae = ed[e] * k.refSize;
            double sp = 0;  // sum_c s_c p_c
#pragma unroll
            for (int c = 0; c < NPE; ++c) sp += (ae * k.s[c]) * qp[(size_t)DIM * N + nd[c]];
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                const double F = ae * (k.rho * k.s[i] * k.g[a]);
                double mv = 0;
#pragma unroll
                for (int j = 0; j < NPE; ++j) mv += ((k.rho * k.MM[i][j] * ae) * inv_dt) * qp[(size_t)a * N + nd[j]];
                const double dtp = k.gfs * (ed[(size_t)(2 + a * NPE + i) * E + e] * sp);
                b[a] += F;
                b[a] += mv;
                b[a] += dtp;
            }
        }
    }
    if (fst)
#pragma unroll
        for (int a = 0; a < DIM; ++a) b[a] += fst[(size_t)a * N + n];
    if ((fl & F_FREE) && !(fl & F_BOUND))
#pragma unroll
        for (int a = 0; a < DIM; ++a) b[a] = qp[(size_t)a * N + n] + k.dt * k.g[a];
    if ((fl & F_BOUND) && (fl & F_DIRICHLET))
#pragma unroll
        for (int a = 0; a < DIM; ++a) b[a] = vbc[(size_t)a * N + n];
    if (!v_single(fl)) {
        const int b0 = nbr_ptr[n], deg = nbr_ptr[n + 1] - b0;
        for (int t = 0; t < deg; ++t) {
            const int m = nbr[b0 + t];
            const uint8_t fm = flags[m];
            if (m == n || !((fm & F_BOUND) && (fm & F_DIRICHLET))) continue;
#pragma unroll
            for (int c = 0; c < DIM; ++c) {
                const double r = vbc[(size_t)c * N + m];
#pragma unroll
                for (int a = 0; a < DIM; ++a) {
                    double* v = valv + rpv[n + (size_t)a * N] + c * deg + t;
                    b[a] -= *v * r;
                    *v = 0.0;
                }
            }
        }
    }
#pragma unroll
    for (int a = 0; a < DIM; ++a) bv[(size_t)a * N + n] = b[a];
}

// Right-hand side of the pressure system, node n (:270-300, :314-323).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_fs_rhs_p(int N, int E, const int* __restrict__ ne_ptr,
                                                    const int* __restrict__ ne_elem, const uint8_t* __restrict__ ne_loc,
                                                    const int* __restrict__ conn, const double* __restrict__ ed,
                                                    const uint8_t* __restrict__ flags, const uint8_t* __restrict__ gauge,
                                                    const double* __restrict__ vt, const double* __restrict__ qp,
                                                    FsConst k, double* __restrict__ bp) {
    constexpr int NPE = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const uint8_t fl = flags[n];
    double b = 0;
    if (!(fl & F_FREE) && !(fl & F_FREE_SURFACE)) {
        for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
            const int e = ne_elem[q];
            const int i = ne_loc[q];
            int nd[NPE];
            load_nodes<DIM>(conn, E, e, nd);
            const double ae = ed[e] * k.refSize;
            double dv = 0, gp[DIM];
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                gp[f] = 0;
#pragma unroll
                for (int j = 0; j < NPE; ++j) {
                    const double gfj = ed[(size_t)(2 + f * NPE + j) * E + e];
                    dv += (ae * k.s[i] * gfj) * vt[(size_t)f * N + nd[j]];
                    gp[f] += gfj * qp[(size_t)DIM * N + nd[j]];
                }
            }
            double lp = 0;
#pragma unroll
            for (int f = 0; f < DIM; ++f) lp += ed[(size_t)(2 + f * NPE + i) * E + e] * gp[f];
            b += -((k.rho / k.dt) * dv);
            b += k.gfs * ((ae * k.l_sum) * lp);
        }
    }
    if ((fl & F_FREE) || gauge[n]) b = 0;
    bp[n] = b;
}

// Right-hand side of the velocity correction, node n (:337-386, :398-410).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_fs_rhs_vc(int N, int E, const int* __restrict__ ne_ptr,
                                                     const int* __restrict__ ne_elem, const uint8_t* __restrict__ ne_loc,
                                                     const int* __restrict__ conn, const double* __restrict__ ed,
                                                     const uint8_t* __restrict__ flags, const double* __restrict__ dp,
                                                     FsConst k, double* __restrict__ bvc) {
    constexpr int NPE = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double b[DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a) b[a] = 0;
    if (!v_single(flags[n])) {
        for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
            const int e = ne_elem[q];
            const int i = ne_loc[q];
            int nd[NPE];
            load_nodes<DIM>(conn, E, e, nd);
            const double ae = ed[e] * k.refSize;
            double sp = 0;
#pragma unroll
            for (int c = 0; c < NPE; ++c) sp += (ae * k.s[c]) * dp[nd[c]];
#pragma unroll
            for (int a = 0; a < DIM; ++a) b[a] += k.dt * (ed[(size_t)(2 + a * NPE + i) * E + e] * sp);
        }
    }
#pragma unroll
    for (int a = 0; a < DIM; ++a) bvc[(size_t)a * N + n] = b[a];
}

// dp = p - gammaFS p_prev
__global__ void k_fs_dp(int N, const double* __restrict__ p, const double* __restrict__ pprev, double gfs,
                        double* __restrict__ dp) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < N) dp[n] = p[n] - gfs * pprev[n];
}

// v = v~ + dv into the iterate
__global__ void k_fs_sum(int n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] + b[i];
}

// sum over the non-free nodes of (x - xp)^2 and xp^2 for nf fields
__global__ void __launch_bounds__(BLOCK) k_fs_res(int N, int nf, const double* __restrict__ x,
                                                  const double* __restrict__ xp, const uint8_t* __restrict__ flags,
                                                  double* __restrict__ partials, unsigned* __restrict__ ticket,
                                                  double* __restrict__ out) {
    __shared__ double sh[32];
    double num = 0, den = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        if (flags[n] & F_FREE) continue;
        for (int f = 0; f < nf; ++f) {
            const double d = x[(size_t)f * N + n] - xp[(size_t)f * N + n];
            num += d * d;
            den += xp[(size_t)f * N + n] * xp[(size_t)f * N + n];
        }
    }
    grid_sum_last<BLOCK>(num, partials, ticket, sh, out);
    __syncthreads();
    grid_sum_last<BLOCK>(den, partials + gridDim.x, ticket + 1, sh, out + 1);
}

// Work vectors (doubles, offsets in units of N): bv (dim), bp, bvc (dim), vt (dim), dv (dim),
// dp, q_iter_prev (dim + 1)
struct FsVec {
    double *bv, *bp, *bvc, *vt, *dv, *dp, *qip;
};

FsVec fs_vec(pfg_ctx* c) {
    const size_t N = std::max(c->N, 1), d = c->dim;
    double* w = ptr<double>(c->fs_vec);
    FsVec v;
    v.bv = w;
    v.bp = v.bv + d * N;
    v.bvc = v.bp + N;
    v.vt = v.bvc + d * N;
    v.dv = v.vt + d * N;
    v.dp = v.dv + d * N;
    v.qip = v.dp + N;
    return v;
}

// Gauge nodes: per connected group of elements its smallest free-surface node, else its
// smallest node (union-find over the elements' nodes); every free-surface node when fs_dir.
std::vector<uint8_t> fs_gauge(int N, int E, int npe, const std::vector<int>& conn, const std::vector<uint8_t>& flags,
                              bool fs_dir) {
    std::vector<uint8_t> g(N, 0);
    if (fs_dir) {
        for (int n = 0; n < N; ++n) g[n] = (flags[n] & F_FREE_SURFACE) ? 1 : 0;
        return g;
    }
    std::vector<int> parent(N);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int x) {
        while (parent[x] != x) x = parent[x] = parent[parent[x]];
        return x;
    };
    std::vector<uint8_t> used(N, 0);
    for (int e = 0; e < E; ++e) {
        const int a = conn[e];
        used[a] = 1;
        for (int k = 1; k < npe; ++k) {
            const int b = conn[(size_t)k * E + e];
            used[b] = 1;
            const int ra = find(a), rb = find(b);
            if (ra != rb) parent[std::max(ra, rb)] = std::min(ra, rb);
        }
    }
    // best node per root: free-surface nodes first, then the smallest index
    std::vector<int> best(N, -1);
    for (int n = 0; n < N; ++n) {
        if (!used[n]) continue;
        const int r = find(n);
        const int cur = best[r];
        const bool fs = flags[n] & F_FREE_SURFACE;
        if (cur < 0 || (fs && !(flags[cur] & F_FREE_SURFACE))) best[r] = n;
    }
    for (int n = 0; n < N; ++n)
        if (best[n] >= 0) g[best[n]] = 1;
    return g;
}

template <int DIM>
int fs_assemble(pfg_ctx* c, const FsConst& k, const double* qprev) {
    const int N = c->N, E = c->E;
    prof_begin(c, PH_PSPG_PAIRS);
    if (c->P > 0)
        k_fs_pairs<DIM><<<div_up(c->P, BLOCK), BLOCK, 0, c->stream>>>(
            c->P, N, E, ptr<int>(c->pair_node), ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<int>(c->ne_ptr),
            ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn), ptr<double>(c->edata),
            ptr<uint8_t>(c->flags), ptr<uint8_t>(c->fs_gauge), ptr<int>(c->fs_rp), k, ptr<double>(c->fs_val),
            ptr<double>(c->fs_lval), ptr<double>(c->fs_mval));
    prof_end(c, PH_PSPG_PAIRS);
    prof_begin(c, PH_PSPG_RHS);
    const FstArgs fa = fst_args(c);
    if (fa.nodes)
        k_fst<DIM, double><<<div_up(fa.n_nodes, BLOCK), BLOCK, 0, c->stream>>>(
            fa, E, ptr<int>(c->conn), PosF64{ptr<double>(c->pos), N}, N, ptr<double>(c->fst_force));
    const FsVec w = fs_vec(c);
    k_fs_rhs_v<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(
        N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn),
        ptr<double>(c->edata), ptr<uint8_t>(c->flags), qprev, ptr<double>(c->vbc), ptr<int>(c->nbr_ptr),
        ptr<int>(c->nbr), ptr<int>(c->fs_rp), ptr<double>(c->fs_val), fst_force<double>(c), k, w.bv);
    prof_end(c, PH_PSPG_RHS);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

// One CG solve of the scalar pair-layout matrix val (L or M) or of the velocity CSR.
int fs_cg(pfg_ctx* c, int n, const int* rp, const int* col, const double* val, const double* b, double* x,
          pfg_step_status* st, bool* ok) {
    int its = 0;
    prof_begin(c, PH_KRYLOV_ITER);
    int rc = cg_solve(c, n, rp, col, val, b, x, ptr<double>(c->fs_cg), ptr<double>(c->fs_red), c->prm.krylov_rel_tol,
                      c->prm.krylov_abs_tol, c->prm.krylov_max_iter, &its, ok);
    prof_end(c, PH_KRYLOV_ITER);
    st->krylov_iterations += its;
    return rc;
}

template <int DIM>
int fs_step_dim(pfg_ctx* c, double dt, pfg_step_status* st) {
    const int N = c->N, E = c->E, R = c->R;
    std::memset(st, 0, sizeof(*st));
    st->dt = dt;
    double* q = ptr<double>(c->q);
    double* qprev = ptr<double>(c->q_prev);
    const FsVec w = fs_vec(c);
    const FsConst k = fs_const(c, dt);
    int rc;
    PFG_CUDA(c, cudaMemcpyAsync(c->pos_save.p, c->pos.p, sizeof(double) * DIM * N, cudaMemcpyDeviceToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(qprev, q, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(w.qip, q, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
    // the iterate starts from the previous step (CG guesses; the reference's direct solves need none)
    PFG_CUDA(c, cudaMemcpyAsync(w.vt, q, sizeof(double) * DIM * N, cudaMemcpyDeviceToDevice, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(w.dv, 0, sizeof(double) * DIM * N, c->stream));
    double* red = ptr<double>(c->fs_red);
    double* res_out = red + 3 * (size_t)c->max_grid + 48;
    unsigned* res_ticket = reinterpret_cast<unsigned*>(res_out + 8);
    double* p_it = q + (size_t)DIM * N;
    const int grid = std::max(1, std::min(c->max_grid, div_up(N, BLOCK)));
    double res = INFINITY;
    int it = 0;
    bool ok = true;
    while (res > c->prm.picard_min_res) {
        if (it > c->prm.picard_max_iter) {
            ok = false;
            break;
        }
        if ((rc = pspg_elem_prep(c, dt, q)) || (rc = fs_assemble<DIM>(c, k, qprev))) return rc;
        bool solved = false;
        if ((rc = fs_cg(c, DIM * N, ptr<int>(c->fs_rp), ptr<int>(c->fs_col), ptr<double>(c->fs_val), w.bv, w.vt, st,
                        &solved)))
            return rc;
        if (!solved) {
            ok = false;
            break;
        }
        prof_begin(c, PH_PSPG_RHS);
        k_fs_rhs_p<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(
            N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn),
            ptr<double>(c->edata), ptr<uint8_t>(c->flags), ptr<uint8_t>(c->fs_gauge), w.vt, qprev, k, w.bp);
        prof_end(c, PH_PSPG_RHS);
        PFG_CHECK_LAUNCH(c);
        // p iterate in place (guess: the previous iterate)
        if ((rc = fs_cg(c, N, ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<double>(c->fs_lval), w.bp, p_it, st,
                        &solved)))
            return rc;
        if (!solved) {
            ok = false;
            break;
        }
        k_fs_dp<<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, p_it, qprev + (size_t)DIM * N, k.gfs, w.dp);
        prof_begin(c, PH_PSPG_RHS);
        k_fs_rhs_vc<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(
            N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn),
            ptr<double>(c->edata), ptr<uint8_t>(c->flags), w.dp, k, w.bvc);
        prof_end(c, PH_PSPG_RHS);
        PFG_CHECK_LAUNCH(c);
        for (int a = 0; a < DIM && ok; ++a) {
            if ((rc = fs_cg(c, N, ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<double>(c->fs_mval),
                            w.bvc + (size_t)a * N, w.dv + (size_t)a * N, st, &solved)))
                return rc;
            ok = solved;
        }
        if (!ok) break;
        k_fs_sum<<<div_up(DIM * N, BLOCK), BLOCK, 0, c->stream>>>(DIM * N, w.vt, w.dv, q);
        if ((rc = pspg_update_positions(c, dt, q))) return rc;
        // residual (:568-629): relative change of v (and p) over the non-free nodes
        prof_begin(c, PH_RESIDUAL);
        k_fs_res<<<grid, BLOCK, 0, c->stream>>>(N, DIM, q, w.qip, ptr<uint8_t>(c->flags), red, res_ticket, res_out);
        if (c->prm.residual == PFG_RES_U_P)
            k_fs_res<<<grid, BLOCK, 0, c->stream>>>(N, 1, p_it, w.qip + (size_t)DIM * N, ptr<uint8_t>(c->flags), red,
                                                    res_ticket, res_out + 2);
        prof_end(c, PH_RESIDUAL);
        PFG_CHECK_LAUNCH(c);
        PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, res_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaMemcpyAsync(w.qip, q, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        const double* h = c->h_scalars;
        const double rv = h[1] == 0.0 ? DBL_MAX : std::sqrt(h[0] / h[1]);
        double rp = 0.0;
        if (c->prm.residual == PFG_RES_U_P) rp = h[3] == 0.0 ? DBL_MAX : std::sqrt(h[2] / h[3]);
        res = std::max(rv, rp);
        st->residual = res;
        ++it;
        if (std::isnan(res)) {
            ok = false;
            break;
        }
    }
    st->picard_iterations = it;
    if (!ok) {
        PFG_CUDA(c, cudaMemcpyAsync(c->pos.p, c->pos_save.p, sizeof(double) * DIM * N, cudaMemcpyDeviceToDevice,
                                    c->stream));
        PFG_CUDA(c, cudaMemcpyAsync(q, qprev, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    st->converged = ok ? 1 : 0;
    return PFG_OK;
}

}  // namespace

// Buffers and patterns of the fractional step for the current mesh.
int fs_alloc(pfg_ctx* c) {
    const int N = c->N, dim = c->dim;
    const size_t Nz = std::max(N, 1), P = std::max(c->P, 1);
    const long long Rv = (long long)dim * N;
    int rc;
    DBuf len, tmp;
    auto cleanup = [&]() {
        release(len);
        release(tmp);
    };
    if ((rc = ensure(c, c->fs_gauge, Nz)) || (rc = ensure(c, c->fs_rp, sizeof(int) * ((size_t)Rv + 1))) ||
        (rc = ensure(c, c->fs_lval, sizeof(double) * P)) || (rc = ensure(c, c->fs_mval, sizeof(double) * P)) ||
        (rc = ensure(c, c->fs_vec, sizeof(double) * Nz * (5 * (size_t)dim + 3))) ||
        (rc = ensure(c, c->fs_cg, sizeof(double) * CG_VECTORS * (size_t)dim * Nz)) ||
        (rc = ensure(c, c->fs_red, sizeof(double) * (3 * (size_t)std::max(c->max_grid, 1) + 64))) ||
        (rc = ensure(c, len, sizeof(int) * (size_t)std::max<long long>(Rv, 1)))) {
        cleanup();
        return rc;
    }
    PFG_CUDA(c, cudaMemsetAsync(c->fs_red.p, 0, sizeof(double) * (3 * (size_t)std::max(c->max_grid, 1) + 64),
                                c->stream));
    const std::vector<uint8_t> g =
        fs_gauge(N, c->E, c->npe, c->h_conn, c->h_flags, c->prm.fs_pressure_dirichlet != 0);
    PFG_CUDA(c, cudaMemcpyAsync(c->fs_gauge.p, g.data(), N, cudaMemcpyHostToDevice, c->stream));
    if (Rv > 0) {
        k_fs_row_len<<<div_up(Rv, BLOCK), BLOCK, 0, c->stream>>>(N, dim, ptr<uint8_t>(c->flags), ptr<int>(c->nbr_ptr),
                                                                  ptr<int>(len));
        PFG_CHECK_LAUNCH(c);
    }
    if ((rc = scan_exclusive(c, ptr<int>(len), ptr<int>(c->fs_rp), (int)Rv, tmp))) {
        cleanup();
        return rc;
    }
    int nnz = 0;
    PFG_CUDA(c, cudaMemcpyAsync(&nnz, ptr<int>(c->fs_rp) + Rv, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    if ((rc = ensure(c, c->fs_col, sizeof(int) * (size_t)std::max(nnz, 1))) ||
        (rc = ensure(c, c->fs_val, sizeof(double) * (size_t)std::max(nnz, 1)))) {
        cleanup();
        return rc;
    }
    if (Rv > 0) {
        k_fs_fill_cols<<<div_up(Rv, BLOCK), BLOCK, 0, c->stream>>>(N, dim, ptr<uint8_t>(c->flags),
                                                                    ptr<int>(c->nbr_ptr), ptr<int>(c->nbr),
                                                                    ptr<int>(c->fs_rp), ptr<int>(c->fs_col));
        PFG_CHECK_LAUNCH(c);
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    cleanup();
    return PFG_OK;
}

int fs_picard_step(pfg_ctx* c, double dt, pfg_step_status* st) {
    return c->dim == 2 ? fs_step_dim<2>(c, dt, st) : fs_step_dim<3>(c, dt, st);
}

}  // namespace pfg
