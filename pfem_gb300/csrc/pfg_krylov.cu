// Node-block-Jacobi preconditioned BiCGSTAB on the assembled CSR system, FP64.
//
// Stands beside the reference's direct solve (Eigen SparseLU<COLAMD>,
// MomContEquationPSPG.inl:281-291).  The PSPG matrix is a saddle-point system whose pressure
// rows have a tiny stabilisation diagonal (tau L) next to O(1) divergence entries, so point
// Jacobi leaves BiCGSTAB stagnating; the preconditioner here inverts, for every node, the
// (dim+1)x(dim+1) block coupling its velocity and pressure unknowns (Gauss-Jordan with partial
// pivoting), which is as parallel as point Jacobi.
//
// SpMV is sub-warp-per-row (G lanes per row, G chosen from the mean row length) with shuffle
// reductions.  All scalars (rho, alpha, omega, the convergence flag) stay on the device: every
// dot product is reduced deterministically by the last block of its kernel, so an iteration
// is five kernels and no host round trip; the host polls the residual every few iterations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

// device scalar slots (doubles after the partials)
enum : int {
    S_RHO = 0,
    S_RHO_OLD,
    S_ALPHA,
    S_OMEGA,
    S_RR,
    S_BB,
    S_TOL2,
    S_DONE,   // 0 running, 1 converged, 2 breakdown
    S_ITERS,
    S_RV,
    S_TS,
    S_TT,
    S_COUNT
};

enum : int { V_R = 0, V_RHAT, V_P, V_V, V_S, V_T, V_PHAT, V_SHAT, V_STAGE1, V_STAGE2, V_SPARE0, V_SPARE1, V_COUNT };

struct KPtrs {
    double* partials;  // 2 * max_grid
    double* sc;        // S_COUNT
    unsigned* ticket;  // 4
};

KPtrs kptrs(pfg_ctx* c) {
    double* red = ptr<double>(c->red);
    KPtrs k;
    k.partials = red;
    k.sc = red + 4 * c->max_grid;
    k.ticket = reinterpret_cast<unsigned*>(red + 4 * c->max_grid + 32);
    return k;
}

// Two-value deterministic grid reduction (see grid_sum_last).
template <int NT>
__device__ __forceinline__ bool grid_sum2_last(double a, double b, double* partials, unsigned* ticket, double* sh,
                                               double& ra, double& rb) {
    a = block_sum<NT>(a, sh);
    b = block_sum<NT>(b, sh);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = a;
        partials[gridDim.x + blockIdx.x] = b;
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double sa = 0, sb = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += NT) {
        sa += ((volatile double*)partials)[i];
        sb += ((volatile double*)partials)[gridDim.x + i];
    }
    sa = block_sum<NT>(sa, sh);
    sb = block_sum<NT>(sb, sh);
    ra = sa;
    rb = sb;
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// Row r of A times x, reduced over the G lanes of a sub-warp; valid on lane 0 of the group.
// Every lane of the warp calls it the same number of times (inactive rows have act = false).
template <int G>
__device__ __forceinline__ double row_dot(int r, bool act, const int* __restrict__ rp, const int* __restrict__ col,
                                          const double* __restrict__ val, const double* __restrict__ x, int lane) {
    const int b = act ? rp[r] : 0, e = act ? rp[r + 1] : 0;
    double s = 0;
    for (int k = b + lane; k < e; k += G) s += val[k] * __ldg(x + col[k]);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    return s;
}

#define ROW_LOOP_BEGIN(G)                                                     \
    const int lane = threadIdx.x % G;                                         \
    const int gpw = 32 / G;                                                   \
    const int wglob = (blockIdx.x * blockDim.x + threadIdx.x) / 32;           \
    const int nwarps = gridDim.x * blockDim.x / 32;                           \
    for (int r0 = wglob * gpw; r0 < R; r0 += nwarps * gpw) {                  \
        const int r = r0 + (threadIdx.x & 31) / G;                            \
        const bool act = r < R;

#define ROW_LOOP_END }

// Node-block inverse: B[f1][f2] = A[(n,f1),(n,f2)], inverted by Gauss-Jordan with partial
// pivoting.  Stored field-major: binv[(f1*(DIM+1)+f2)*N + n].  A singular block (never seen
// for assembled PSPG blocks) falls back to the inverse of its diagonal.
template <int DIM>
__global__ void k_block_inverse(int N, const int* __restrict__ rp, const double* __restrict__ val,
                                const int* __restrict__ diag, double* __restrict__ binv, int* __restrict__ err) {
    constexpr int B = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double a[B][2 * B];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        const int r = n + f1 * N;
        const int dp = diag[r];
        const int b0 = rp[r], len = rp[r + 1] - b0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            a[f1][f2] = 0;
            a[f1][B + f2] = (f1 == f2) ? 1.0 : 0.0;
        }
        if (len == 1) {
            a[f1][f1] = val[dp];
        } else {
            const int deg = len / B;
            const int self = dp - b0 - f1 * deg;
#pragma unroll
            for (int f2 = 0; f2 < B; ++f2) a[f1][f2] = val[b0 + f2 * deg + self];
        }
    }
    double dg[B];
#pragma unroll
    for (int f = 0; f < B; ++f) dg[f] = a[f][f];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < B; ++k) {
        int piv = k;
        double best = fabs(a[k][k]);
#pragma unroll
        for (int i = k + 1; i < B; ++i)
            if (fabs(a[i][k]) > best) {
                best = fabs(a[i][k]);
                piv = i;
            }
        if (best == 0.0) ok = false;
        if (piv != k) {
#pragma unroll
            for (int j = 0; j < 2 * B; ++j) {
                const double t = a[k][j];
                a[k][j] = a[piv][j];
                a[piv][j] = t;
            }
        }
        const double inv = ok ? 1.0 / a[k][k] : 0.0;
#pragma unroll
        for (int j = 0; j < 2 * B; ++j) a[k][j] *= inv;
#pragma unroll
        for (int i = 0; i < B; ++i) {
            if (i == k) continue;
            const double f = a[i][k];
#pragma unroll
            for (int j = 0; j < 2 * B; ++j) a[i][j] -= f * a[k][j];
        }
    }
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            double v = a[f1][B + f2];
            if (!ok) v = (f1 == f2) ? (dg[f1] != 0.0 ? 1.0 / dg[f1] : 1.0) : 0.0;
            binv[(size_t)(f1 * B + f2) * N + n] = v;
        }
    if (!ok) atomicOr(err, ERR_KRYLOV_BREAKDOWN);
}

// z_n = Binv_n y_n for all fields of node n
template <int DIM>
__device__ __forceinline__ void block_apply(int n, int N, const double* __restrict__ binv, const double (&y)[DIM + 1],
                                            double* __restrict__ z) {
    constexpr int B = DIM + 1;
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        double s = 0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) s += binv[(size_t)(f1 * B + f2) * N + n] * y[f2];
        z[(size_t)f1 * N + n] = s;
    }
}

// r = b - A x ; rhat = r ; p = v = 0 ; dots r.r and b.b
template <int G>
__global__ void __launch_bounds__(BLOCK) k_init(int R, const int* __restrict__ rp, const int* __restrict__ col,
                                                const double* __restrict__ val, const double* __restrict__ b,
                                                const double* __restrict__ x, double* __restrict__ V, size_t ld,
                                                KPtrs kp, double rtol, double atol) {
    __shared__ double sh[32];
    double rr = 0, bb = 0;
    ROW_LOOP_BEGIN(G)
    double ax = row_dot<G>(r, act, rp, col, val, x, lane);
    if (act && lane == 0) {
        const double rv = b[r] - ax;
        V[V_R * ld + r] = rv;
        V[V_RHAT * ld + r] = rv;
        V[V_P * ld + r] = 0;
        V[V_V * ld + r] = 0;
        rr += rv * rv;
        bb += b[r] * b[r];
    }
    ROW_LOOP_END
    double trr, tbb;
    if (grid_sum2_last<BLOCK>(rr, bb, kp.partials, kp.ticket, sh, trr, tbb) && threadIdx.x == 0) {
        double* sc = kp.sc;
        sc[S_RR] = trr;
        sc[S_BB] = tbb;
        sc[S_RHO] = trr;
        sc[S_RHO_OLD] = 1;
        sc[S_ALPHA] = 1;
        sc[S_OMEGA] = 1;
        const double tol = fmax(rtol * sqrt(tbb), atol);
        sc[S_TOL2] = tol * tol;
        sc[S_ITERS] = 0;
        sc[S_DONE] = (trr <= tol * tol) ? 1.0 : 0.0;
    }
}

// beta = (rho/rho_old)(alpha/omega); p = r + beta (p - omega v); phat = Binv p   (per node)
template <int DIM>
__global__ void k_update_p(int N, double* __restrict__ V, size_t ld, const double* __restrict__ binv,
                           const double* __restrict__ sc) {
    if (sc[S_DONE] != 0.0) return;
    const double beta = (sc[S_RHO] / sc[S_RHO_OLD]) * (sc[S_ALPHA] / sc[S_OMEGA]);
    const double om = sc[S_OMEGA];
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        double p[DIM + 1];
#pragma unroll
        for (int f = 0; f <= DIM; ++f) {
            const size_t r = (size_t)f * N + n;
            p[f] = V[V_R * ld + r] + beta * (V[V_P * ld + r] - om * V[V_V * ld + r]);
            V[V_P * ld + r] = p[f];
        }
        block_apply<DIM>(n, N, binv, p, V + V_PHAT * ld);
    }
}

// v = A phat ; alpha = rho / (rhat . v)
template <int G>
__global__ void __launch_bounds__(BLOCK) k_spmv_alpha(int R, const int* __restrict__ rp, const int* __restrict__ col,
                                                      const double* __restrict__ val, double* __restrict__ V,
                                                      size_t ld, KPtrs kp) {
    __shared__ double sh[32];
    if (kp.sc[S_DONE] != 0.0) return;
    double acc = 0;
    const double* phat = V + V_PHAT * ld;
    ROW_LOOP_BEGIN(G)
    double y = row_dot<G>(r, act, rp, col, val, phat, lane);
    if (act && lane == 0) {
        V[V_V * ld + r] = y;
        acc += V[V_RHAT * ld + r] * y;
    }
    ROW_LOOP_END
    __shared__ bool last;
    double tot = block_sum<BLOCK>(acc, sh);
    if (threadIdx.x == 0) {
        kp.partials[blockIdx.x] = tot;
        __threadfence();
        last = atomicAdd(kp.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) s += ((volatile double*)kp.partials)[i];
    s = block_sum<BLOCK>(s, sh);
    if (threadIdx.x == 0) {
        *kp.ticket = 0u;
        double* sc = kp.sc;
        sc[S_RV] = s;
        if (s == 0.0 || !isfinite(s)) {
            sc[S_DONE] = 2;
        } else {
            sc[S_ALPHA] = sc[S_RHO] / s;
        }
    }
}

// s = r - alpha v ; shat = Binv s   (per node)
template <int DIM>
__global__ void k_update_s(int N, double* __restrict__ V, size_t ld, const double* __restrict__ binv,
                           const double* __restrict__ sc) {
    if (sc[S_DONE] != 0.0) return;
    const double al = sc[S_ALPHA];
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        double s[DIM + 1];
#pragma unroll
        for (int f = 0; f <= DIM; ++f) {
            const size_t r = (size_t)f * N + n;
            s[f] = V[V_R * ld + r] - al * V[V_V * ld + r];
            V[V_S * ld + r] = s[f];
        }
        block_apply<DIM>(n, N, binv, s, V + V_SHAT * ld);
    }
}

// t = A shat ; omega = (t.s)/(t.t)
template <int G>
__global__ void __launch_bounds__(BLOCK) k_spmv_omega(int R, const int* __restrict__ rp, const int* __restrict__ col,
                                                      const double* __restrict__ val, double* __restrict__ V,
                                                      size_t ld, KPtrs kp) {
    __shared__ double sh[32];
    if (kp.sc[S_DONE] != 0.0) return;
    double ts = 0, tt = 0;
    const double* shat = V + V_SHAT * ld;
    ROW_LOOP_BEGIN(G)
    double y = row_dot<G>(r, act, rp, col, val, shat, lane);
    if (act && lane == 0) {
        V[V_T * ld + r] = y;
        ts += y * V[V_S * ld + r];
        tt += y * y;
    }
    ROW_LOOP_END
    double rts, rtt;
    if (grid_sum2_last<BLOCK>(ts, tt, kp.partials, kp.ticket, sh, rts, rtt) && threadIdx.x == 0) {
        double* sc = kp.sc;
        sc[S_TS] = rts;
        sc[S_TT] = rtt;
        // t = 0: s is already the solution update; take the half step x += alpha phat
        sc[S_OMEGA] = (rtt == 0.0 || !isfinite(rtt)) ? 0.0 : rts / rtt;
    }
}

// x += alpha phat + omega shat ; r = s - omega t ; rho_new = rhat.r ; rr = r.r
__global__ void __launch_bounds__(BLOCK) k_update_x(int R, double* __restrict__ x, double* __restrict__ V, size_t ld,
                                                    KPtrs kp) {
    __shared__ double sh[32];
    if (kp.sc[S_DONE] != 0.0) return;
    const double al = kp.sc[S_ALPHA], om = kp.sc[S_OMEGA];
    double rh = 0, rr = 0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x) {
        x[r] += al * V[V_PHAT * ld + r] + om * V[V_SHAT * ld + r];
        const double rv = V[V_S * ld + r] - om * V[V_T * ld + r];
        V[V_R * ld + r] = rv;
        rh += V[V_RHAT * ld + r] * rv;
        rr += rv * rv;
    }
    double trh, trr;
    if (grid_sum2_last<BLOCK>(rh, rr, kp.partials, kp.ticket, sh, trh, trr) && threadIdx.x == 0) {
        double* sc = kp.sc;
        sc[S_RHO_OLD] = sc[S_RHO];
        sc[S_RHO] = trh;
        sc[S_RR] = trr;
        sc[S_ITERS] += 1;
        if (!isfinite(trr))
            sc[S_DONE] = 2;
        else if (trr <= sc[S_TOL2])
            sc[S_DONE] = 1;
        else if (trh == 0.0 || om == 0.0)
            sc[S_DONE] = 2;
    }
}

// ||b - A x||_2 (Picard "Ax_f" residual, MomContEquationPSPG.inl:366-371)
template <int G>
__global__ void __launch_bounds__(BLOCK) k_residual(int R, const int* __restrict__ rp, const int* __restrict__ col,
                                                    const double* __restrict__ val, const double* __restrict__ b,
                                                    const double* __restrict__ x, double* partials, unsigned* ticket,
                                                    double* out) {
    __shared__ double sh[32];
    double rr = 0;
    ROW_LOOP_BEGIN(G)
    double ax = row_dot<G>(r, act, rp, col, val, x, lane);
    if (act && lane == 0) {
        const double d = ax - b[r];
        rr += d * d;
    }
    ROW_LOOP_END
    grid_sum_last<BLOCK>(rr, partials, ticket, sh, out);
}

int lanes_per_row(pfg_ctx* c) {
    const double mean = c->R ? (double)c->nnz / c->R : 1.0;
    if (mean <= 6) return 4;
    if (mean <= 24) return 8;
    if (mean <= 48) return 16;
    return 32;
}

template <int G, int DIM>
int bicgstab_g(pfg_ctx* c, double* d_x, int* iters, double* res) {
    const int R = c->R, N = c->N;
    double* V = ptr<double>(c->kv);
    const size_t ld = (size_t)R;
    KPtrs kp = kptrs(c);
    const int* rp = ptr<int>(c->row_ptr);
    const int* col = ptr<int>(c->col);
    const double* val = ptr<double>(c->val);
    double* binv = ptr<double>(c->binv);
    const int grid_rows = std::max(1, std::min(c->max_grid, div_up((long long)R * G, BLOCK)));
    const int grid_vec = std::max(1, std::min(c->max_grid, div_up(R, BLOCK)));
    const int grid_node = std::max(1, std::min(c->max_grid, div_up(N, BLOCK)));
    k_block_inverse<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, rp, val, ptr<int>(c->diag_pos), binv,
                                                                    ptr<int>(c->err_word));
    k_init<G><<<grid_rows, BLOCK, 0, c->stream>>>(R, rp, col, val, ptr<double>(c->rhs), d_x, V, ld, kp,
                                                  c->prm.krylov_rel_tol, c->prm.krylov_abs_tol);
    PFG_CHECK_LAUNCH(c);
    const int max_it = std::max(1, c->prm.krylov_max_iter);
    const int chunk = 8;
    int done_it = 0;
    double* h = c->h_scalars;
    while (done_it < max_it) {
        const int n = std::min(chunk, max_it - done_it);
        for (int k = 0; k < n; ++k) {
            prof_begin(c, PH_KRYLOV_ITER);
            k_update_p<DIM><<<grid_node, BLOCK, 0, c->stream>>>(N, V, ld, binv, kp.sc);
            prof_begin(c, PH_KRYLOV_SPMV);
            k_spmv_alpha<G><<<grid_rows, BLOCK, 0, c->stream>>>(R, rp, col, val, V, ld, kp);
            prof_end(c, PH_KRYLOV_SPMV);
            k_update_s<DIM><<<grid_node, BLOCK, 0, c->stream>>>(N, V, ld, binv, kp.sc);
            prof_begin(c, PH_KRYLOV_SPMV);
            k_spmv_omega<G><<<grid_rows, BLOCK, 0, c->stream>>>(R, rp, col, val, V, ld, kp);
            prof_end(c, PH_KRYLOV_SPMV);
            k_update_x<<<grid_vec, BLOCK, 0, c->stream>>>(R, d_x, V, ld, kp);
            prof_end(c, PH_KRYLOV_ITER);
        }
        PFG_CHECK_LAUNCH(c);
        done_it += n;
        PFG_CUDA(c, cudaMemcpyAsync(h, kp.sc, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (h[S_DONE] != 0.0) break;
    }
    *iters = (int)h[S_ITERS];
    *res = std::sqrt(h[S_RR]);
    return PFG_OK;
}

template <int G>
int residual_g(pfg_ctx* c, const double* d_x, double* res) {
    const int R = c->R;
    KPtrs kp = kptrs(c);
    const int grid_rows = std::max(1, std::min(c->max_grid, div_up((long long)R * G, BLOCK)));
    double* out = kp.sc + S_COUNT;
    prof_begin(c, PH_RESIDUAL);
    k_residual<G><<<grid_rows, BLOCK, 0, c->stream>>>(R, ptr<int>(c->row_ptr), ptr<int>(c->col), ptr<double>(c->val),
                                                      ptr<double>(c->rhs), d_x, kp.partials, kp.ticket, out);
    prof_end(c, PH_RESIDUAL);
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, out, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    *res = std::sqrt(c->h_scalars[0]);
    return PFG_OK;
}

template <int DIM>
int bicgstab_dim(pfg_ctx* c, double* d_x, int* iters, double* res) {
    switch (lanes_per_row(c)) {
        case 4: return bicgstab_g<4, DIM>(c, d_x, iters, res);
        case 8: return bicgstab_g<8, DIM>(c, d_x, iters, res);
        case 16: return bicgstab_g<16, DIM>(c, d_x, iters, res);
        default: return bicgstab_g<32, DIM>(c, d_x, iters, res);
    }
}

}  // namespace

int krylov_alloc(pfg_ctx* c) {
    int rc = ensure(c, c->kv, sizeof(double) * V_COUNT * (size_t)std::max(c->R, 1));
    if (rc) return rc;
    return ensure(c, c->binv, sizeof(double) * (size_t)(c->dim + 1) * (c->dim + 1) * std::max(c->N, 1));
}

int bicgstab(pfg_ctx* c, double* d_x, int* iters, double* res) {
    return c->dim == 2 ? bicgstab_dim<2>(c, d_x, iters, res) : bicgstab_dim<3>(c, d_x, iters, res);
}

int spmv_residual_norm(pfg_ctx* c, const double* d_x, double* res) {
    switch (lanes_per_row(c)) {
        case 4: return residual_g<4>(c, d_x, res);
        case 8: return residual_g<8>(c, d_x, res);
        case 16: return residual_g<16>(c, d_x, res);
        default: return residual_g<32>(c, d_x, res);
    }
}

}  // namespace pfg
