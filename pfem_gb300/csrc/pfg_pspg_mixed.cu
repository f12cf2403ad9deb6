// Mixed-precision incompressible PSPG step: FP32 assembly and FP32 Krylov iterations, FP64
// geometry and an FP64 matrix-free residual that drives iterative refinement.
//
// The reference solves A(q) q = b(q) with a direct FP64 LU at every Picard iteration
// (MomContEquationPSPG.inl:281-291).  Here the matrix is assembled in FP32 (the FP32 copy
// only steers the correction solves), and every residual r = b - A x is evaluated in FP64
// straight from the element formulas (no FP64 matrix is stored).  One linear solve is
//     x <- x + BiCGSTAB_fp32(A32, r)   until ||r|| <= max(rel_tol ||b||, abs_tol),
// the classic mixed-precision iterative refinement: its fixed point is the FP64 system's
// solution, so the Picard iterates agree with the FP64 path to the refinement tolerance.
// The residual evaluated right after the Picard re-assembly is, at the same time, the
// Picard "Ax_f" residual (:366-371) and the first refinement residual of the next solve.
//
// Everything runs over "instances": independent meshes stored back to back in one node /
// element numbering (one instance for a single mesh).  Node-wise kernels run on segments of
// NB nodes that never straddle two instances, so every dot product and norm is reduced per
// instance, deterministically, by the last segment of that instance to finish.  Instances
// carry their own rho, mu, dt, Picard counters and Krylov scalars; converged or failed
// instances drop out of the launches while the others keep iterating.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

constexpr int NB = 128;          // nodes per segment (= threads of the node kernels)
constexpr int SPMV_BLOCK = 256;  // threads of the segment SpMV kernels

// per-instance int fields
enum : int { I_B0 = 0, I_B1, I_N0, I_N1, I_ACTIVE, I_STATUS, I_IT, I_KIT, I_TICKET, I_COUNT = 12 };
// per-instance double fields
enum : int { D_RHO = 0, D_MU, D_DT, D_RR, D_BB, D_RES, D_RES_FIRST, D_PAD, D_COUNT = 8 };
// per-instance FP32 Krylov scalars
enum : int { M_RHO = 0, M_RHO_OLD, M_ALPHA, M_OMEGA, M_RR, M_TOL2, M_DONE, M_ITERS, M_COUNT = 8 };
// FP32 Krylov vectors
enum : int { W_R = 0, W_RHAT, W_P, W_V, W_S, W_T, W_PHAT, W_SHAT, W_COUNT };
// device counters
enum : int { C_NEED = 0, C_ACTIVE = 1 };

struct Mx {
    const int* seg;   // [3 * n_seg]: instance, first node, end node
    int* ii;          // [I_COUNT * n_inst]
    double* id;       // [D_COUNT * n_inst]
    float* sc;        // [M_COUNT * n_inst]
    double* part;     // [2 * n_seg]
    int* cnt;         // [4]
    const int* node_inst;
};

struct MxConst {
    double refSize, sumw;
    double MM[4][4];
    double s[4];
    double g[3];
    double rtol, atol, eta, min_res;
    int max_iter;
};

Mx mx_ptrs(pfg_ctx* c) {
    Mx m;
    m.seg = ptr<int>(c->mx_seg);
    m.ii = ptr<int>(c->mx_ii);
    m.id = ptr<double>(c->mx_id);
    m.sc = ptr<float>(c->mx_sc);
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
        k.s[i] = g.s[i];
        for (int j = 0; j < 4; ++j) k.MM[i][j] = g.MM[i][j];
    }
    for (int f = 0; f < 3; ++f) k.g[f] = c->prm.gravity[f];
    k.rtol = c->prm.krylov_rel_tol;
    k.atol = c->prm.krylov_abs_tol;
    k.eta = c->prm.inner_rel_tol > 0 ? c->prm.inner_rel_tol : 1e-4;
    k.min_res = c->prm.picard_min_res;
    k.max_iter = c->prm.picard_max_iter;
    return k;
}

// Per-instance deterministic reduction of NV values: each segment block writes its partials,
// the last block of the instance to arrive sums the partials of the instance's blocks in
// block order.  Returns true in the last block (totals valid in thread 0).
template <int NT, int NV, class T>
__device__ __forceinline__ bool inst_reduce(T (&v)[NV], int b, int b0, int b1, T* part, unsigned* ticket, double* sh) {
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = (T)block_sum<NT>((double)v[i], sh);
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
        v[i] = (T)block_sum<NT>((double)s, sh);
    }
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// ---- element kernels ----------------------------------------------------------------------

// Geometry (FP64, Element.cpp:15-135) and tau (MomContEquationPSPG.inl:237-259) per element;
// FP64 copy for the residual, FP32 copy [|e|, tau, gradN] for the FP32 assembly.
template <int DIM>
__global__ void k_mx_prep(int E, int N, const int* __restrict__ conn, const double* __restrict__ pos,
                          const double* __restrict__ q_iter, Mx m, double refSize, double* __restrict__ ed,
                          float* __restrict__ ed32) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[DIM + 1];
    load_nodes<DIM>(conn, E, e, nd);
    const int inst = m.node_inst[nd[0]];
    if (!m.ii[inst * I_COUNT + I_ACTIVE]) return;
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
    ed[e] = g.detJ;
    ed[(size_t)E + e] = tau;
    ed32[e] = (float)(g.detJ * refSize);
    ed32[(size_t)E + e] = (float)tau;
#pragma unroll
    for (int f = 0; f < DIM; ++f)
#pragma unroll
        for (int i = 0; i <= DIM; ++i) {
            ed[(size_t)(2 + f * (DIM + 1) + i) * E + e] = G[f][i];
            ed32[(size_t)(2 + f * (DIM + 1) + i) * E + e] = (float)G[f][i];
        }
}

// FP32 matrix values, one thread per node pair (same gather and pattern as the FP64 path).
// Dirichlet columns are zeroed; their right-hand-side share lives in the FP64 residual.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_mx_pairs(int P, int N, int E, const int* __restrict__ pair_node,
                                                    const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                                                    const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                                                    const uint8_t* __restrict__ ne_loc, const int* __restrict__ conn,
                                                    const float* __restrict__ ed, const uint8_t* __restrict__ flags,
                                                    const int* __restrict__ row_ptr, float* __restrict__ val, Mx m,
                                                    MxConst k) {
    constexpr int NPE = DIM + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P) return;
    const int n = pair_node[t];
    const int inst = m.node_inst[n];
    if (!m.ii[inst * I_COUNT + I_ACTIVE]) return;
    const int b0 = nbr_ptr[n];
    const int deg = nbr_ptr[n + 1] - b0;
    const int rank = t - b0;
    const int mm = nbr[t];
    const uint8_t fn = flags[n];
    if (fn & F_FREE) {
#pragma unroll
        for (int f = 0; f <= DIM; ++f) val[row_ptr[n + f * N]] = 1.0f;
        return;
    }
    const float rho = (float)m.id[inst * D_COUNT + D_RHO];
    const float mu_sum = (float)(m.id[inst * D_COUNT + D_MU] * k.sumw);
    const float l_sum = (float)(k.sumw / m.id[inst * D_COUNT + D_RHO]);
    const float inv_dt = (float)(1.0 / m.id[inst * D_COUNT + D_DT]);
    float acc[NPE][NPE];
#pragma unroll
    for (int a = 0; a < NPE; ++a)
#pragma unroll
        for (int b = 0; b < NPE; ++b) acc[a][b] = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        int j = -1;
#pragma unroll
        for (int jj = 0; jj < NPE; ++jj)
            if (__ldg(conn + (size_t)jj * E + e) == mm) j = jj;
        if (j < 0) continue;
        const int i = ne_loc[q];
        const float ae = ed[e];
        const float tau = ed[(size_t)E + e];
        float gi[DIM], gj[DIM];
#pragma unroll
        for (int f = 0; f < DIM; ++f) {
            gi[f] = ed[(size_t)(2 + f * NPE + i) * E + e];
            gj[f] = ed[(size_t)(2 + f * NPE + j) * E + e];
        }
        float dot = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f) dot += gi[f] * gj[f];
        const float mij = inv_dt * (rho * (float)k.MM[i][j] * ae);
        const float kf = ae * mu_sum;
        const float si = (float)k.s[i], sj = (float)k.s[j];
#pragma unroll
        for (int f1 = 0; f1 < DIM; ++f1) {
#pragma unroll
            for (int f2 = 0; f2 < DIM; ++f2) {
                const float kv = kf * ((f1 == f2 ? dot : 0.0f) + gi[f2] * gj[f1]);
                acc[f1][f2] += (f1 == f2 ? mij : 0.0f) + kv;
            }
            acc[f1][DIM] += -(ae * sj * gi[f1]);
        }
        const float ctau = tau * inv_dt;
#pragma unroll
        for (int f2 = 0; f2 < DIM; ++f2) acc[DIM][f2] += ctau * (ae * gi[f2] * sj) + ae * si * gj[f2];
        acc[DIM][DIM] += tau * (ae * l_sum * dot);
    }
    const bool bound = fn & F_BOUND;
    const bool mdir = (flags[mm] & F_BOUND) && (flags[mm] & F_DIRICHLET);
#pragma unroll
    for (int f1 = 0; f1 <= DIM; ++f1) {
        const int r = n + f1 * N;
        const int rp = row_ptr[r];
        if (f1 < DIM && bound) {
            if (mm == n) val[rp] = 1.0f;
            continue;
        }
#pragma unroll
        for (int f2 = 0; f2 <= DIM; ++f2) {
            float a = acc[f1][f2];
            if (mdir && f2 < DIM && !(mm == n && f1 == f2)) a = 0.0f;
            val[rp + f2 * deg + rank] = a;
        }
    }
}

// ---- node-block Jacobi preconditioner (FP32) ----------------------------------------------

template <int DIM>
__global__ void k_mx_binv(int N, const int* __restrict__ rp, const float* __restrict__ val,
                          const int* __restrict__ diag, float* __restrict__ binv, Mx m) {
    constexpr int B = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    if (!m.ii[m.node_inst[n] * I_COUNT + I_ACTIVE]) return;
    float a[B][2 * B];
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        const int r = n + f1 * N;
        const int dp = diag[r];
        const int b0 = rp[r], len = rp[r + 1] - b0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            a[f1][f2] = 0;
            a[f1][B + f2] = (f1 == f2) ? 1.0f : 0.0f;
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
    float dg[B];
#pragma unroll
    for (int f = 0; f < B; ++f) dg[f] = a[f][f];
    bool ok = true;
#pragma unroll
    for (int kk = 0; kk < B; ++kk) {
        int piv = kk;
        float best = fabsf(a[kk][kk]);
#pragma unroll
        for (int i = kk + 1; i < B; ++i)
            if (fabsf(a[i][kk]) > best) {
                best = fabsf(a[i][kk]);
                piv = i;
            }
        if (best == 0.0f) ok = false;
        if (piv != kk) {
#pragma unroll
            for (int j = 0; j < 2 * B; ++j) {
                const float t = a[kk][j];
                a[kk][j] = a[piv][j];
                a[piv][j] = t;
            }
        }
        const float inv = ok ? 1.0f / a[kk][kk] : 0.0f;
#pragma unroll
        for (int j = 0; j < 2 * B; ++j) a[kk][j] *= inv;
#pragma unroll
        for (int i = 0; i < B; ++i) {
            if (i == kk) continue;
            const float f = a[i][kk];
#pragma unroll
            for (int j = 0; j < 2 * B; ++j) a[i][j] -= f * a[kk][j];
        }
    }
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1)
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) {
            float v = a[f1][B + f2];
            if (!ok) v = (f1 == f2) ? (dg[f1] != 0.0f ? 1.0f / dg[f1] : 1.0f) : 0.0f;
            binv[(size_t)(f1 * B + f2) * N + n] = v;
        }
}

template <int DIM>
__device__ __forceinline__ void block_apply32(int n, int N, const float* __restrict__ binv, const float (&y)[DIM + 1],
                                              float* __restrict__ z) {
    constexpr int B = DIM + 1;
#pragma unroll
    for (int f1 = 0; f1 < B; ++f1) {
        float s = 0;
#pragma unroll
        for (int f2 = 0; f2 < B; ++f2) s += binv[(size_t)(f1 * B + f2) * N + n] * y[f2];
        z[(size_t)f1 * N + n] = s;
    }
}

// ---- FP64 matrix-free residual ----------------------------------------------------------------

// r = b - A x for the nodes of one segment, A and b being the PSPG system of
// m_buildAbPSPG + m_applyBCPSPG (MomContEquationPSPG.inl:6-235) at the element data `ed`
// (geometry and tau of the current Picard iterate).  Dirichlet velocity entries of x are
// replaced by their prescribed values, which reproduces the column elimination of
// :216-229 exactly; identity rows (free nodes, bound-node velocities) give r = b - x.
// Also seeds the FP32 correction solve: r32 = rhat = r, p = v = 0.  With `check`, the
// residual is the Picard residual: the instance's iteration count, convergence and failure
// are decided here (PicardAlgo.cpp:48-90).
template <int DIM>
__global__ void __launch_bounds__(NB) k_mx_resid(Mx m, int N, int E, const int* __restrict__ ne_ptr,
                                                 const int* __restrict__ ne_elem, const uint8_t* __restrict__ ne_loc,
                                                 const int* __restrict__ conn, const double* __restrict__ ed,
                                                 const uint8_t* __restrict__ flags, const double* __restrict__ x,
                                                 const double* __restrict__ qprev, const double* __restrict__ vbc,
                                                 MxConst k, float* __restrict__ W, size_t ld, int check) {
    constexpr int NPE = DIM + 1;
    __shared__ double sh[32];
    const int b = blockIdx.x;
    const int inst = m.seg[3 * b];
    int* ii = m.ii + inst * I_COUNT;
    if (!ii[I_ACTIVE]) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    const bool valid = n < m.seg[3 * b + 2];
    double* idd = m.id + inst * D_COUNT;
    const double rho = idd[D_RHO], mu = idd[D_MU], dt = idd[D_DT];
    const double inv_dt = 1 / dt;
    double rr = 0, bb = 0;
    if (valid) {
        const uint8_t fl = flags[n];
        const bool bound = fl & F_BOUND, isfree = fl & F_FREE;
        const bool dir = bound && (fl & F_DIRICHLET);
        double bv[DIM], av[DIM], bp = 0, ap = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f) bv[f] = av[f] = 0;
        const double kfs = mu * k.sumw, lfs = k.sumw / rho;
        for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
            const int e = ne_elem[q];
            const int i = ne_loc[q];
            int nd[NPE];
            load_nodes<DIM>(conn, E, e, nd);
            const double ae = ed[e] * k.refSize;
            const double tau = ed[(size_t)E + e];
            double G[DIM][NPE], X[DIM][NPE], VP[DIM][NPE], Pj[NPE];
#pragma unroll
            for (int j = 0; j < NPE; ++j) {
                const int nj = nd[j];
                const uint8_t fj = flags[nj];
                const bool dj = (fj & F_BOUND) && (fj & F_DIRICHLET);
#pragma unroll
                for (int f = 0; f < DIM; ++f) {
                    G[f][j] = ed[(size_t)(2 + f * NPE + j) * E + e];
                    X[f][j] = dj ? vbc[(size_t)f * N + nj] : x[(size_t)f * N + nj];
                    VP[f][j] = qprev[(size_t)f * N + nj];
                }
                Pj[j] = x[(size_t)DIM * N + nj];
            }
            double dot[NPE];
#pragma unroll
            for (int j = 0; j < NPE; ++j) {
                double t = 0;
#pragma unroll
                for (int f = 0; f < DIM; ++f) t += G[f][i] * G[f][j];
                dot[j] = t;
            }
            double sP = 0, lP = 0;
#pragma unroll
            for (int j = 0; j < NPE; ++j) {
                sP += k.s[j] * Pj[j];
                lP += dot[j] * Pj[j];
            }
            // momentum rows (assembled only for nodes that are not bound, :68)
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                double mvp = 0;
#pragma unroll
                for (int j = 0; j < NPE; ++j) mvp += (rho * k.MM[i][j] * ae * inv_dt) * VP[f][j];
                bv[f] += ae * (rho * k.s[i] * k.g[f]) + mvp;
            }
            if (!bound) {
                double Lg[DIM][DIM];  // Lg[a][c] = sum_j dN_j/dx_c X_a,j
#pragma unroll
                for (int a = 0; a < DIM; ++a)
#pragma unroll
                    for (int c2 = 0; c2 < DIM; ++c2) {
                        double t = 0;
#pragma unroll
                        for (int j = 0; j < NPE; ++j) t += G[c2][j] * X[a][j];
                        Lg[a][c2] = t;
                    }
                const double kf = ae * kfs;
#pragma unroll
                for (int f = 0; f < DIM; ++f) {
                    double mx = 0, kx = 0;
#pragma unroll
                    for (int j = 0; j < NPE; ++j) {
                        mx += (rho * k.MM[i][j] * ae * inv_dt) * X[f][j];
                        kx += dot[j] * X[f][j];
                    }
#pragma unroll
                    for (int f2 = 0; f2 < DIM; ++f2) kx += G[f2][i] * Lg[f2][f];
                    av[f] += mx + kf * kx - ae * G[f][i] * sP;
                }
            }
            // continuity row
            double gdot = 0, cvp = 0, cx = 0, dv = 0;
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                gdot += G[f][i] * k.g[f];
                double sv = 0, sx = 0;
#pragma unroll
                for (int j = 0; j < NPE; ++j) {
                    sv += k.s[j] * VP[f][j];
                    sx += k.s[j] * X[f][j];
                    dv += G[f][j] * X[f][j];
                }
                cvp += G[f][i] * sv;
                cx += G[f][i] * sx;
            }
            const double ctau = tau * inv_dt;
            bp += tau * (ae * k.sumw * gdot) + ctau * ae * cvp;
            ap += ctau * ae * cx + ae * k.s[i] * dv + tau * ae * lfs * lP;
        }
        double r[DIM + 1], bn[DIM + 1];
        if (isfree) {  // identity rows; b from :190-204 and :211-214
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                bn[f] = bound ? bv[f] : qprev[(size_t)f * N + n] + dt * k.g[f];
                if (dir) bn[f] = vbc[(size_t)f * N + n];
                r[f] = bn[f] - x[(size_t)f * N + n];
            }
            bn[DIM] = 0;
            r[DIM] = -x[(size_t)DIM * N + n];
        } else {
#pragma unroll
            for (int f = 0; f < DIM; ++f) {
                if (bound) {
                    bn[f] = dir ? vbc[(size_t)f * N + n] : bv[f];
                    r[f] = bn[f] - x[(size_t)f * N + n];
                } else {
                    bn[f] = bv[f];
                    r[f] = bv[f] - av[f];
                }
            }
            bn[DIM] = bp;
            r[DIM] = bp - ap;
        }
#pragma unroll
        for (int f = 0; f <= DIM; ++f) {
            const size_t row = (size_t)f * N + n;
            const float r32 = (float)r[f];
            W[W_R * ld + row] = r32;
            W[W_RHAT * ld + row] = r32;
            W[W_P * ld + row] = 0.0f;
            W[W_V * ld + row] = 0.0f;
            rr += r[f] * r[f];
            bb += bn[f] * bn[f];
        }
    }
    double v[2] = {rr, bb};
    if (!inst_reduce<NB, 2, double>(v, b, ii[I_B0], ii[I_B1], m.part, reinterpret_cast<unsigned*>(ii + I_TICKET), sh))
        return;
    if (threadIdx.x != 0) return;
    rr = v[0];
    bb = v[1];
    idd[D_RR] = rr;
    idd[D_BB] = bb;
    bool active = true;
    if (check) {
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
    const bool need = active && rr > tol * tol;
    float* sc = m.sc + inst * M_COUNT;
    sc[M_RHO] = (float)rr;
    sc[M_RHO_OLD] = 1.0f;
    sc[M_ALPHA] = 1.0f;
    sc[M_OMEGA] = 1.0f;
    sc[M_RR] = (float)rr;
    sc[M_TOL2] = (float)(k.eta * k.eta * rr);
    sc[M_ITERS] = 0.0f;
    sc[M_DONE] = need ? 0.0f : 1.0f;
    if (need) atomicAdd(m.cnt + C_NEED, 1);
    if (active) atomicAdd(m.cnt + C_ACTIVE, 1);
}

// ---- FP32 BiCGSTAB on segments --------------------------------------------------------------

// Row r of A32 times y over G lanes (valid on lane 0 of the group).
template <int G>
__device__ __forceinline__ float row_dot32(int r, bool act, const int* __restrict__ rp, const int* __restrict__ col,
                                           const float* __restrict__ val, const float* __restrict__ y, int lane) {
    const int b = act ? rp[r] : 0, e = act ? rp[r + 1] : 0;
    float s = 0;
    for (int kk = b + lane; kk < e; kk += G) s += val[kk] * __ldg(y + col[kk]);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    return s;
}

// p = r + beta (p - omega v); phat = Binv p
template <int DIM>
__global__ void __launch_bounds__(NB) k_mx_up_p(Mx m, int N, float* __restrict__ W, size_t ld,
                                                const float* __restrict__ binv) {
    const int b = blockIdx.x;
    const float* sc = m.sc + m.seg[3 * b] * M_COUNT;
    if (sc[M_DONE] != 0.0f) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    if (n >= m.seg[3 * b + 2]) return;
    const float beta = (sc[M_RHO] / sc[M_RHO_OLD]) * (sc[M_ALPHA] / sc[M_OMEGA]);
    const float om = sc[M_OMEGA];
    float p[DIM + 1];
#pragma unroll
    for (int f = 0; f <= DIM; ++f) {
        const size_t r = (size_t)f * N + n;
        p[f] = W[W_R * ld + r] + beta * (W[W_P * ld + r] - om * W[W_V * ld + r]);
        W[W_P * ld + r] = p[f];
    }
    block_apply32<DIM>(n, N, binv, p, W + W_PHAT * ld);
}

// s = r - alpha v; shat = Binv s
template <int DIM>
__global__ void __launch_bounds__(NB) k_mx_up_s(Mx m, int N, float* __restrict__ W, size_t ld,
                                                const float* __restrict__ binv) {
    const int b = blockIdx.x;
    const float* sc = m.sc + m.seg[3 * b] * M_COUNT;
    if (sc[M_DONE] != 0.0f) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    if (n >= m.seg[3 * b + 2]) return;
    const float al = sc[M_ALPHA];
    float s[DIM + 1];
#pragma unroll
    for (int f = 0; f <= DIM; ++f) {
        const size_t r = (size_t)f * N + n;
        s[f] = W[W_R * ld + r] - al * W[W_V * ld + r];
        W[W_S * ld + r] = s[f];
    }
    block_apply32<DIM>(n, N, binv, s, W + W_SHAT * ld);
}

// out = A32 in over the rows of the segment's nodes (all fields); dots for alpha or omega.
// mode 0: v = A phat, alpha = rho / (rhat . v).  mode 1: t = A shat, omega = (t.s)/(t.t).
template <int G, int DIM, int MODE>
__global__ void __launch_bounds__(SPMV_BLOCK) k_mx_spmv(Mx m, int N, const int* __restrict__ rp,
                                                        const int* __restrict__ col, const float* __restrict__ val,
                                                        float* __restrict__ W, size_t ld) {
    __shared__ double sh[32];
    const int b = blockIdx.x;
    const int inst = m.seg[3 * b];
    float* sc = m.sc + inst * M_COUNT;
    if (sc[M_DONE] != 0.0f) return;
    const int n0 = m.seg[3 * b + 1], cnt = m.seg[3 * b + 2] - n0;
    const int rows = cnt * (DIM + 1);
    const int lane = threadIdx.x % G;
    const float* in = W + (MODE == 0 ? W_PHAT : W_SHAT) * ld;
    float* out = W + (MODE == 0 ? W_V : W_T) * ld;
    float d0 = 0, d1 = 0;
    for (int t0 = 0; t0 < rows; t0 += SPMV_BLOCK / G) {
        const int t = t0 + threadIdx.x / G;
        const bool act = t < rows;
        int r = 0;
        if (act) {
            const int f = t / cnt;
            r = f * N + n0 + (t - f * cnt);
        }
        const float y = row_dot32<G>(r, act, rp, col, val, in, lane);
        if (act && lane == 0) {
            out[r] = y;
            if (MODE == 0) {
                d0 += W[W_RHAT * ld + r] * y;
            } else {
                d0 += y * W[W_S * ld + r];
                d1 += y * y;
            }
        }
    }
    const int* ii = m.ii + inst * I_COUNT;
    float v[2] = {d0, d1};
    if (!inst_reduce<SPMV_BLOCK, 2, float>(v, b, ii[I_B0], ii[I_B1], reinterpret_cast<float*>(m.part),
                                           reinterpret_cast<unsigned*>(m.ii + inst * I_COUNT + I_TICKET), sh))
        return;
    if (threadIdx.x != 0) return;
    if (MODE == 0) {
        if (v[0] == 0.0f || !isfinite(v[0])) {
            sc[M_DONE] = 2.0f;
            atomicSub(m.cnt + C_NEED, 1);
        } else {
            sc[M_ALPHA] = sc[M_RHO] / v[0];
        }
    } else {
        sc[M_OMEGA] = (v[1] == 0.0f || !isfinite(v[1])) ? 0.0f : v[0] / v[1];
    }
}

// x += alpha phat + omega shat (FP64 solution); r = s - omega t; rho = rhat.r; rr = r.r
template <int DIM>
__global__ void __launch_bounds__(NB) k_mx_up_x(Mx m, int N, double* __restrict__ x, float* __restrict__ W,
                                                size_t ld) {
    __shared__ double sh[32];
    const int b = blockIdx.x;
    const int inst = m.seg[3 * b];
    float* sc = m.sc + inst * M_COUNT;
    if (sc[M_DONE] != 0.0f) return;
    const int n = m.seg[3 * b + 1] + threadIdx.x;
    const float al = sc[M_ALPHA], om = sc[M_OMEGA];
    float rh = 0, rr = 0;
    if (n < m.seg[3 * b + 2]) {
#pragma unroll
        for (int f = 0; f <= DIM; ++f) {
            const size_t r = (size_t)f * N + n;
            x[r] += (double)(al * W[W_PHAT * ld + r]) + (double)(om * W[W_SHAT * ld + r]);
            const float rv = W[W_S * ld + r] - om * W[W_T * ld + r];
            W[W_R * ld + r] = rv;
            rh += W[W_RHAT * ld + r] * rv;
            rr += rv * rv;
        }
    }
    int* ii = m.ii + inst * I_COUNT;
    float v[2] = {rh, rr};
    if (!inst_reduce<NB, 2, float>(v, b, ii[I_B0], ii[I_B1], reinterpret_cast<float*>(m.part),
                                   reinterpret_cast<unsigned*>(ii + I_TICKET), sh))
        return;
    if (threadIdx.x != 0) return;
    sc[M_RHO_OLD] = sc[M_RHO];
    sc[M_RHO] = v[0];
    sc[M_RR] = v[1];
    sc[M_ITERS] += 1.0f;
    ii[I_KIT] += 1;
    float done = 0.0f;
    if (!isfinite(v[1]))
        done = 2.0f;
    else if (v[1] <= sc[M_TOL2])
        done = 1.0f;
    else if (v[0] == 0.0f || om == 0.0f)
        done = 2.0f;
    if (done != 0.0f) {
        sc[M_DONE] = done;
        atomicSub(m.cnt + C_NEED, 1);
    }
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

// Lanes per SpMV row from the dimension alone (mean row length ~21 in 2D, ~60 in 3D), so an
// instance's arithmetic does not depend on the other instances it is batched with.
int lanes(pfg_ctx* c) { return c->dim == 2 ? 8 : 16; }

int read_counters(pfg_ctx* c, int* need, int* active) {
    PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, c->mx_cnt.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    const int* h = reinterpret_cast<const int*>(c->h_scalars);
    *need = h[C_NEED];
    *active = h[C_ACTIVE];
    return PFG_OK;
}

template <int DIM>
int mx_assemble(pfg_ctx* c, const double* q_iter, const MxConst& k) {
    const int N = c->N, E = c->E;
    Mx m = mx_ptrs(c);
    if (E > 0) {
        prof_begin(c, PH_PSPG_ELEM);
        k_mx_prep<DIM><<<div_up(E, BLOCK), BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), q_iter,
                                                                  m, k.refSize, ptr<double>(c->edata),
                                                                  ptr<float>(c->edata32));
        prof_end(c, PH_PSPG_ELEM);
        PFG_CHECK_LAUNCH(c);
    }
    prof_begin(c, PH_PSPG_PAIRS);
    k_mx_pairs<DIM><<<div_up(c->P, BLOCK), BLOCK, 0, c->stream>>>(
        c->P, N, E, ptr<int>(c->pair_node), ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<int>(c->ne_ptr),
        ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn), ptr<float>(c->edata32),
        ptr<uint8_t>(c->flags), ptr<int>(c->row_ptr), ptr<float>(c->val32), m, k);
    k_mx_binv<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, ptr<int>(c->row_ptr), ptr<float>(c->val32),
                                                              ptr<int>(c->diag_pos), ptr<float>(c->binv32), m);
    prof_end(c, PH_PSPG_PAIRS);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

template <int DIM>
int mx_residual(pfg_ctx* c, const MxConst& k, int check, int* need, int* active) {
    Mx m = mx_ptrs(c);
    PFG_CUDA(c, cudaMemsetAsync(c->mx_cnt.p, 0, 4 * sizeof(int), c->stream));
    prof_begin(c, PH_RESIDUAL);
    k_mx_resid<DIM><<<c->n_seg, NB, 0, c->stream>>>(
        m, c->N, c->E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn),
        ptr<double>(c->edata), ptr<uint8_t>(c->flags), ptr<double>(c->q), ptr<double>(c->q_prev),
        ptr<double>(c->vbc), k, ptr<float>(c->kv32), (size_t)c->R, check);
    prof_end(c, PH_RESIDUAL);
    PFG_CHECK_LAUNCH(c);
    return read_counters(c, need, active);
}

// Correction solves of every instance that needs one, until all are done or the iteration
// cap is reached.  x (the FP64 iterate) is updated in place.
template <int G, int DIM>
int mx_inner(pfg_ctx* c, int* need) {
    Mx m = mx_ptrs(c);
    const int N = c->N;
    const size_t ld = (size_t)c->R;
    float* W = ptr<float>(c->kv32);
    const float* binv = ptr<float>(c->binv32);
    const int* rp = ptr<int>(c->row_ptr);
    const int* col = ptr<int>(c->col);
    const float* val = ptr<float>(c->val32);
    double* x = ptr<double>(c->q);
    const int max_it = std::max(1, c->prm.krylov_max_iter);
    const int chunk = 8;
    int done_it = 0;
    int active = 0;
    while (*need > 0 && done_it < max_it) {
        const int n = std::min(chunk, max_it - done_it);
        for (int it = 0; it < n; ++it) {
            prof_begin(c, PH_KRYLOV_ITER);
            k_mx_up_p<DIM><<<c->n_seg, NB, 0, c->stream>>>(m, N, W, ld, binv);
            k_mx_spmv<G, DIM, 0><<<c->n_seg, SPMV_BLOCK, 0, c->stream>>>(m, N, rp, col, val, W, ld);
            k_mx_up_s<DIM><<<c->n_seg, NB, 0, c->stream>>>(m, N, W, ld, binv);
            k_mx_spmv<G, DIM, 1><<<c->n_seg, SPMV_BLOCK, 0, c->stream>>>(m, N, rp, col, val, W, ld);
            k_mx_up_x<DIM><<<c->n_seg, NB, 0, c->stream>>>(m, N, x, W, ld);
            prof_end(c, PH_KRYLOV_ITER);
        }
        PFG_CHECK_LAUNCH(c);
        done_it += n;
        int rc = read_counters(c, need, &active);
        if (rc) return rc;
    }
    return PFG_OK;
}

template <int DIM>
int mx_inner_dim(pfg_ctx* c, int* need) {
    switch (lanes(c)) {
        case 8: return mx_inner<8, DIM>(c, need);
        default: return mx_inner<16, DIM>(c, need);
    }
}

template <int DIM>
int mx_picard(pfg_ctx* c, const double* dts, pfg_step_status* st) {
    const int K = c->n_inst;
    const size_t R = c->R;
    int rc;
    // per-instance tables: counters reset, dt of this step, all instances active
    std::vector<int>& hi = c->h_mx_ii;
    std::vector<double>& hd = c->h_mx_id;
    for (int i = 0; i < K; ++i) {
        int* r = hi.data() + (size_t)i * I_COUNT;
        r[I_ACTIVE] = 1;
        r[I_STATUS] = 0;
        r[I_IT] = 0;
        r[I_KIT] = 0;
        r[I_TICKET] = 0;
        hd[(size_t)i * D_COUNT + D_DT] = dts[i];
    }
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_ii.p, hi.data(), sizeof(int) * hi.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_id.p, hd.data(), sizeof(double) * hd.size(), cudaMemcpyHostToDevice, c->stream));
    // prepare: save the node list, qPrev = states, build A32 at the current geometry
    PFG_CUDA(c, cudaMemcpyAsync(c->pos_save.p, c->pos.p, sizeof(double) * c->dim * c->N, cudaMemcpyDeviceToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->q_prev.p, c->q.p, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
    const MxConst k = mx_const(c);
    if ((rc = mx_assemble<DIM>(c, ptr<double>(c->q_prev), k))) return rc;
    int need = 0, active = 0;
    if ((rc = mx_residual<DIM>(c, k, 0, &need, &active))) return rc;
    const int max_ref = c->prm.refine_max_iter > 0 ? c->prm.refine_max_iter : 30;
    while (true) {
        // linear solve of every active instance: refinement sweeps
        for (int sweep = 0; sweep < max_ref && need > 0; ++sweep) {
            if ((rc = mx_inner_dim<DIM>(c, &need))) return rc;
            if ((rc = mx_residual<DIM>(c, k, 0, &need, &active))) return rc;
        }
        // Picard update: positions, re-assembly, residual check
        k_mx_positions<DIM><<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(
            c->N, ptr<uint8_t>(c->flags), ptr<double>(c->pos_save), ptr<double>(c->q), mx_ptrs(c), ptr<double>(c->pos));
        PFG_CHECK_LAUNCH(c);
        if ((rc = mx_assemble<DIM>(c, ptr<double>(c->q), k))) return rc;
        if ((rc = mx_residual<DIM>(c, k, 1, &need, &active))) return rc;
        if (active == 0) break;
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
    }
    return PFG_OK;
}

}  // namespace

int mx_alloc(pfg_ctx* c) {
    const size_t R = std::max(c->R, 1), N = std::max(c->N, 1), E = std::max(c->E, 1);
    const int ned = 2 + c->dim * (c->dim + 1);
    int rc;
    if ((rc = ensure(c, c->val32, sizeof(float) * (size_t)std::max<int64_t>(c->nnz, 1))) ||
        (rc = ensure(c, c->edata32, sizeof(float) * ned * E)) ||
        (rc = ensure(c, c->kv32, sizeof(float) * W_COUNT * R)) ||
        (rc = ensure(c, c->binv32, sizeof(float) * (size_t)(c->dim + 1) * (c->dim + 1) * N)) ||
        (rc = ensure(c, c->mx_cnt, 64)) || (rc = ensure(c, c->node_inst, sizeof(int) * N)))
        return rc;
    // one instance covering the whole mesh until pfg_set_instances says otherwise
    const int off[2] = {0, c->N};
    const double rho = c->prm.rho, mu = c->prm.mu;
    return mx_set_instances(c, 1, off, &rho, &mu);
}

int mx_set_instances(pfg_ctx* c, int n_inst, const int* node_off, const double* rho, const double* mu) {
    const int N = c->N;
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
        (rc = ensure(c, c->mx_sc, sizeof(float) * (size_t)n_inst * M_COUNT)) ||
        (rc = ensure(c, c->mx_part, sizeof(double) * 2 * (size_t)c->n_seg)))
        return rc;
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_seg.p, seg.data(), sizeof(int) * seg.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->node_inst.p, node_inst.data(), sizeof(int) * (size_t)N, cudaMemcpyHostToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_ii.p, c->h_mx_ii.data(), sizeof(int) * c->h_mx_ii.size(), cudaMemcpyHostToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->mx_id.p, c->h_mx_id.data(), sizeof(double) * c->h_mx_id.size(),
                                cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(c->mx_sc.p, 0, sizeof(float) * (size_t)n_inst * M_COUNT, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int mx_picard_step(pfg_ctx* c, const double* dts, pfg_step_status* st) {
    return c->dim == 2 ? mx_picard<2>(c, dts, st) : mx_picard<3>(c, dts, st);
}

}  // namespace pfg
