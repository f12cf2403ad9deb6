// Weakly compressible explicit step (CDS_dpdt, CDS_rho or CDS_drhodt with the Tait-Murnaghan
// equation of state).
//
// Reference: SolverWCompNewton::m_solveWCompNewtonNoT (WCompNewton/Solver.cpp:236-276),
// ContEqWCompNewton::m_buildSystemdpdt/m_applyBCdpdt/solve (ContEquation.inl:123-169,
// :334-413), m_buildF0/m_buildSystem/m_applyBC (:171-302) for the density forms,
// MomEqWCompNewton::m_buildSystem/m_applyBC/solve (MomEquation.inl:201-374) and
// SolverWCompNewton::computeNextDT (Solver.cpp:192-234).
//
// One step is six kernels, captured once into a CUDA graph:
//   predict   (node)    v1/2 = v + dt/2 a ; x += dt v1/2 for non-fixed nodes
//   cont_elem (element) per element node: lumped mass and the continuity right-hand side
//   cont_node (node)    gather over the node's elements in element order -> p, rho (Tait)
//   mom_elem  (element) per element node: lumped rho-mass and FTot = -K v + D^T p + F(rho g)
//   mom_node  (node)    gather -> a = F / M (with BCs), v = v1/2 + dt/2 a
//   dt        (element) min over elements of sc^2 h^2 / max(u^2, c^2, 4 alpha^2/h^2) -> next dt
// The density forms solve the continuity equation for rho and take p from it: CDS_drhodt with the
// D factor rho_g and the mass times rho; CDS_rho with F0 = M rho built by one more element kernel
// (rho_pre) before the prediction moves the nodes (ContEqWCompNewton::preCompute) and only the
// lumped mass after it.  Their boundary condition: free and free-surface nodes take rho*.
//
// Precision.  Node state (x, v, p, rho, a) is FP64 in both forms; geometry (J, detJ, the
// area-weighted shape gradients A_fi = |e| dN_i/dx_f) is FP64; the element arithmetic type R
// is double (plain form) or float (mixed form).  The two terms that nearly cancel node by node
// are written as differences from the node's own value so that FP32 arithmetic keeps them
// accurate; both rewrites are exact algebra:
//   continuity (Meduri):  sum_e sum_j M_ij p_j = p_i ML_i + sum_e sum_j M_ij (p_j - p_i)
//   momentum pressure:    sum_e A_fi pbar_e   = p_i S sum_e A_fi + sum_e A_fi sum_j s_j (p_j - p_i)
// (S = sum_j s_j = sum_g w_g).  The p_i-weighted parts are formed in FP64 at the node.
// Element partials are summed at the node in ascending element order (the order of the
// reference's serial scatters), so results do not depend on scheduling.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "pfg_device.cuh"
#include "pfg_fst.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

struct WcConst {
    double K0, K0p, rho_star, mu, sc, max_dt;
    double g[3];
    int meduri;
    int ver;           // pfg_wc_version: 0 CDS_dpdt, 1 CDS_rho, 2 CDS_drhodt
    double MM[4][4];   // sum_g w N_i N_j
    double s[4];       // sum_g w N_i
    double S;          // sum_i s_i
    double refSize;
    double mu_sum;     // sum_g mu w_g (getK factor)
    // problem "BoussinesqWC" (MomEquation.inl:36-51, 105-130): body-force factor
    // rho_g (1 - alpha (T_g - Tr)) and, with phase change, the Carman-Kozeny factor
    // C (1 - fl_g)^2 / (fl_g^3 + eps) at the element Gauss points; CFL diffusion
    // max(mu, k / cv) / rho (Solver.cpp:215-219)
    int bq, ck, ng;
    double alpha, t_ref, k_cv, ck_c, ck_eps, tm, dtm;
    double gN[4][4], gw[4];
};

// Liquid fraction of MomEqWCompNewton::m_getFl (MomEquation.inl:377-381): the cubic smoothstep
// over the melting range (Tm - DT/2, Tm + DT/2), 1 above it.
__device__ __forceinline__ double fl_wc(const WcConst& k, double T) {
    const double d3 = k.dtm * k.dtm * k.dtm;
    return static_cast<double>(T > k.tm - k.dtm / 2) * static_cast<double>(T < k.tm + k.dtm / 2) *
               (-2 / d3 * T * T * T + 6 * k.tm / d3 * T * T + (3 / (2 * k.dtm) - 6 * k.tm * k.tm / d3) * T +
                (0.5 - 1.5 * k.tm / k.dtm + 2 * k.tm * k.tm * k.tm / d3)) +
           static_cast<double>(T > k.tm + k.dtm / 2);
}

WcConst make_const(pfg_ctx* c) {
    const GaussConst gc = gauss_const(c->dim);
    WcConst k{};
    k.K0 = c->prm.K0;
    k.K0p = c->prm.K0p;
    k.rho_star = c->prm.rho_star;
    k.mu = c->prm.mu;
    k.sc = c->prm.security_coeff;
    k.max_dt = c->prm.max_dt;
    for (int f = 0; f < 3; ++f) k.g[f] = c->prm.gravity[f];
    k.meduri = c->prm.meduri;
    k.ver = c->prm.wc_version;
    k.S = 0;
    for (int i = 0; i < 4; ++i) {
        k.s[i] = gc.s[i];
        if (i <= c->dim) k.S += gc.s[i];
        for (int j = 0; j < 4; ++j) k.MM[i][j] = gc.MM[i][j];
    }
    k.refSize = gc.refSize;
    k.mu_sum = 0;
    for (int q = 0; q < gc.n; ++q) k.mu_sum += c->prm.mu * gc.w[q];
    k.bq = c->prm.boussinesq != 0;
    k.ck = k.bq && c->prm.heat_phase_change != 0;
    k.ng = gc.n;
    for (int q = 0; q < 4; ++q) {
        k.gw[q] = gc.w[q];
        for (int i = 0; i < 4; ++i) k.gN[q][i] = gc.N[q][i];
    }
    k.alpha = c->prm.alpha_t;
    k.t_ref = c->prm.t_ref;
    k.k_cv = k.bq ? c->prm.heat_k / c->prm.heat_cv : 0.0;
    k.ck_c = c->prm.ck_c;
    k.ck_eps = c->prm.ck_eps;
    k.tm = c->prm.heat_tm;
    k.dtm = c->prm.heat_dt_melt;
    return k;
}

// slots of ctx->wc_dt (doubles)
enum : int { T_DT = 0, T_TIME = 1, T_MIN = 2, T_TICKET = 3 };

// Element partial layout (array of structures, one record per element):
//   R  part: [ML_0..ML_d, cont_0..cont_d, MLrho_0..MLrho_d, Fs_{f,i}...]   (dim+3)(dim+1) values
//   FP64 part: [W_{f,i}] = A_{f,i}                                         dim(dim+1) values
template <int DIM>
struct ElLayout {
    static constexpr int NPE = DIM + 1;
    static constexpr int ML = 0, CONT = NPE, MLR = 2 * NPE, FS = 3 * NPE;
    static constexpr int NR = 3 * NPE + DIM * NPE;
    static constexpr int ND = DIM * NPE;
};

// Area-weighted shape gradients A[f][i] = |e| dN_i/dx_f from the FP64 Jacobian: no division.
// 2D: |e| = detJ/2 and invJ = adj(J)/detJ; 3D: |e| = detJ/6 with the cofactors of J.
template <int DIM>
__device__ __forceinline__ void area_gradients(const Geom<DIM>& g, double refSize, double (&A)[DIM][DIM + 1]) {
    if constexpr (DIM == 2) {
        const auto& J = g.J;
        // invJ * detJ = [[J11, -J01], [-J10, J00]]; dN_{k+1}/dx_f = invJ[k][f]
        const double adj[2][2] = {{J[1][1], -J[0][1]}, {-J[1][0], J[0][0]}};
#pragma unroll
        for (int f = 0; f < 2; ++f) {
            A[f][1] = refSize * adj[0][f];
            A[f][2] = refSize * adj[1][f];
            A[f][0] = -(A[f][1] + A[f][2]);
        }
    } else {
        const auto& J = g.J;
        double adj[3][3];
        adj[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        adj[0][1] = J[2][1] * J[0][2] - J[2][2] * J[0][1];
        adj[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
        adj[1][0] = J[2][0] * J[1][2] - J[1][0] * J[2][2];
        adj[1][1] = J[0][0] * J[2][2] - J[2][0] * J[0][2];
        adj[1][2] = J[1][0] * J[0][2] - J[0][0] * J[1][2];
        adj[2][0] = J[1][0] * J[2][1] - J[2][0] * J[1][1];
        adj[2][1] = J[2][0] * J[0][1] - J[0][0] * J[2][1];
        adj[2][2] = J[0][0] * J[1][1] - J[1][0] * J[0][1];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            A[f][1] = refSize * adj[0][f];
            A[f][2] = refSize * adj[1][f];
            A[f][3] = refSize * adj[2][f];
            A[f][0] = -(A[f][1] + A[f][2] + A[f][3]);
        }
    }
}

template <int DIM>
__device__ __forceinline__ void jacobian(const double* __restrict__ pos, int N, const int (&nd)[DIM + 1], Geom<DIM>& g) {
#pragma unroll
    for (int r = 0; r < DIM; ++r) {
        const double o = pos[(size_t)r * N + nd[0]];
#pragma unroll
        for (int cc = 0; cc < DIM; ++cc) g.J[r][cc] = pos[(size_t)r * N + nd[cc + 1]] - o;
    }
    if constexpr (DIM == 2) {
        g.detJ = g.J[0][0] * g.J[1][1] - g.J[1][0] * g.J[0][1];
    } else {
        const auto& J = g.J;
        g.detJ = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1]
               - J[2][0] * J[1][1] * J[0][2] - J[2][1] * J[1][2] * J[0][0] - J[2][2] * J[1][0] * J[0][1];
    }
}

template <int DIM>
__global__ void k_wc_predict(int N, const uint8_t* __restrict__ flags, double* __restrict__ s,
                             double* __restrict__ pos, double* __restrict__ tdt) {
    const double dt = tdt[T_DT];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n == 0) tdt[T_TIME] += dt;  // Problem::updateTime with the step's dt
    if (n >= N) return;
    const bool fixed = flags[n] & F_FIXED;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        double* v = s + (size_t)d * N;
        const double a = s[(size_t)(DIM + 2 + d) * N + n];
        const double vh = v[n] + 0.5 * dt * a;
        v[n] = vh;
        if (!fixed) pos[(size_t)d * N + n] += vh * dt;
    }
}

// CDS_rho, m_buildF0 (ContEquation.inl:194-230) on the positions before the prediction moves
// them: cont_i = |e| sum_j MM_ij rho_j, the consistent mass times rho.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_wc_rho_pre(int E, int N, const int* __restrict__ conn,
                                                      const double* __restrict__ pos, const double* __restrict__ s,
                                                      WcConst k, double* __restrict__ elr) {
    using L = ElLayout<DIM>;
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    jacobian<DIM>(pos, N, nd, g);
    const double ae = g.detJ * k.refSize;
    double Rh[NPE];
#pragma unroll
    for (int j = 0; j < NPE; ++j) Rh[j] = s[(size_t)(DIM + 1) * N + nd[j]];
    double* out = elr + (size_t)e * L::NR;
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        double mr = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) mr += k.MM[i][j] * Rh[j];
        out[L::CONT + i] = ae * mr;
    }
}

// Continuity (m_buildSystemdpdt): per element node i, ML_i = |e| s_i and
//   cont_i = -dt (K0 s_i + K0' sum_j MM_ij p_j) |e| div v  [+ |e| sum_j MM_ij (p_j - p_i)  (Meduri)]
// CDS_drhodt (m_buildSystem): the same with rho for p and the D factor sum_j MM_ij rho_j;
// CDS_rho: ML only (cont is k_wc_rho_pre's).
template <int DIM, class R>
__global__ void __launch_bounds__(BLOCK) k_wc_cont_elem(int E, int N, const int* __restrict__ conn,
                                                        const double* __restrict__ pos, const double* __restrict__ s,
                                                        const double* __restrict__ tdt, WcConst k,
                                                        R* __restrict__ elr) {
    using L = ElLayout<DIM>;
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double dt = tdt[T_DT];
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    jacobian<DIM>(pos, N, nd, g);
    double A[DIM][NPE];
    area_gradients<DIM>(g, k.refSize, A);
    const double ae = g.detJ * k.refSize;
    R* out = elr + (size_t)e * L::NR;
    if (k.ver == 1) {
#pragma unroll
        for (int i = 0; i < NPE; ++i) out[L::ML + i] = (R)(ae * k.s[i]);
        return;
    }
    const int uf = k.ver == 0 ? DIM : DIM + 1;  // the unknown: p (dpdt) or rho (drhodt)
    double P[NPE];
    R adiv = 0;  // |e| div v
#pragma unroll
    for (int j = 0; j < NPE; ++j) {
        P[j] = s[(size_t)uf * N + nd[j]];
#pragma unroll
        for (int f = 0; f < DIM; ++f) adiv += (R)A[f][j] * (R)s[(size_t)f * N + nd[j]];
    }
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        R mp = 0, mdp = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) {
            mp += (R)k.MM[i][j] * (R)P[j];
            mdp += (R)k.MM[i][j] * (R)(P[j] - P[i]);
        }
        // sum_g w (K0 + K0' p_g) N_i, or sum_g w rho_g N_i
        const R swn = k.ver == 0 ? (R)(k.K0 * k.s[i]) + (R)k.K0p * mp : mp;
        R cont = -(R)dt * swn * adiv;
        if (k.meduri) cont += (R)ae * mdp;
        out[L::ML + i] = (R)(ae * k.s[i]);
        out[L::CONT + i] = cont;
    }
}

// p = p_i + sum cont / sum ML (Meduri) or sum cont / sum ML + p_i*0 (lumped); free nodes p = 0
// (m_applyBCdpdt, ContEquation.inl:343-348); rho from Tait-Murnaghan (:319-332).
template <int DIM, class R>
__global__ void k_wc_cont_node(int N, const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                               const uint8_t* __restrict__ ne_loc, const uint8_t* __restrict__ flags,
                               const R* __restrict__ elr, WcConst k, double* __restrict__ s) {
    using L = ElLayout<DIM>;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double m = 0, f0 = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const R* rec = elr + (size_t)ne_elem[q] * L::NR;
        const int i = ne_loc[q];
        m += (double)rec[L::ML + i];
        f0 += (double)rec[L::CONT + i];
    }
    double* P = s + (size_t)DIM * N;
    double* rho = s + (size_t)(DIM + 1) * N;
    if (k.ver != 0) {
        // density forms: m_applyBC (ContEquation.inl:177-192), rho = invM F0, then
        // p = (K0/K0') ((rho/rho*)^K0' - 1) (:305-317); CDS_rho's F0 is the whole consistent
        // mass product, CDS_drhodt's the difference form as for p
        double r;
        if (flags[n] & (F_FREE | F_FREE_SURFACE))
            r = k.rho_star;
        else
            r = k.ver == 1 ? f0 * (1 / m) : rho[n] + (1 / m) * f0;
        rho[n] = r;
        P[n] = (k.K0 / k.K0p) * (pow(r / k.rho_star, k.K0p) - 1);
        return;
    }
    if (flags[n] & F_FREE) {
        P[n] = 0.0;
        rho[n] = k.rho_star;  // ((K0'/K0) 0 + 1)^(1/K0') rho*
        return;
    }
    // both forms: p_i ML + sum_e (...) over ML  ->  p_i + (sum)/ML   (Meduri);
    // lumped form: (p_i ML - dt D v)/ML = p_i + (sum)/ML as well
    const double inv = 1 / m;
    const double p = P[n] + inv * f0;
    P[n] = p;
    if constexpr (sizeof(R) == 8) {
        rho[n] = pow((k.K0p / k.K0) * p + 1, 1 / k.K0p) * k.rho_star;
    } else {
        // rho - rho* = rho* expm1(log1p(K0' p / K0) / K0'), evaluated in FP32
        const float x = (float)((k.K0p / k.K0) * p);
        const float d = expm1f(log1pf(x) * (float)(1 / k.K0p));
        rho[n] = k.rho_star + k.rho_star * (double)d;
    }
}

// Momentum (m_buildSystem): per element node i and direction f,
//   MLrho_i = |e| sum_j MM_ij rho_j                      (diagBlock + lump of the rho-mass)
//   Fs_fi   = -(K v)_fi + A_fi sum_j s_j (p_j - p_i) + MLrho_i g_f
//   W_fi    = A_fi                                       (FP64; times p_i S at the node)
//   BoussinesqWC (T != null): the body force |e| sum_g w_g N_i rho_g (1 - alpha (T_g - Tr)) g_f,
//   and with phase change minus the Carman-Kozeny |e| sum_g w_g N_i ck_g v_f(g)
//   (diagBlock(getM) V, MomEquation.inl:271-276)
template <int DIM, class R>
__global__ void __launch_bounds__(BLOCK) k_wc_mom_elem(int E, int N, const int* __restrict__ conn,
                                                       const double* __restrict__ pos, const double* __restrict__ s,
                                                       WcConst k, R* __restrict__ elr, double* __restrict__ eld,
                                                       const double* __restrict__ T) {
    using L = ElLayout<DIM>;
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    jacobian<DIM>(pos, N, nd, g);
    double Ad[DIM][NPE];
    area_gradients<DIM>(g, k.refSize, Ad);
    const double ae = g.detJ * k.refSize;
    R A[DIM][NPE], V[DIM][NPE], Rh[NPE];
    double P[NPE];
#pragma unroll
    for (int j = 0; j < NPE; ++j) {
        P[j] = s[(size_t)DIM * N + nd[j]];
        Rh[j] = (R)s[(size_t)(DIM + 1) * N + nd[j]];
#pragma unroll
        for (int f = 0; f < DIM; ++f) {
            V[f][j] = (R)s[(size_t)f * N + nd[j]];
            A[f][j] = (R)Ad[f][j];
        }
    }
    // velocity gradient times |e|: Lg[a][b] = sum_j A[b][j] v_a(j); divA = trace
    R Lg[DIM][DIM];
    R divA = 0;
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
        for (int b = 0; b < DIM; ++b) {
            R t = 0;
#pragma unroll
            for (int j = 0; j < NPE; ++j) t += A[b][j] * V[a][j];
            Lg[a][b] = t;
        }
#pragma unroll
    for (int a = 0; a < DIM; ++a) divA += Lg[a][a];
    // K v with Ddev = [4/3 -2/3; -2/3 4/3] (normal) and 1 (shear), MomEquation.inl:63-83:
    //   (K v)_{f1,i} = mu_sum/|e| [ sum_j (A_i.A_j) v_f1(j) + sum_f2 A_f2,i Lg[f2][f1] - 2/3 A_f1,i divA ]
    const R kf = (R)(k.mu_sum / ae);
    double fbq[NPE] = {}, ckv[DIM][NPE] = {};
    if (T) {
        double te[NPE];
#pragma unroll
        for (int a = 0; a < NPE; ++a) te[a] = T[nd[a]];
        for (int q = 0; q < k.ng; ++q) {
            double Tg = 0, rg = 0, vg[DIM] = {};
#pragma unroll
            for (int a = 0; a < NPE; ++a) {
                Tg += k.gN[q][a] * te[a];
                rg += k.gN[q][a] * (double)Rh[a];
#pragma unroll
                for (int f = 0; f < DIM; ++f) vg[f] += k.gN[q][a] * (double)V[f][a];
            }
            const double fg = rg * (1 - k.alpha * (Tg - k.t_ref));
            double ckg = 0;
            if (k.ck) {
                const double fl = fl_wc(k, Tg);
                ckg = k.ck_c * (1 - fl) * (1 - fl) / (fl * fl * fl + k.ck_eps);
            }
#pragma unroll
            for (int i = 0; i < NPE; ++i) {
                fbq[i] += (fg * k.gN[q][i]) * k.gw[q];
#pragma unroll
                for (int f = 0; f < DIM; ++f) ckv[f][i] += (ckg * k.gN[q][i] * vg[f]) * k.gw[q];
            }
        }
    }
    R* out = elr + (size_t)e * L::NR;
    double* outd = eld + (size_t)e * L::ND;
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        R mr = 0, dp = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) {
            mr += (R)k.MM[i][j] * Rh[j];
            dp += (R)k.s[j] * (R)(P[j] - P[i]);
        }
        const R mlr = (R)ae * mr;
        out[L::MLR + i] = mlr;
        R gg[NPE];
#pragma unroll
        for (int j = 0; j < NPE; ++j) {
            R t = 0;
#pragma unroll
            for (int f = 0; f < DIM; ++f) t += A[f][i] * A[f][j];
            gg[j] = t;
        }
#pragma unroll
        for (int f1 = 0; f1 < DIM; ++f1) {
            R kv = 0;
#pragma unroll
            for (int j = 0; j < NPE; ++j) kv += gg[j] * V[f1][j];
#pragma unroll
            for (int f2 = 0; f2 < DIM; ++f2) kv += A[f2][i] * Lg[f2][f1];
            kv -= (R)(2.0 / 3.0) * A[f1][i] * divA;
            if (T)
                out[L::FS + f1 * NPE + i] = -kf * kv + A[f1][i] * dp + (R)(ae * fbq[i]) * (R)k.g[f1] -
                                            (R)(ae * ckv[f1][i]);
            else
                out[L::FS + f1 * NPE + i] = -kf * kv + A[f1][i] * dp + mlr * (R)k.g[f1];
            outd[f1 * NPE + i] = Ad[f1][i];
        }
    }
}

// a = F / M with the surface tension of the node's free-surface facets (MomEquation.inl:
// 311-335) and the momentum BCs (:341-372); v = v1/2 + dt/2 a.  Also the per-node quantities
// of computeNextDT: max(u^2, c^2) and mu/rho.
template <int DIM, class R>
__global__ void k_wc_mom_node(int N, const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                              const uint8_t* __restrict__ ne_loc, const uint8_t* __restrict__ flags,
                              const R* __restrict__ elr, const double* __restrict__ eld,
                              const double* __restrict__ vbc, const double* __restrict__ tdt, WcConst k,
                              double* __restrict__ s, R* __restrict__ nodal, const double* __restrict__ fst) {
    using L = ElLayout<DIM>;
    constexpr int NPE = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const double dt = tdt[T_DT];
    double m = 0, F[DIM], W[DIM];
#pragma unroll
    for (int f = 0; f < DIM; ++f) F[f] = W[f] = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q], i = ne_loc[q];
        const R* rec = elr + (size_t)e * L::NR;
        const double* recd = eld + (size_t)e * L::ND;
        m += (double)rec[L::MLR + i];
#pragma unroll
        for (int f = 0; f < DIM; ++f) {
            F[f] += (double)rec[L::FS + f * NPE + i];
            W[f] += recd[f * NPE + i];
        }
    }
    const double pS = s[(size_t)DIM * N + n] * k.S;
#pragma unroll
    for (int f = 0; f < DIM; ++f) F[f] += pS * W[f];
    if (fst)
#pragma unroll
        for (int f = 0; f < DIM; ++f) F[f] += fst[(size_t)f * N + n];
    double inv = 1 / m;
    const uint8_t fl = flags[n];
    if ((fl & F_FREE) && !(fl & F_BOUND)) {  // free fall (MomEquation.inl:347-354)
#pragma unroll
        for (int f = 0; f < DIM; ++f) F[f] = k.g[f];
        inv = 1;
    } else if ((fl & F_BOUND) && (fl & F_DIRICHLET)) {  // V_bc used as acceleration (:355-371)
#pragma unroll
        for (int f = 0; f < DIM; ++f) F[f] = vbc[(size_t)f * N + n];
        inv = 1;
    }
    double u2 = 0;
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        const double a = inv * F[f];
        s[(size_t)(DIM + 2 + f) * N + n] = a;
        const double v = s[(size_t)f * N + n] + 0.5 * dt * a;
        s[(size_t)f * N + n] = v;
        u2 += v * v;
    }
    if (nodal) {
        const double p = s[(size_t)DIM * N + n], rho = s[(size_t)(DIM + 1) * N + n];
        const double c2 = (k.K0 + k.K0p * p) / rho;
        nodal[n] = (R)fmax(u2, c2);
        nodal[(size_t)N + n] = (R)(fmax(k.mu, k.k_cv) / rho);
    }
}

// computeNextDT: dt^2_e = sc^2 he^2 / max_nodes(max(u^2, c^2), 4 alpha^2/he^2), he = 2 Rin;
// block min, grid min by the last block, dt = min(sqrt(min), maxDT).
template <int DIM, class R>
__global__ void __launch_bounds__(BLOCK) k_wc_dt(int E, int N, const int* __restrict__ conn,
                                                 const double* __restrict__ pos, const R* __restrict__ nodal,
                                                 WcConst k, double* __restrict__ partials, double* __restrict__ tdt) {
    __shared__ double sh[32];
    double best = 1.79769313486231570e308;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        int nd[DIM + 1];
        load_nodes<DIM>(conn, E, e, nd);
        double X[DIM + 1][DIM];
#pragma unroll
        for (int a = 0; a <= DIM; ++a)
#pragma unroll
            for (int d = 0; d < DIM; ++d) X[a][d] = pos[(size_t)d * N + nd[a]];
        R he;
        if constexpr (DIM == 2) {  // Element::getRin 2D (Element.cpp:228-241)
            const double j00 = X[1][0] - X[0][0], j01 = X[2][0] - X[0][0];
            const double j10 = X[1][1] - X[0][1], j11 = X[2][1] - X[0][1];
            const R size = (R)((j00 * j11 - j10 * j01) * k.refSize);
            auto dist = [&](int a, int b) {
                const R dx = (R)(X[a][0] - X[b][0]), dy = (R)(X[a][1] - X[b][1]);
                return sqrt(dx * dx + dy * dy);
            };
            const R sp = (dist(0, 1) + dist(1, 2) + dist(0, 2)) / (R)2;
            he = (R)2 * (size / sp);
        } else {  // Element::getRin 3D (Element.cpp:242-293)
            Geom<3> g;
            jacobian<3>(pos, N, nd, g);
            const R size = (R)(g.detJ * k.refSize);
            auto nrm = [&](int a0, int a1, int a2) {
                const R ux = (R)(X[a1][0] - X[a0][0]), uy = (R)(X[a1][1] - X[a0][1]), uz = (R)(X[a1][2] - X[a0][2]);
                const R wx = (R)(X[a2][0] - X[a0][0]), wy = (R)(X[a2][1] - X[a0][1]), wz = (R)(X[a2][2] - X[a0][2]);
                const R cx = uy * wz - uz * wy, cy = uz * wx - ux * wz, cz = ux * wy - uy * wx;
                return sqrt(cx * cx + cy * cy + cz * cz);
            };
            const R sum = nrm(0, 1, 2) + nrm(0, 3, 2) + nrm(0, 1, 3) + nrm(3, 1, 2);
            he = (R)2 * ((R)6 * size / sum);
        }
        R m1 = 0, m2 = 0;
#pragma unroll
        for (int a = 0; a <= DIM; ++a) {
            m1 = fmax(m1, nodal[nd[a]]);
            m2 = fmax(m2, nodal[(size_t)N + nd[a]]);
        }
        const R maxSq = fmax(m1, (R)4 * m2 * m2 / (he * he));
        best = fmin(best, (double)((R)(k.sc * k.sc) * he * he / maxSq));
    }
    best = block_min<BLOCK>(best, sh);
    __shared__ bool last;
    unsigned* ticket = reinterpret_cast<unsigned*>(tdt + T_TICKET);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = best;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double mn = 1.79769313486231570e308;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) mn = fmin(mn, ((volatile double*)partials)[i]);
    mn = block_min<BLOCK>(mn, sh);
    if (threadIdx.x == 0) {
        tdt[T_DT] = fmin(sqrt(mn), k.max_dt);
        tdt[T_MIN] = mn;
        *ticket = 0u;
    }
}

// per-node dt quantities from the current state (for pfg_next_dt outside a step)
template <class R>
__global__ void k_wc_nodal(int N, int dim, const double* __restrict__ s, WcConst k, R* __restrict__ nodal) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double u2 = 0;
    for (int f = 0; f < dim; ++f) u2 += s[(size_t)f * N + n] * s[(size_t)f * N + n];
    const double p = s[(size_t)dim * N + n], rho = s[(size_t)(dim + 1) * N + n];
    nodal[n] = (R)fmax(u2, (k.K0 + k.K0p * p) / rho);
    nodal[(size_t)N + n] = (R)(fmax(k.mu, k.k_cv) / rho);
}

template <int DIM>
__global__ void k_wc_mass(int E, int N, const int* __restrict__ conn, const double* __restrict__ pos,
                          const double* __restrict__ s, double refSize, double* partials, unsigned* ticket,
                          double* out) {
    __shared__ double sh[32];
    double acc = 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        int nd[DIM + 1];
        load_nodes<DIM>(conn, E, e, nd);
        Geom<DIM> g;
        jacobian<DIM>(pos, N, nd, g);
        double mid = 0;
#pragma unroll
        for (int a = 0; a <= DIM; ++a) mid += s[(size_t)(DIM + 1) * N + nd[a]];
        mid /= (double)(DIM + 1);
        acc += mid * (g.detJ * refSize);
    }
    grid_sum_last<BLOCK>(acc, partials, ticket, sh, out);
}

// dt in both precisions: the plain step reads the double, the mixed step the float copy
// Every instance's time-step slot (8 doubles each; one slot unless the mixed form is batched).
__global__ void k_set_dt(double* tdt, double v, int n_slots) {
    for (int i = 0; i < n_slots; ++i) {
        double* t = tdt + 8 * i;
        t[T_DT] = v;
        reinterpret_cast<float*>(t + 4)[0] = (float)v;
    }
}

__global__ void k_set_time(double* tdt, double t, double v, int n_slots) {
    for (int i = 0; i < n_slots; ++i) {
        double* s = tdt + 8 * i;
        s[T_DT] = v;
        s[T_TIME] = t;
        reinterpret_cast<float*>(s + 4)[0] = (float)v;
    }
}

bool mixed(pfg_ctx* c) { return c->prm.precision == PFG_PREC_MIXED; }

template <int DIM>
int launch_step(pfg_ctx* c, bool adapt, const WcConst& k) {
    using R = double;
    const int N = c->N, E = c->E;
    double* s = ptr<double>(c->ws);
    R* elr = ptr<R>(c->wc_el);
    double* eld = ptr<double>(c->wc_eld);
    R* nodal = ptr<R>(c->wc_nodal);
    double* tdt = ptr<double>(c->wc_dt);
    const int gn = div_up(N, BLOCK), ge = std::max(1, div_up(E, BLOCK));
    if (k.ver == 1 && E > 0) {  // CDS_rho: F0 = M rho on the positions before the move
        prof_begin(c, PH_WC_CONT_ELEM);
        k_wc_rho_pre<DIM><<<ge, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), s, k, elr);
        prof_end(c, PH_WC_CONT_ELEM);
    }
    prof_begin(c, PH_WC_PREDICT);
    k_wc_predict<DIM><<<gn, BLOCK, 0, c->stream>>>(N, ptr<uint8_t>(c->flags), s, ptr<double>(c->pos), tdt);
    prof_end(c, PH_WC_PREDICT);
    if (k.bq) {  // BoussinesqWC: the heat step between the prediction and the continuity equation
        int rc = wc_heat_launch(c, tdt);
        if (rc) return rc;
    }
    if (E > 0) {
        prof_begin(c, PH_WC_CONT_ELEM);
        k_wc_cont_elem<DIM, R><<<ge, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), s, tdt, k,
                                                            elr);
        prof_end(c, PH_WC_CONT_ELEM);
    }
    prof_begin(c, PH_WC_CONT_NODE);
    k_wc_cont_node<DIM, R><<<gn, BLOCK, 0, c->stream>>>(N, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem),
                                                        ptr<uint8_t>(c->ne_loc), ptr<uint8_t>(c->flags), elr, k, s);
    prof_end(c, PH_WC_CONT_NODE);
    if (E > 0) {
        prof_begin(c, PH_WC_MOM_ELEM);
        k_wc_mom_elem<DIM, R><<<ge, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), s, k, elr,
                                                           eld, k.bq ? ptr<double>(c->heat_t) : nullptr);
        prof_end(c, PH_WC_MOM_ELEM);
    }
    prof_begin(c, PH_WC_MOM_NODE);
    const FstArgs fa = fst_args(c);
    if (fa.nodes)
        k_fst<DIM, double><<<div_up(fa.n_nodes, BLOCK), BLOCK, 0, c->stream>>>(
            fa, E, ptr<int>(c->conn), PosF64{ptr<double>(c->pos), N}, N, ptr<double>(c->fst_force));
    k_wc_mom_node<DIM, R><<<gn, BLOCK, 0, c->stream>>>(N, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem),
                                                       ptr<uint8_t>(c->ne_loc), ptr<uint8_t>(c->flags), elr, eld,
                                                       ptr<double>(c->vbc), tdt, k, s, adapt ? nodal : nullptr,
                                                       fst_force<double>(c));
    prof_end(c, PH_WC_MOM_NODE);
    if (adapt && E > 0) {
        const int grid = std::min(c->max_grid, ge);
        prof_begin(c, PH_WC_DT);
        k_wc_dt<DIM, R><<<grid, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), nodal, k,
                                                       ptr<double>(c->red), tdt);
        prof_end(c, PH_WC_DT);
    }
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

int launch_any(pfg_ctx* c, bool adapt) {
    if (mixed(c)) return wcm_launch_step(c, adapt);
    const WcConst k = make_const(c);
    return c->dim == 2 ? launch_step<2>(c, adapt, k) : launch_step<3>(c, adapt, k);
}

template <int DIM>
int dt_only(pfg_ctx* c, const WcConst& k) {
    using R = double;
    const int E = c->E, N = c->N;
    if (E == 0) return fail(c, PFG_ERR_STATE, "no elements");
    k_wc_nodal<R><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, DIM, ptr<double>(c->ws), k, ptr<R>(c->wc_nodal));
    const int grid = std::min(c->max_grid, div_up(E, BLOCK));
    k_wc_dt<DIM, R><<<grid, BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), ptr<R>(c->wc_nodal),
                                                   k, ptr<double>(c->red), ptr<double>(c->wc_dt));
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

// Capture one step (per dt mode) into a CUDA graph; replayed for every step.
int step_graph(pfg_ctx* c, bool adapt, cudaGraphExec_t* out) {
    cudaGraphExec_t& ex = c->wc_graph[adapt ? 1 : 0];
    if (!ex) {
        cudaGraph_t g = nullptr;
        PFG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int rc = launch_any(c, adapt);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            ex = nullptr;
            return cuda_fail(c, e, "cudaGraphInstantiate");
        }
    }
    *out = ex;
    return PFG_OK;
}

}  // namespace

void wc_release_graphs(pfg_ctx* c) {
    for (auto& g : c->wc_graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

// Buffers.  Plain form: ws = FP64 states (2d+2)N, wc_el/wc_eld = element partials, wc_nodal =
// FP64 CFL quantities.  Mixed form: ws = double-float state, wc_el = FP32 element records,
// wc_nodal = FP32 CFL quantities, wc_eld = FP32 copy of the Dirichlet velocities.
int wc_alloc(pfg_ctx* c) {
    const size_t N = c->N, E = std::max(c->E, 1);
    int rc;
    wc_release_graphs(c);
    if (mixed(c)) {
        c->wc_cur = 0;
        const size_t elb = std::max(wcm_elem_bytes(c), (size_t)(4096 + 64) * sizeof(float));
        if ((rc = ensure(c, c->ws, wcm_state_bytes(c))) || (rc = ensure(c, c->wc_el, elb)) ||
            (rc = ensure(c, c->wc_eld, sizeof(float) * c->dim * N)) ||
            (rc = ensure(c, c->wc_nodal, sizeof(float) * 2 * N)) || (rc = ensure(c, c->wc_dt, 64)))
            return rc;
        PFG_CUDA(c, cudaMemsetAsync(c->ws.p, 0, wcm_state_bytes(c), c->stream));
        if ((rc = wcm_positions_in(c)) || (rc = wcm_vbc_refresh(c))) return rc;
    } else {
        const int nr = c->dim == 2 ? ElLayout<2>::NR : ElLayout<3>::NR;
        const int ndd = c->dim == 2 ? ElLayout<2>::ND : ElLayout<3>::ND;
        if ((rc = ensure(c, c->ws, sizeof(double) * (2 * c->dim + 2) * N)) ||
            (rc = ensure(c, c->wc_el, sizeof(double) * (size_t)nr * E)) ||
            (rc = ensure(c, c->wc_eld, sizeof(double) * ndd * E)) ||
            (rc = ensure(c, c->wc_nodal, sizeof(double) * 2 * N)) || (rc = ensure(c, c->wc_dt, 64)))
            return rc;
        PFG_CUDA(c, cudaMemsetAsync(c->ws.p, 0, sizeof(double) * (2 * c->dim + 2) * N, c->stream));
    }
    c->n_wc_inst = 1;
    PFG_CUDA(c, cudaMemsetAsync(c->wc_dt.p, 0, 64, c->stream));
    k_set_time<<<1, 1, 0, c->stream>>>(ptr<double>(c->wc_dt), c->host_time, c->prm.max_dt, 1);
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wc_set_time(pfg_ctx* c, double time, double next_dt) {
    k_set_time<<<1, 1, 0, c->stream>>>(ptr<double>(c->wc_dt), time, next_dt, c->n_wc_inst);
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->host_time = time;
    return PFG_OK;
}

int wc_dirichlet_changed(pfg_ctx* c) {
    if (!mixed(c)) return PFG_OK;
    int rc = wcm_vbc_refresh(c);
    if (rc) return rc;
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

// Make ctx->pos current (the mixed form keeps positions as double-float pairs).
int wc_sync_positions(pfg_ctx* c) {
    if (!mixed(c)) return PFG_OK;
    return wcm_positions_out(c);
}

int wc_set_states(pfg_ctx* c, const double* h) {
    if (mixed(c)) return wcm_set_states(c, h);
    const size_t n = (size_t)(2 * c->dim + 2) * c->N;
    PFG_CUDA(c, cudaMemcpyAsync(c->ws.p, h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wc_get_states(pfg_ctx* c, double* h) {
    if (mixed(c)) return wcm_get_states(c, h);
    const size_t n = (size_t)(2 * c->dim + 2) * c->N;
    PFG_CUDA(c, cudaMemcpyAsync(h, c->ws.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wc_enqueue(pfg_ctx* c, double dt, int nsteps) {
    const bool adapt = !(dt > 0);
    if (c->prm.boussinesq) {
        bool changed = false;
        int rc = wc_heat_prepare(c, &changed);
        if (rc) return rc;
        if (changed) wc_release_graphs(c);
    }
    if (!adapt) {
        k_set_dt<<<1, 1, 0, c->stream>>>(ptr<double>(c->wc_dt), dt, c->n_wc_inst);
        PFG_CHECK_LAUNCH(c);
    }
    if (c->prof) {
        // phase timers need events between kernels: launch each phase as its own kernel
        for (int i = 0; i < nsteps; ++i) {
            int rc = launch_any(c, adapt);
            if (rc) return rc;
        }
    } else {
        cudaGraphExec_t ex;
        int rc = step_graph(c, adapt, &ex);
        if (rc) return rc;
        for (int i = 0; i < nsteps; ++i) PFG_CUDA(c, cudaGraphLaunch(ex, c->stream));
    }
    c->wc_pending += nsteps;
    return PFG_OK;
}

int wc_sync(pfg_ctx* c, pfg_step_status* st) {
    std::memset(st, 0, sizeof(*st));
    PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, c->wc_dt.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    st->converged = 1;
    st->steps_done = c->wc_pending;
    st->dt = c->h_scalars[0];
    st->time = c->h_scalars[1];
    c->host_time = st->time;
    c->wc_pending = 0;
    return PFG_OK;
}

// Batched mixed contexts: every instance's dt and time (slot i of wc_dt) into st[i].
int wc_sync_batch(pfg_ctx* c, pfg_step_status* st) {
    const int K = c->n_wc_inst;
    std::vector<double> slots((size_t)8 * K);
    PFG_CUDA(c, cudaMemcpyAsync(slots.data(), c->wc_dt.p, sizeof(double) * slots.size(), cudaMemcpyDeviceToHost,
                                c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int i = 0; i < K; ++i) {
        std::memset(&st[i], 0, sizeof(st[i]));
        st[i].converged = 1;
        st[i].steps_done = c->wc_pending;
        st[i].dt = slots[(size_t)8 * i + T_DT];
        st[i].time = slots[(size_t)8 * i + T_TIME];
    }
    c->host_time = st[0].time;
    c->wc_pending = 0;
    return PFG_OK;
}

int wc_steps(pfg_ctx* c, double dt, int nsteps, pfg_step_status* st) {
    c->wc_pending = 0;
    int rc = wc_enqueue(c, dt, nsteps);
    if (rc) return rc;
    return wc_sync(c, st);
}

int wc_next_dt(pfg_ctx* c, double* dt) {
    int rc;
    if (mixed(c)) {
        rc = wcm_next_dt(c);
    } else {
        const WcConst k = make_const(c);
        rc = c->dim == 2 ? dt_only<2>(c, k) : dt_only<3>(c, k);
    }
    if (rc) return rc;
    PFG_CUDA(c, cudaMemcpyAsync(dt, c->wc_dt.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

int wc_mass(pfg_ctx* c, double* out) {
    double* red = ptr<double>(c->red);
    double* res = red + c->max_grid * 4 + 40;
    unsigned* ticket = reinterpret_cast<unsigned*>(red + c->max_grid * 4 + 48);
    const GaussConst g = gauss_const(c->dim);
    const int grid = std::max(1, std::min(c->max_grid, div_up(std::max(c->E, 1), BLOCK)));
    const double* s = ptr<double>(c->ws);
    int rc;
    if (mixed(c)) {
        // FP64 sum over an FP64 image of the state
        const size_t n = (size_t)(2 * c->dim + 2) * c->N;
        if ((rc = ensure(c, c->stage, sizeof(double) * n)) || (rc = wcm_state_to_stage(c)) ||
            (rc = wcm_positions_out(c)))
            return rc;
        s = ptr<double>(c->stage);
    }
    if (c->dim == 2)
        k_wc_mass<2><<<grid, BLOCK, 0, c->stream>>>(c->E, c->N, ptr<int>(c->conn), ptr<double>(c->pos), s, g.refSize,
                                                    red, ticket, res);
    else
        k_wc_mass<3><<<grid, BLOCK, 0, c->stream>>>(c->E, c->N, ptr<int>(c->conn), ptr<double>(c->pos), s, g.refSize,
                                                    red, ticket, res);
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, res, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    *out = c->h_scalars[0];
    return PFG_OK;
}

}  // namespace pfg
