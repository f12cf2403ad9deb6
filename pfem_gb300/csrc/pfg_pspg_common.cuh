// PSPG element formulas shared by the FP64 path (pfg_pspg.cu) and the mixed-precision,
// multi-instance path (pfg_pspg_mixed.cu).  Header-only device code.
//
// Element matrices are closed forms of the reference's Gauss-point products
// (MatricesBuilder.inl:216-386), with the sums over Gauss points taken from the same tables:
//   M_ij  = rho |e| sum_g w_g N_i N_j                     (getM, factor rho)
//   K     = mu |e| [d_f1f2 gradN_i.gradN_j + dN_i/dx_f2 dN_j/dx_f1]   (B^T Ddev B, Ddev=diag(2..,1..))
//   D_ij,f = |e| s_i dN_j/dx_f,  s_i = sum_g w_g N_i      (getD, factor 1, m = [1..1,0..])
//   C_ij,f = |e| dN_i/dx_f s_j                            (getC)
//   L_ij  = |e| (sum_g w_g / rho) gradN_i.gradN_j         (getL, factor 1/rho)
//   F_i,f = rho |e| g_f s_i,  H_i = |e| sum_g w_g gradN_i.g  (getF, getH)
// and the element system of m_buildAbPSPG (MomContEquationPSPG.inl:30-53):
//   [ M/dt (x) I + K      -D^T   ] [v]   [ F + M/dt v_prev         ]
//   [ tau/dt C + D       tau L   ] [p] = [ tau H + tau/dt C v_prev ]
#pragma once

#include "pfg_device.cuh"
#include "pfg_fst.cuh"

namespace pfg {

// Coefficients of one fluid (one instance) and the Gauss tables.
struct PspgCoef {
    double rho, dt, refSize;
    double mu_sum;    // sum_g mu w_g          (getK factor)
    double l_sum;     // sum_g (1/rho) w_g     (getL factor)
    double h_sum;     // sum_g w_g             (getH factor 1)
};

// Problem "Boussinesq" (MomContEquation.inl:164-199): the body-force factor rho (1 - alpha (T - Tr))
// and the PSPG gravity factor 1 - alpha (T - Tr) at each Gauss point, T interpolated from the node
// temperatures.  Summed over the Gauss points they are, per element node i,
//   F:  rho [(1 + alpha Tr) s_i - alpha sum_k MM_ik T_k]     H:  (1 + alpha Tr) sum_g w_g - alpha sum_k s_k T_k
// with s_i = sum_g w_g N_i and MM_ik = sum_g w_g N_i N_k.  T == nullptr: not Boussinesq.
struct BoussArgs {
    const double* T;
    double alpha, Tr;
};

inline BoussArgs boussinesq_args(pfg_ctx* c) {
    BoussArgs b{nullptr, 0.0, 0.0};
    if (c->prm.boussinesq) {
        b.T = ptr<double>(c->heat_t);
        b.alpha = c->prm.alpha_t;
        b.Tr = c->prm.t_ref;
    }
    return b;
}

struct PspgTables {
    double MM[4][4];  // sum_g w N_i N_j
    double s[4];      // sum_g w N_i
    double g[3];
};

// Element data layout (structure of arrays, stride E):
//   [detJ, tau, gradN[f][i] (f-major), ksum]
// ksum = sum_g mu_e w_g, the viscous factor of getK (MatricesBuilder.inl:276-290)
template <int DIM>
constexpr int ed_count() {
    return 3 + DIM * (DIM + 1);
}
template <int DIM>
constexpr int ed_ksum() {
    return 2 + DIM * (DIM + 1);
}

// The viscosity law of the K factor (setKcomputeFactor, MomContEquation.inl:102-131): mu, or
// for a Bingham fluid (problem "Bingham", tau0 > 0) mu + tau0 (1 - exp(-mReg gd)) / gd (tau0 mReg
// when gd < 1e-15), gd = sqrt(V^T B^T ddev B V) of the element's iterate velocities, ddev =
// diag(2, 2, 1) in 2D and diag(2, 2, 2, 1, 1, 1) in 3D (:73-94).  Summed over the Gauss points
// like the reference's factor.
struct ViscArgs {
    double w[4];
    int ng;
    double tau0, mreg;
};

inline ViscArgs visc_args(const pfg_ctx* c) {
    const GaussConst g = gauss_const(c->dim);
    ViscArgs v{};
    v.ng = g.n;
    for (int i = 0; i < g.n; ++i) v.w[i] = g.w[i];
    v.tau0 = c->prm.tau0;
    v.mreg = c->prm.m_reg;
    return v;
}

template <int DIM>
__device__ __forceinline__ double k_sum(const ViscArgs& va, double mu, const double (&G)[DIM][DIM + 1],
                                        const double* __restrict__ q, int N, const int (&nd)[DIM + 1]) {
    double mue = mu;
    if (va.tau0 > 0) {
        double v[DIM][DIM + 1];
#pragma unroll
        for (int f = 0; f < DIM; ++f)
#pragma unroll
            for (int i = 0; i <= DIM; ++i) v[f][i] = q[(size_t)f * N + nd[i]];
        // strain rates (getB, MatricesBuilder.inl:129-164): normal d v_f / d x_f and engineering shears
        double e[DIM][DIM];
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) {
                double s = 0;
#pragma unroll
                for (int i = 0; i <= DIM; ++i) s += G[b][i] * v[a][i];
                e[a][b] = s;  // d v_a / d x_b
            }
        double gd2 = 0;
#pragma unroll
        for (int a = 0; a < DIM; ++a) gd2 += 2 * e[a][a] * e[a][a];
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = a + 1; b < DIM; ++b) {
                const double sh = e[a][b] + e[b][a];
                gd2 += sh * sh;
            }
        const double gd = sqrt(gd2);
        mue = mu + (gd < 1e-15 ? va.tau0 * va.mreg : va.tau0 * (1 - exp(-va.mreg * gd)) / gd);
    }
    double s = 0;
    for (int g = 0; g < va.ng; ++g) s += mue * va.w[g];
    return s;
}

// Block (n, m) of the assembled matrix before boundary conditions: the sum, in ascending
// element order, of the element-matrix entries of the elements containing both nodes (the
// order in which Eigen's setFromTriplets sums the reference's triplets).
template <int DIM>
__device__ __forceinline__ void pspg_pair_block(int n, int m, int E, const int* __restrict__ ne_ptr,
                                                const int* __restrict__ ne_elem, const uint8_t* __restrict__ ne_loc,
                                                const int* __restrict__ conn, const double* __restrict__ ed,
                                                const PspgCoef& k, const PspgTables& t,
                                                double (&acc)[DIM + 1][DIM + 1]) {
    constexpr int NPE = DIM + 1;
#pragma unroll
    for (int a = 0; a < NPE; ++a)
#pragma unroll
        for (int b = 0; b < NPE; ++b) acc[a][b] = 0;
    const double inv_dt = 1 / k.dt;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        int j = -1;
#pragma unroll
        for (int jj = 0; jj < NPE; ++jj)
            if (__ldg(conn + (size_t)jj * E + e) == m) j = jj;
        if (j < 0) continue;
        const int i = ne_loc[q];
        const double detJ = ed[e];
        const double tau = ed[(size_t)E + e];
        const double ae = detJ * k.refSize;
        double gi[DIM], gj[DIM];
#pragma unroll
        for (int f = 0; f < DIM; ++f) {
            gi[f] = ed[(size_t)(2 + f * NPE + i) * E + e];
            gj[f] = ed[(size_t)(2 + f * NPE + j) * E + e];
        }
        double dot = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f) dot += gi[f] * gj[f];
        const double mij = inv_dt * (k.rho * t.MM[i][j] * ae);
        const double kf = ae * ed[(size_t)ed_ksum<DIM>() * E + e];
#pragma unroll
        for (int f1 = 0; f1 < DIM; ++f1) {
#pragma unroll
            for (int f2 = 0; f2 < DIM; ++f2) {
                const double kv = kf * ((f1 == f2 ? dot : 0.0) + gi[f2] * gj[f1]);
                acc[f1][f2] += (f1 == f2 ? mij : 0.0) + kv;
            }
            acc[f1][DIM] += -(ae * t.s[j] * gi[f1]);
        }
        const double ctau = tau * inv_dt;
#pragma unroll
        for (int f2 = 0; f2 < DIM; ++f2) acc[DIM][f2] += ctau * (ae * gi[f2] * t.s[j]) + ae * t.s[i] * gj[f2];
        acc[DIM][DIM] += tau * (ae * k.l_sum * dot);
    }
}

// Right-hand side of node n (doublet scatter :93-97,:140-144 in element order) followed by
// m_applyBCPSPG: the surface tension of the node's free-surface facets (:155-187, facet
// order) and the node boundary conditions (:189-232).
template <int DIM>
__device__ __forceinline__ void pspg_node_rhs(int n, int N, int E, const int* __restrict__ ne_ptr,
                                              const int* __restrict__ ne_elem, const uint8_t* __restrict__ ne_loc,
                                              const int* __restrict__ conn, const double* __restrict__ ed,
                                              uint8_t fl, const double* __restrict__ q_prev,
                                              const double* __restrict__ vbc, bool apply_bc, const PspgCoef& k,
                                              const PspgTables& t, const double* __restrict__ fst,
                                              const BoussArgs& bq, double (&bv)[DIM], double& bp) {
    constexpr int NPE = DIM + 1;
#pragma unroll
    for (int f = 0; f < DIM; ++f) bv[f] = 0;
    bp = 0;
    const double inv_dt = 1 / k.dt;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        const int i = ne_loc[q];
        int nd[NPE];
        load_nodes<DIM>(conn, E, e, nd);
        const double detJ = ed[e];
        const double tau = ed[(size_t)E + e];
        const double ae = detJ * k.refSize;
        double gi[DIM];
#pragma unroll
        for (int f = 0; f < DIM; ++f) gi[f] = ed[(size_t)(2 + f * NPE + i) * E + e];
        double vp[DIM][NPE];
#pragma unroll
        for (int f = 0; f < DIM; ++f)
#pragma unroll
            for (int j = 0; j < NPE; ++j) vp[f][j] = q_prev[(size_t)f * N + nd[j]];
        // Gauss sums of the body-force factor over N_i and of the gravity factor
        double fs = t.s[i], hs = k.h_sum;
        if (bq.T) {
            double mt = 0, st = 0;
#pragma unroll
            for (int j = 0; j < NPE; ++j) {
                const double Tj = bq.T[nd[j]];
                mt += t.MM[i][j] * Tj;
                st += t.s[j] * Tj;
            }
            const double c0 = 1 + bq.alpha * bq.Tr;
            fs = c0 * t.s[i] - bq.alpha * mt;
            hs = c0 * k.h_sum - bq.alpha * st;
        }
        // momentum rows: F + (M/dt) v_prev
#pragma unroll
        for (int f = 0; f < DIM; ++f) {
            double mv = 0;
#pragma unroll
            for (int j = 0; j < NPE; ++j) mv += inv_dt * (k.rho * t.MM[i][j] * ae) * vp[f][j];
            const double F = ae * (k.rho * fs * t.g[f]);
            bv[f] += F + mv;
        }
        // continuity row: tau H + (tau/dt) C v_prev
        double gdot = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f) gdot += gi[f] * t.g[f];
        const double H = tau * (ae * hs * gdot);
        double cv = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f)
#pragma unroll
            for (int j = 0; j < NPE; ++j) cv += (ae * gi[f] * t.s[j]) * vp[f][j];
        bp += H + (tau * inv_dt) * cv;
    }
    if (apply_bc) {
        if (fst)
#pragma unroll
            for (int f = 0; f < DIM; ++f) bv[f] += fst[(size_t)f * N + n];
        if (fl & F_FREE) {
            bp = 0;
            if (!(fl & F_BOUND))
#pragma unroll
                for (int f = 0; f < DIM; ++f) bv[f] = q_prev[(size_t)f * N + n] + k.dt * t.g[f];
        }
        if ((fl & F_BOUND) && (fl & F_DIRICHLET))
#pragma unroll
            for (int f = 0; f < DIM; ++f) bv[f] = vbc[(size_t)f * N + n];
    }
}

// Writes the (n, m) block into the CSR values with the identity rows and the Dirichlet column
// elimination of m_applyBCPSPG (:108-128, :216-229); the eliminated entries' share of the
// right-hand side goes to rhs (when non-null).  val32, when non-null, receives the FP32 rounding
// of each value.
template <int DIM>
__device__ __forceinline__ void pspg_write_block(int n, int m, int N, int deg, int rank, uint8_t fn, uint8_t fm,
                                                 const int* __restrict__ row_ptr, const double (&acc)[DIM + 1][DIM + 1],
                                                 bool apply_bc, const double* __restrict__ vbc,
                                                 double* __restrict__ rhs, double* __restrict__ val,
                                                 float* __restrict__ val32) {
    const bool bound = fn & F_BOUND;
    const bool mdir = apply_bc && (fm & F_BOUND) && (fm & F_DIRICHLET);
#pragma unroll
    for (int f1 = 0; f1 <= DIM; ++f1) {
        const int r = n + f1 * N;
        const int rp = row_ptr[r];
        if (f1 < DIM && bound) {  // identity velocity rows of bound nodes (:119-126)
            if (m == n) {
                val[rp] = 1.0;
                if (val32) val32[rp] = 1.0f;
            }
            continue;
        }
#pragma unroll
        for (int f2 = 0; f2 <= DIM; ++f2) {
            double a = acc[f1][f2];
            // Dirichlet column elimination (:216-229): value moved to the RHS, entry kept at 0
            if (mdir && f2 < DIM && !(m == n && f1 == f2)) {
                const double vb = vbc[(size_t)f2 * N + m];
                if (vb != 0.0 && rhs) atomicAdd(rhs + r, -a * vb);
                a = 0.0;
            }
            val[rp + f2 * deg + rank] = a;
            if (val32) val32[rp + f2 * deg + rank] = (float)a;
        }
    }
}

}  // namespace pfg
