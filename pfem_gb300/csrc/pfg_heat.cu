// Heat equation of the incompressible solver (HeatEqIncompNewton, IncompNewton/HeatEquation.inl)
// on the device: assembly over the node pairs, boundary terms gathered at the nodes, and an FP64
// conjugate-gradient solve.
//
// One pass of HeatEqIncompNewton::solve without phase change (runOnlyOnce, :195-196):
//   (cv rho M + dt k L) T = cv rho M T_prev - dt (QN + SGamma_h + SGamma_r)     (:226-305, :307-375)
// with identity rows for free nodes and Dirichlet nodes, the Dirichlet columns moved to the
// right-hand side (:377-393).  M and L are MatrixBuilder::getM / getL (MatricesBuilder.inl:216-229,
// 308-321) with the factors cv rho and k (HeatEquation.inl:54-74).
//
// Layout: the scalar system reuses the node adjacency of the flow system (nbr_ptr / nbr, sorted,
// diagonal included) as its CSR pattern, values in node-pair order, so row n's entry for its
// neighbour of rank r sits at nbr_ptr[n] + r.  Each value is gathered by one thread from the
// elements the two nodes share, in ascending element order with M before L inside an element:
// the order in which Eigen's setFromTriplets sums the reference's triplets (:248-270, :295).
// The boundary facets a node belongs to are listed per node in ascending facet order (the
// reference's facet loop order), so the right-hand side needs no atomics either.
//
// The reference factorises the system with SparseLU; here it is SPD (M and L symmetric, the
// Dirichlet elimination symmetric, identity rows decoupled), so Jacobi-preconditioned CG in FP64
// solves it to the Krylov tolerances of the context (the system is mass dominated: a few dozen
// iterations).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "pfg_device.cuh"
#include "pfg_df.cuh"
#include "pfg_internal.cuh"

namespace pfg {

namespace {

constexpr uint8_t HT_T = PFG_HEAT_T, HT_Q = PFG_HEAT_Q, HT_QH = PFG_HEAT_QH, HT_QR = PFG_HEAT_QR;

struct HeatConst {
    DF m_df[4][4];    // cv rho MM_ij in double-float (the pair gather without phase change)
    DF ldt_df;        // dt * sum_g k w_g in double-float
    double MM[4][4];  // sum_g w_g N_i N_j
    double mfac;      // cv rho (the M factor, :54-59)
    double lsum;      // sum_g k w_g (the L factor summed over the Gauss points, :70-74)
    double refSize;   // reference element size
    double dt;
    // facet terms
    double h, tinf, eps_rad;
    double fw[3], fsf[3][3], fxi[3][2];  // facet Gauss rule: weights, shape functions, points
    double fref;                         // refSize(dim - 1)
    // phase change (HeatEquation.inl:36-45, 60-66): M factor (cv + dfl/dT(T_g) Lm) rho at the
    // element Gauss points, T_g from the node temperatures of the current Picard iterate
    int phase, ng;
    double gN[4][4], gw[4];              // element Gauss rule: N_i at point g, weights
    double cv, rho, tm, dtm, lm;
};

// d fl / dT of the liquid fraction (HeatEquation.inl:421-425): nonzero inside the melting
// range (Tm - DT/2, Tm + DT/2), where fl is the cubic smoothstep of (T - Tm) / DT
__device__ __forceinline__ double dfl_dt(const HeatConst& k, double T) {
    const double d3 = k.dtm * k.dtm * k.dtm;
    const double in = static_cast<double>(T > k.tm - k.dtm / 2) * static_cast<double>(T < k.tm + k.dtm / 2);
    return in * (-2 * 3 / d3 * T * T + 6 * 2 * k.tm / d3 * T + (3 / (2 * k.dtm) - 6 * k.tm * k.tm / d3));
}

// Element mass entry M_ij / |e|: cv rho MM_ij, or with phase change sum_g (f_g N_i N_j) w_g
// with f_g from the element's node temperatures ts (getM, MatricesBuilder.inl:216-229).
template <int DIM>
__device__ __forceinline__ double heat_m(const HeatConst& k, int i, int j, const double (&ts)[DIM + 1]) {
    if (!k.phase) return k.mfac * k.MM[i][j];
    double s = 0;
    for (int g = 0; g < k.ng; ++g) {
        double Tg = 0;
#pragma unroll
        for (int a = 0; a <= DIM; ++a) Tg += k.gN[g][a] * ts[a];
        const double f = (k.cv + dfl_dt(k, Tg) * k.lm) * k.rho;
        s += (f * (k.gN[g][i] * k.gN[g][j])) * k.gw[g];
    }
    return s;
}

HeatConst heat_const(pfg_ctx* c, double dt) {
    const GaussConst g = gauss_const(c->dim);
    HeatConst k{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) k.MM[i][j] = g.MM[i][j];
    k.mfac = c->prm.heat_cv * c->prm.rho;
    k.phase = c->prm.heat_phase_change != 0;
    k.ng = g.n;
    for (int q = 0; q < 4; ++q) {
        k.gw[q] = g.w[q];
        for (int i = 0; i < 4; ++i) k.gN[q][i] = g.N[q][i];
    }
    k.cv = c->prm.heat_cv;
    k.rho = c->prm.rho;
    k.tm = c->prm.heat_tm;
    k.dtm = c->prm.heat_dt_melt;
    k.lm = c->prm.heat_lm;
    k.lsum = 0;
    for (int q = 0; q < g.n; ++q) k.lsum += c->prm.heat_k * g.w[q];
    k.refSize = g.refSize;
    k.dt = dt;
    k.h = c->prm.heat_h;
    k.tinf = c->prm.heat_t_inf;
    k.eps_rad = c->prm.heat_eps_rad;
    // three-point facet rule (nGPLD = 3, HeatEquation.inl:13-22; Mesh.cpp:342-530)
    if (c->dim == 2) {
        const double x[3] = {-std::sqrt(3.0 / 5.0), 0.0, std::sqrt(3.0 / 5.0)};
        const double w[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};
        for (int q = 0; q < 3; ++q) {
            k.fxi[q][0] = x[q];
            k.fw[q] = w[q];
            k.fsf[q][0] = (1 - x[q]) / 2;
            k.fsf[q][1] = (1 + x[q]) / 2;
        }
        k.fref = 2.0;
    } else {
        const double p[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}, {2.0 / 3.0, 1.0 / 6.0}};
        for (int q = 0; q < 3; ++q) {
            k.fxi[q][0] = p[q][0];
            k.fxi[q][1] = p[q][1];
            k.fw[q] = 1.0 / 3.0;
            k.fsf[q][0] = 1 - p[q][0] - p[q][1];
            k.fsf[q][1] = p[q][0];
            k.fsf[q][2] = p[q][1];
        }
        k.fref = 0.5;
    }
    // double-float copies for the pair gather (after mfac, MM and lsum are set)
    auto split = [](double d) { const float h = (float)d; return DF{h, (float)(d - (double)h)}; };
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) k.m_df[i][j] = split(k.mfac * k.MM[i][j]);
    k.ldt_df = split(dt * k.lsum);
    return k;
}

// detJ and shape gradients of every element (slots 0 and 2.. of the flow element data; the
// flow assembly recomputes them before its own use).
template <int DIM>
__global__ void k_heat_geom(int E, int N, const int* __restrict__ conn, const double* __restrict__ pos,
                            double refSize, double* __restrict__ ed, DF* __restrict__ edf) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[DIM + 1];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    compute_geom<DIM>(pos, N, nd, g);
    double G[DIM][DIM + 1];
    grad_n<DIM>(g, G);
    ed[e] = g.detJ;
#pragma unroll
    for (int f = 0; f < DIM; ++f)
#pragma unroll
        for (int i = 0; i <= DIM; ++i) ed[(size_t)(2 + f * (DIM + 1) + i) * E + e] = G[f][i];
    // double-float copy for the pair gather: |e| = detJ refSize in slot 0, the gradients after
    edf[e] = df_from(g.detJ * refSize);
#pragma unroll
    for (int f = 0; f < DIM; ++f)
#pragma unroll
        for (int i = 0; i <= DIM; ++i) edf[(size_t)(2 + f * (DIM + 1) + i) * E + e] = df_from(G[f][i]);
}

// Value of the pair (n, m), one thread per pair: sum over the shared elements of
// Me(i,j) = (cv rho MM_ij) |e| and Le(i,j) = dt (|e| k_sum) gradN_i . gradN_j; identity rows for
// free and Dirichlet nodes (:287-293).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_heat_pairs(int P, int E, const int* __restrict__ pair_node,
                                                      const int* __restrict__ nbr, const int* __restrict__ ne_ptr,
                                                      const int* __restrict__ ne_elem,
                                                      const uint8_t* __restrict__ ne_loc, const int* __restrict__ conn,
                                                      const double* __restrict__ ed,
                                                      const uint8_t* __restrict__ flags,
                                                      const uint8_t* __restrict__ hflags, double* __restrict__ val,
                                                      const double* __restrict__ ts, const DF* __restrict__ edf,
                                                      HeatConst k) {
    constexpr int NPE = DIM + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P) return;
    const int n = pair_node[t], m = nbr[t];
    if ((hflags[n] & HT_T) || (flags[n] & F_FREE)) {
        val[t] = m == n ? 1.0 : 0.0;
        return;
    }
    if (!k.phase) {
        // double-float on the FP32 pipe (GB300's FP64 pipe runs at 1/64 of it; the FP64
        // gather below kept it 85% busy): |e| cv rho MM_ij + dt k_sum |e| gradN_i . gradN_j
        DF acc{0.0f, 0.0f};
        for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
            const int e = ne_elem[q];
            int j = -1;
#pragma unroll
            for (int jj = 0; jj < NPE; ++jj)
                if (__ldg(conn + (size_t)jj * E + e) == m) j = jj;
            if (j < 0) continue;
            const int i = ne_loc[q];
            const DF ae = edf[e];
            DF dot = df_mul(edf[(size_t)(2 + i) * E + e], edf[(size_t)(2 + j) * E + e]);
#pragma unroll
            for (int f = 1; f < DIM; ++f)
                dot = df_add(dot, df_mul(edf[(size_t)(2 + f * NPE + i) * E + e], edf[(size_t)(2 + f * NPE + j) * E + e]));
            acc = df_add(acc, df_mul(k.m_df[i][j], ae));
            acc = df_add(acc, df_mul(df_mul(k.ldt_df, ae), dot));
        }
        val[t] = df_to(acc);
        return;
    }
    double acc = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        int j = -1;
#pragma unroll
        for (int jj = 0; jj < NPE; ++jj)
            if (__ldg(conn + (size_t)jj * E + e) == m) j = jj;
        if (j < 0) continue;
        const int i = ne_loc[q];
        const double ae = ed[e] * k.refSize;
        double dot = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f)
            dot += ed[(size_t)(2 + f * NPE + i) * E + e] * ed[(size_t)(2 + f * NPE + j) * E + e];
        double te[NPE] = {};
        if (k.phase)
#pragma unroll
            for (int a = 0; a < NPE; ++a) te[a] = ts[__ldg(conn + (size_t)a * E + e)];
        acc += heat_m<DIM>(k, i, j, te) * ae;
        acc += k.dt * ((ae * k.lsum) * dot);
    }
    val[t] = acc;
}

// Facet f's geometry: measure factor detJ (Facet::computeDetJ, Facet.cpp:60-77) and, for the
// flux term, the unit normal turned away from the element's other node (Facet::computeNormal,
// :130-210).
template <int DIM>
__device__ __forceinline__ double facet_detj(const double* __restrict__ pos, int N, const int (&fn)[DIM]) {
    if constexpr (DIM == 2) {
        const double j0 = (pos[fn[1]] - pos[fn[0]]) / 2, j1 = (pos[(size_t)N + fn[1]] - pos[(size_t)N + fn[0]]) / 2;
        return sqrt(j0 * j0 + j1 * j1);
    } else {
        double u[3], w[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            u[d] = pos[(size_t)d * N + fn[1]] - pos[(size_t)d * N + fn[0]];
            w[d] = pos[(size_t)d * N + fn[2]] - pos[(size_t)d * N + fn[0]];
        }
        const double g0 = u[1] * w[2] - w[1] * u[2], g1 = u[2] * w[0] - w[2] * u[0], g2 = u[0] * w[1] - w[0] * u[1];
        return sqrt(g0 * g0 + g1 * g1 + g2 * g2);
    }
}

template <int DIM>
__device__ __forceinline__ void facet_normal(const double* __restrict__ pos, int N, const int (&fn)[DIM], int out,
                                             double (&nv)[DIM]) {
    if constexpr (DIM == 2) {
        nv[0] = pos[(size_t)N + fn[1]] - pos[(size_t)N + fn[0]];
        nv[1] = pos[fn[0]] - pos[fn[1]];
    } else {
        double u[3], w[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            u[d] = pos[(size_t)d * N + fn[1]] - pos[(size_t)d * N + fn[0]];
            w[d] = pos[(size_t)d * N + fn[2]] - pos[(size_t)d * N + fn[0]];
        }
        nv[0] = u[1] * w[2] - u[2] * w[1];
        nv[1] = u[2] * w[0] - u[0] * w[2];
        nv[2] = u[0] * w[1] - u[1] * w[0];
    }
    double dot = 0, nn = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        dot += nv[d] * (pos[(size_t)d * N + out] - pos[(size_t)d * N + fn[0]]);
        nn += nv[d] * nv[d];
    }
    const double s = dot > 0 ? -1.0 : 1.0;
    const double norm = sqrt(nn);
#pragma unroll
    for (int d = 0; d < DIM; ++d) nv[d] = (s * nv[d]) / norm;
}

struct HeatFacets {
    const int* ptr;         // N + 1 offsets into ent
    const int* ent;         // facet * 4 + facet-local node
    const uint8_t* fflags;  // HT_Q / HT_QH / HT_QR of each facet
    const int* fnodes;      // dim x F
    const int* felem;
    const double* q;        // (F, 3, dim) flux vectors at the Gauss points, or null
    int F;
};

// Subtracts node n's facet terms from its heat right-hand side b, one after the other: dt
// times the prescribed flux QN, the convection and the radiation SGamma of its listed facets in
// facet order (HeatEquation.inl:315-375 of either solver), at the facet-node temperatures ts.
template <int DIM>
__device__ __forceinline__ void heat_facet_terms(int n, int N, int E, const int* __restrict__ conn,
                                                 const double* __restrict__ pos, const double* __restrict__ ts,
                                                 const HeatFacets& hf, const HeatConst& k, double dt, double& b) {
    constexpr int NPE = DIM + 1;
    constexpr double sigma = 5.670374419e-8;  // Stefan-Boltzmann constant (:90)
    for (int q = hf.ptr[n]; q < hf.ptr[n + 1]; ++q) {
        const int ent = hf.ent[q];
        const int f = ent >> 2, kk = ent & 3;
        const uint8_t ff = hf.fflags[f];
        int fn[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) fn[d] = hf.fnodes[(size_t)d * hf.F + f];
        const double detJ = facet_detj<DIM>(pos, N, fn);
        if (ff & HT_Q) {  // getQN, MatricesBuilder.inl:246-272
            const int e = hf.felem[f];
            int out = -1;
#pragma unroll
            for (int a = 0; a < NPE; ++a) {
                const int v = conn[(size_t)a * E + e];
                bool on = false;
#pragma unroll
                for (int d = 0; d < DIM; ++d) on |= v == fn[d];
                if (!on) out = v;
            }
            double nv[DIM];
            facet_normal<DIM>(pos, N, fn, out, nv);
            double qn = 0;
#pragma unroll
            for (int g = 0; g < 3; ++g) {
                double qdn = 0;
#pragma unroll
                for (int d = 0; d < DIM; ++d) qdn += hf.q[((size_t)f * 3 + g) * DIM + d] * nv[d];
                qn += (qdn * k.fw[g]) * k.fsf[g][kk];
            }
            b -= dt * ((qn * k.fref) * detJ);
        }
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {  // getSGamma, MatricesBuilder.inl:357-370 (:76-94)
            if (!(ff & (pass == 0 ? HT_QH : HT_QR))) continue;
            double sg = 0;
#pragma unroll
            for (int g = 0; g < 3; ++g) {
                double T = 0;
#pragma unroll
                for (int d = 0; d < DIM; ++d) T += k.fsf[g][d] * ts[fn[d]];
                const double fac = pass == 0 ? k.h * (T - k.tinf)
                                             : sigma * k.eps_rad * (T * T * T * T - k.tinf * k.tinf * k.tinf * k.tinf);
                sg += (fac * k.fsf[g][kk]) * k.fw[g];
            }
            b -= dt * (sg * (detJ * k.fref));
        }
    }
}

// Right-hand side of node n: element gather of cv rho M T_prev (:240-283), the facet terms in
// facet order (:315-375), the node conditions (:377-393) and the Dirichlet column elimination
// of row n in ascending column order (the reference's node loop order), which zeroes the
// eliminated values.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_heat_rhs(int N, int E, const int* __restrict__ ne_ptr,
                                                    const int* __restrict__ ne_elem,
                                                    const uint8_t* __restrict__ ne_loc, const int* __restrict__ conn,
                                                    const double* __restrict__ ed, const double* __restrict__ pos,
                                                    const uint8_t* __restrict__ flags,
                                                    const uint8_t* __restrict__ hflags,
                                                    const double* __restrict__ t_prev, const double* __restrict__ ts,
                                                    const double* __restrict__ tbc,
                                                    const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                                                    double* __restrict__ val, HeatFacets hf, HeatConst k,
                                                    double* __restrict__ rhs) {
    constexpr int NPE = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double b = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const int e = ne_elem[q];
        const int i = ne_loc[q];
        int nd[NPE];
        load_nodes<DIM>(conn, E, e, nd);
        const double ae = ed[e] * k.refSize;
        double te[NPE] = {};
        if (k.phase)
#pragma unroll
            for (int a = 0; a < NPE; ++a) te[a] = ts[nd[a]];
        double s = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) s += (heat_m<DIM>(k, i, j, te) * ae) * t_prev[nd[j]];
        b += s;
    }
    heat_facet_terms<DIM>(n, N, E, conn, pos, ts, hf, k, k.dt, b);
    const uint8_t h = hflags[n];
    const bool fr = flags[n] & F_FREE;
    if (h & HT_T) {
        b = tbc[n];
    } else if (fr) {
        b = t_prev[n];
    } else {
        for (int t = nbr_ptr[n]; t < nbr_ptr[n + 1]; ++t) {
            const int m = nbr[t];
            if (m != n && (hflags[m] & HT_T)) {
                b -= val[t] * tbc[m];
                val[t] = 0.0;
            }
        }
    }
    rhs[n] = b;
}

// ---- Jacobi-preconditioned conjugate gradients over the pair-ordered CSR -----------------

// ---- Jacobi-preconditioned conjugate gradients, Chronopoulos-Gear form ------------------
//
// The classic recurrences rearranged so that one iteration needs one SpMV kernel with one
// fused reduction (gamma = r.z, delta = w.z with w = A z, and ||r||^2) and one pointwise kernel
// (Chronopoulos and Gear, J. Comput. Appl. Math. 25, 1989): s = A p is carried by recurrence.
//   pointwise: p = z + beta p; s = w + beta s; x += alpha p; r -= alpha s; z = r / diag
//   spmv:      w = A z; gamma, delta, rr; beta = gamma / gamma_old;
//              alpha = gamma / (delta - beta gamma / alpha_old)
// Mathematically the same iterates as classic CG; the rounding differs.

enum : int { S_GAMMA = 0, S_ALPHA, S_BETA, S_RR, S_TOL2, S_DONE, S_ITERS, S_BB, S_NUM, S_DEN, S_FIRST, S_COUNT };
enum : int { V_R = 0, V_Z, V_P, V_S, V_W, V_DIAG, V_COUNT };  // V_DIAG holds the inverse diagonal
static_assert(V_COUNT == CG_VECTORS, "cg_solve's work vectors");

struct CgPtrs {
    double* partials;  // 3 * max_grid
    double* sc;        // S_COUNT
    unsigned* ticket;
};

CgPtrs cg_ptrs(pfg_ctx* c) {
    double* red = ptr<double>(c->heat_red);
    CgPtrs k;
    k.partials = red;
    k.sc = red + 3 * (size_t)c->max_grid;
    k.ticket = reinterpret_cast<unsigned*>(k.sc + 32);
    return k;
}

// Three-value version of grid_sum2.
template <int NT>
__device__ __forceinline__ bool grid_sum3(double a, double b, double c, double* partials, unsigned* ticket,
                                          double* sh, double& ra, double& rb, double& rc) {
    a = block_sum<NT>(a, sh);
    b = block_sum<NT>(b, sh);
    c = block_sum<NT>(c, sh);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = a;
        partials[gridDim.x + blockIdx.x] = b;
        partials[2 * gridDim.x + blockIdx.x] = c;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double sa = 0, sb = 0, sc = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += NT) {
        sa += ((volatile double*)partials)[i];
        sb += ((volatile double*)partials)[gridDim.x + i];
        sc += ((volatile double*)partials)[2 * gridDim.x + i];
    }
    ra = block_sum<NT>(sa, sh);
    rb = block_sum<NT>(sb, sh);
    rc = block_sum<NT>(sc, sh);
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

template <int NT>
__device__ __forceinline__ bool grid_sum2(double a, double b, double* partials, unsigned* ticket, double* sh,
                                          double& ra, double& rb) {
    a = block_sum<NT>(a, sh);
    b = block_sum<NT>(b, sh);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = a;
        partials[gridDim.x + blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double sa = 0, sb = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += NT) {
        sa += ((volatile double*)partials)[i];
        sb += ((volatile double*)partials)[gridDim.x + i];
    }
    ra = block_sum<NT>(sa, sh);
    rb = block_sum<NT>(sb, sh);
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// r = b - A x, z = r / diag, p = s = 0; tolerance max(rtol ||b||, atol), capped at
// max(cap, 2e-16 ||b||) (the heat Picard loop with an absolute "Ax_f" residual needs the linear
// solve below its minRes, down to the rounding level an LU solve reaches).
__global__ void __launch_bounds__(BLOCK) k_cg_init(int N, const int* __restrict__ rp, const int* __restrict__ col,
                                                   const double* __restrict__ val, const double* __restrict__ b,
                                                   const double* __restrict__ x, double* __restrict__ V, size_t ld,
                                                   CgPtrs k, double rtol, double atol, double cap) {
    __shared__ double sh[32];
    double bb = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        double ax = 0, d = 1.0;
        for (int t = rp[n]; t < rp[n + 1]; ++t) {
            const int m = col[t];
            ax += val[t] * x[m];
            if (m == n) d = val[t];
        }
        const double r = b[n] - ax;
        const double dinv = 1.0 / d;  // one FP64 division per row per solve, multiplies after
        V[V_R * ld + n] = r;
        V[V_Z * ld + n] = r * dinv;
        V[V_P * ld + n] = 0.0;
        V[V_S * ld + n] = 0.0;
        V[V_DIAG * ld + n] = dinv;
        bb += b[n] * b[n];
    }
    double s1, unused;
    if (grid_sum2<BLOCK>(bb, 0.0, k.partials, k.ticket, sh, s1, unused) && threadIdx.x == 0) {
        k.sc[S_BB] = s1;
        const double tol = fmin(fmax(rtol * sqrt(s1), atol), fmax(cap, 2e-16 * sqrt(s1)));
        k.sc[S_TOL2] = tol * tol;
        k.sc[S_ITERS] = 0;
        k.sc[S_DONE] = 0;
        k.sc[S_GAMMA] = 0;
        k.sc[S_ALPHA] = 1;
        k.sc[S_BETA] = 0;
        k.sc[S_FIRST] = 1;
    }
}

// w = A z with gamma = r.z, delta = w.z and ||r||^2 in one reduction; the last block updates
// the scalars and the convergence state (1 converged, 2 breakdown or NaN, 3 iteration cap).
// G lanes per row, the group's sum a shuffle reduction in a fixed order.  Measured on the C3
// heat system (ncu, one cold launch of the earlier p.q SpMV): one thread per row 38.5 us,
// 8 lanes per row 49.3 us (issue bound on the per-row overhead of ~13-entry rows): G = 1.
template <int G>
__global__ void __launch_bounds__(BLOCK) k_cg_spmv(int N, const int* __restrict__ rp, const int* __restrict__ col,
                                                   const double* __restrict__ val, double* __restrict__ V, size_t ld,
                                                   CgPtrs k, int max_it) {
    __shared__ double sh[32];
    if (k.sc[S_DONE] != 0.0) return;
    const double* z = V + V_Z * ld;
    const double* r = V + V_R * ld;
    const int lane = threadIdx.x % G;
    constexpr int GPW = 32 / G;  // rows per warp and trip
    const int wglob = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int nwarps = gridDim.x * blockDim.x / 32;
    double ga = 0, de = 0, rr = 0;
    // all lanes of a warp share r0, so they run the same trips (the shuffles need the warp)
    for (int r0 = wglob * GPW; r0 < N; r0 += nwarps * GPW) {
        const int n = r0 + (threadIdx.x & 31) / G;
        const bool act = n < N;
        const int b = act ? rp[n] : 0, e = act ? rp[n + 1] : 0;
        double w = 0;
        for (int t = b + lane; t < e; t += G) w += val[t] * z[col[t]];
        if constexpr (G > 1) {
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o, G);
        }
        if (act && lane == 0) {
            V[V_W * ld + n] = w;
            const double zn = z[n], rn = r[n];
            ga += rn * zn;
            de += w * zn;
            rr += rn * rn;
        }
    }
    double g, s_de, s_rr;
    if (!grid_sum3<BLOCK>(ga, de, rr, k.partials, k.ticket, sh, g, s_de, s_rr)) return;
    if (threadIdx.x == 0) {
        const bool first = k.sc[S_FIRST] != 0.0;
        const double it = k.sc[S_ITERS] + (first ? 0.0 : 1.0);
        k.sc[S_ITERS] = it;
        k.sc[S_FIRST] = 0;
        k.sc[S_RR] = s_rr;
        const double gold = k.sc[S_GAMMA];
        const double beta = gold != 0.0 ? g / gold : 0.0;
        const double den = s_de - beta * g / k.sc[S_ALPHA];
        k.sc[S_BETA] = beta;
        k.sc[S_ALPHA] = den != 0.0 ? g / den : 0.0;
        k.sc[S_GAMMA] = g;
        if (s_rr <= k.sc[S_TOL2]) k.sc[S_DONE] = 1;
        else if (!(s_rr == s_rr) || !(den > 0.0)) k.sc[S_DONE] = 2;  // NaN or loss of definiteness
        else if (it >= max_it) k.sc[S_DONE] = 3;
    }
}

// p = z + beta p; s = w + beta s; x += alpha p; r -= alpha s; z = r / diag
__global__ void __launch_bounds__(BLOCK) k_cg_update(int N, double* __restrict__ x, double* __restrict__ V, size_t ld,
                                                     CgPtrs k) {
    if (k.sc[S_DONE] != 0.0) return;
    const double alpha = k.sc[S_ALPHA], beta = k.sc[S_BETA];
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const double p = V[V_Z * ld + n] + beta * V[V_P * ld + n];
        const double sv = V[V_W * ld + n] + beta * V[V_S * ld + n];
        V[V_P * ld + n] = p;
        V[V_S * ld + n] = sv;
        x[n] += alpha * p;
        const double r = V[V_R * ld + n] - alpha * sv;
        V[V_R * ld + n] = r;
        V[V_Z * ld + n] = r * V[V_DIAG * ld + n];  // inverse diagonal
    }
}

// ---- mixed precision (contexts in PFG_PREC_MIXED): Jacobi CG corrections in FP32 under an FP64
// refinement of r = b - A x; the same recurrences as above on FP32 vectors, FP64 reductions --------
enum : int { V32_R = 0, V32_Z, V32_P, V32_S, V32_W, V32_DIAG, V32_D, V32_COUNT };

// the FP32 copy of the matrix values
__global__ void k_heat_val32(int P, const double* __restrict__ val, float* __restrict__ val32) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P) val32[p] = (float)val[p];
}

// r = b - A x in FP64, its FP32 copy (the correction solve's right-hand side), ||r||^2 into
// sc[S_NUM] and ||b||^2 into sc[S_DEN]
__global__ void __launch_bounds__(BLOCK) k_heat_r64(int N, const int* __restrict__ rp, const int* __restrict__ col,
                                                    const double* __restrict__ val, const double* __restrict__ b,
                                                    const double* __restrict__ x, float* __restrict__ rhs32,
                                                    CgPtrs k) {
    __shared__ double sh[32];
    double rr = 0, bb = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        double ax = 0;
        for (int t = rp[n]; t < rp[n + 1]; ++t) ax += val[t] * x[col[t]];
        const double r = b[n] - ax;
        rhs32[n] = (float)r;
        rr += r * r;
        bb += b[n] * b[n];
    }
    double s1, s2;
    if (grid_sum2<BLOCK>(rr, bb, k.partials, k.ticket, sh, s1, s2) && threadIdx.x == 0) {
        k.sc[S_NUM] = s1;
        k.sc[S_DEN] = s2;
    }
}

// d = 0, r = rhs, z = r / diag, p = s = 0 (diag from the FP32 matrix); tolerance eta ||rhs||
__global__ void __launch_bounds__(BLOCK) k_cg32_init(int N, const int* __restrict__ rp, const int* __restrict__ col,
                                                     const float* __restrict__ val, const float* __restrict__ rhs,
                                                     float* __restrict__ V, size_t ld, CgPtrs k, double eta) {
    __shared__ double sh[32];
    double bb = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        float d = 1.0f;
        for (int t = rp[n]; t < rp[n + 1]; ++t)
            if (col[t] == n) d = val[t];
        const float r = rhs[n];
        const float dinv = 1.0f / d;
        V[V32_R * ld + n] = r;
        V[V32_Z * ld + n] = r * dinv;
        V[V32_P * ld + n] = 0.0f;
        V[V32_S * ld + n] = 0.0f;
        V[V32_DIAG * ld + n] = dinv;
        V[V32_D * ld + n] = 0.0f;
        bb += (double)r * (double)r;
    }
    double s1, unused;
    if (grid_sum2<BLOCK>(bb, 0.0, k.partials, k.ticket, sh, s1, unused) && threadIdx.x == 0) {
        k.sc[S_BB] = s1;
        k.sc[S_TOL2] = eta * eta * s1;
        k.sc[S_ITERS] = 0;
        k.sc[S_DONE] = 0;
        k.sc[S_GAMMA] = 0;
        k.sc[S_ALPHA] = 1;
        k.sc[S_BETA] = 0;
        k.sc[S_FIRST] = 1;
    }
}

// w = A z with gamma, delta and ||r||^2 (k_cg_spmv on FP32 arrays; each thread's sums in FP32,
// the grid reduction and the scalars in FP64)
__global__ void __launch_bounds__(BLOCK) k_cg32_spmv(int N, const int* __restrict__ rp, const int* __restrict__ col,
                                                     const float* __restrict__ val, float* __restrict__ V, size_t ld,
                                                     CgPtrs k, int max_it) {
    __shared__ double sh[32];
    if (k.sc[S_DONE] != 0.0) return;
    const float* z = V + V32_Z * ld;
    const float* r = V + V32_R * ld;
    float ga = 0, de = 0, rr = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        float w = 0;
        for (int t = rp[n]; t < rp[n + 1]; ++t) w += val[t] * z[col[t]];
        V[V32_W * ld + n] = w;
        const float zn = z[n], rn = r[n];
        ga += rn * zn;
        de += w * zn;
        rr += rn * rn;
    }
    double g, s_de, s_rr;
    if (!grid_sum3<BLOCK>(ga, de, rr, k.partials, k.ticket, sh, g, s_de, s_rr)) return;
    if (threadIdx.x == 0) {
        const bool first = k.sc[S_FIRST] != 0.0;
        const double it = k.sc[S_ITERS] + (first ? 0.0 : 1.0);
        k.sc[S_ITERS] = it;
        k.sc[S_FIRST] = 0;
        k.sc[S_RR] = s_rr;
        const double gold = k.sc[S_GAMMA];
        const double beta = gold != 0.0 ? g / gold : 0.0;
        const double den = s_de - beta * g / k.sc[S_ALPHA];
        k.sc[S_BETA] = beta;
        k.sc[S_ALPHA] = den != 0.0 ? g / den : 0.0;
        k.sc[S_GAMMA] = g;
        if (s_rr <= k.sc[S_TOL2]) k.sc[S_DONE] = 1;
        else if (!(s_rr == s_rr) || !(den > 0.0)) k.sc[S_DONE] = 2;
        else if (it >= max_it) k.sc[S_DONE] = 3;
    }
}

// p = z + beta p; s = w + beta s; d += alpha p; r -= alpha s; z = r / diag
__global__ void __launch_bounds__(BLOCK) k_cg32_update(int N, float* __restrict__ V, size_t ld, CgPtrs k) {
    if (k.sc[S_DONE] != 0.0) return;
    const float alpha = (float)k.sc[S_ALPHA], beta = (float)k.sc[S_BETA];
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const float p = V[V32_Z * ld + n] + beta * V[V32_P * ld + n];
        const float sv = V[V32_W * ld + n] + beta * V[V32_S * ld + n];
        V[V32_P * ld + n] = p;
        V[V32_S * ld + n] = sv;
        V[V32_D * ld + n] += alpha * p;
        const float r = V[V32_R * ld + n] - alpha * sv;
        V[V32_R * ld + n] = r;
        V[V32_Z * ld + n] = r * V[V32_DIAG * ld + n];
    }
}

// x += d (the FP32 correction)
__global__ void k_heat_add_d(int N, const float* __restrict__ d, double* __restrict__ x) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < N) x[n] += (double)d[n];
}

// Squared relative change of the non-free nodes (residual "T", HeatEquation.inl:153-180):
// sum (x - xp)^2 and sum xp^2 into sc[S_NUM], sc[S_DEN]; or, with b, ||b - A x||^2 into
// sc[S_NUM] (residual "Ax_f", :182-185).
__global__ void __launch_bounds__(BLOCK) k_heat_res(int N, const double* __restrict__ x, const double* __restrict__ xp,
                                                    const uint8_t* __restrict__ flags, const int* __restrict__ rp,
                                                    const int* __restrict__ col, const double* __restrict__ val,
                                                    const double* __restrict__ b, CgPtrs k) {
    __shared__ double sh[32];
    double num = 0, den = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        if (b) {
            double ax = 0;
            for (int t = rp[n]; t < rp[n + 1]; ++t) ax += val[t] * x[col[t]];
            const double r = b[n] - ax;
            num += r * r;
        } else if (!(flags[n] & F_FREE)) {
            const double d = x[n] - xp[n];
            num += d * d;
            den += xp[n] * xp[n];
        }
    }
    double s1, s2;
    if (grid_sum2<BLOCK>(num, den, k.partials, k.ticket, sh, s1, s2) && threadIdx.x == 0) {
        k.sc[S_NUM] = s1;
        k.sc[S_DEN] = s2;
    }
}

HeatFacets heat_facets(pfg_ctx* c);

template <int DIM>
void heat_assemble(pfg_ctx* c, const HeatConst& k, const double* tprev, const double* ts) {
    const int N = c->N, E = c->E;
    prof_begin(c, PH_HEAT_ASSEMBLY);
    if (E > 0)
        k_heat_geom<DIM><<<div_up(E, BLOCK), BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos),
                                                                    k.refSize, ptr<double>(c->edata),
                                                                    ptr<DF>(c->edata_df));
    if (c->P > 0)
        k_heat_pairs<DIM><<<div_up(c->P, BLOCK), BLOCK, 0, c->stream>>>(
            c->P, E, ptr<int>(c->pair_node), ptr<int>(c->nbr), ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem),
            ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn), ptr<double>(c->edata), ptr<uint8_t>(c->flags),
            ptr<uint8_t>(c->heat_flags), ptr<double>(c->heat_val), ts, ptr<DF>(c->edata_df), k);
    const HeatFacets hf = heat_facets(c);
    k_heat_rhs<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(
        N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn),
        ptr<double>(c->edata), ptr<double>(c->pos), ptr<uint8_t>(c->flags), ptr<uint8_t>(c->heat_flags), tprev, ts,
        ptr<double>(c->heat_tbc), ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<double>(c->heat_val), hf, k,
        ptr<double>(c->heat_rhs));
    prof_end(c, PH_HEAT_ASSEMBLY);
}

// CG solve of the assembled system from x0 = T_prev (solveWithGuess, :126) into x.  Returns
// the convergence flag; iterations and the last recursive residual accumulate in st.
int heat_cg(pfg_ctx* c, const double* tprev, double* x, pfg_step_status* st, bool* ok, double cap) {
    const int N = c->N;
    double* V = ptr<double>(c->heat_cg);
    const size_t ld = (size_t)std::max(N, 1);
    if (tprev != x)
        PFG_CUDA(c, cudaMemcpyAsync(x, tprev, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    const CgPtrs kp = cg_ptrs(c);
    const int grid = std::max(1, std::min(c->max_grid, div_up(N, BLOCK)));
    const int* rp = ptr<int>(c->nbr_ptr);
    const int* col = ptr<int>(c->nbr);
    const double* val = ptr<double>(c->heat_val);
    k_cg_init<<<grid, BLOCK, 0, c->stream>>>(N, rp, col, val, ptr<double>(c->heat_rhs), x, V, ld, kp,
                                             c->prm.krylov_rel_tol, c->prm.krylov_abs_tol, cap);
    const int max_it = std::max(1, c->prm.krylov_max_iter);
    // w0 = A z0 with the first scalars (no iteration counted)
    prof_begin(c, PH_HEAT_SPMV);
    k_cg_spmv<1><<<grid, BLOCK, 0, c->stream>>>(N, rp, col, val, V, ld, kp, max_it);
    prof_end(c, PH_HEAT_SPMV);
    PFG_CHECK_LAUNCH(c);
    double* h = c->h_scalars;
    int done_it = 0;
    while (done_it < max_it) {
        const int n = std::min(8, max_it - done_it);
        for (int it = 0; it < n; ++it) {
            k_cg_update<<<grid, BLOCK, 0, c->stream>>>(N, x, V, ld, kp);
            prof_begin(c, PH_HEAT_SPMV);
            k_cg_spmv<1><<<grid, BLOCK, 0, c->stream>>>(N, rp, col, val, V, ld, kp, max_it);
            prof_end(c, PH_HEAT_SPMV);
        }
        PFG_CHECK_LAUNCH(c);
        done_it += n;
        PFG_CUDA(c, cudaMemcpyAsync(h, kp.sc, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (h[S_DONE] != 0.0) break;
    }
    *ok = h[S_DONE] == 1.0;
    st->krylov_iterations += (int)h[S_ITERS];
    return PFG_OK;
}

// The same solve in mixed precision: from x0 = T_prev, FP64 residuals r = b - A x and FP32 Jacobi
// CG corrections A d = r (to eta = 1e-4 of ||r||, or, for a sweep that needs less, 0.2 of the
// remaining reduction, at most 0.01), x += d, until ||r|| meets the FP64 solve's tolerance.  A
// sweep that does not shrink ||r|| tenfold, a breakdown, or 30 sweeps hand the rest to the FP64
// CG from the current x.
int heat_cg_mixed(pfg_ctx* c, const double* tprev, double* x, pfg_step_status* st, bool* ok, double cap) {
    const int N = c->N, P = c->P;
    const size_t ld = (size_t)std::max(N, 1);
    float* V = ptr<float>(c->heat_cg32);
    float* val32 = V + V32_COUNT * ld;
    float* rhs32 = ptr<float>(c->heat_rhs32);
    const int* rp = ptr<int>(c->nbr_ptr);
    const int* col = ptr<int>(c->nbr);
    const double* val = ptr<double>(c->heat_val);
    const CgPtrs kp = cg_ptrs(c);
    const int grid = std::max(1, std::min(c->max_grid, div_up(N, BLOCK)));
    PFG_CUDA(c, cudaMemcpyAsync(x, tprev, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    if (P > 0) k_heat_val32<<<div_up(P, BLOCK), BLOCK, 0, c->stream>>>(P, val, val32);
    const int max_it = std::max(1, c->prm.krylov_max_iter);
    double* h = c->h_scalars;
    double rr_prev = INFINITY;
    for (int sweep = 0; sweep < 30; ++sweep) {
        k_heat_r64<<<grid, BLOCK, 0, c->stream>>>(N, rp, col, val, ptr<double>(c->heat_rhs), x, rhs32, kp);
        PFG_CHECK_LAUNCH(c);
        PFG_CUDA(c, cudaMemcpyAsync(h, kp.sc, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        const double rr = h[S_NUM], bnorm = std::sqrt(h[S_DEN]);
        const double tol = std::fmin(std::fmax(c->prm.krylov_rel_tol * bnorm, c->prm.krylov_abs_tol),
                                     std::fmax(cap, 2e-16 * bnorm));
        if (std::isnan(rr)) {
            *ok = false;
            return PFG_OK;
        }
        if (std::sqrt(rr) <= tol) {
            *ok = true;
            return PFG_OK;
        }
        if (!(rr <= 0.01 * rr_prev)) break;  // FP32 corrections stopped contracting
        rr_prev = rr;
        const double eta = std::fmax(1e-4, std::fmin(0.01, 0.2 * tol / std::sqrt(rr)));
        k_cg32_init<<<grid, BLOCK, 0, c->stream>>>(N, rp, col, val32, rhs32, V, ld, kp, eta);
        prof_begin(c, PH_HEAT_SPMV);
        k_cg32_spmv<<<grid, BLOCK, 0, c->stream>>>(N, rp, col, val32, V, ld, kp, max_it);
        prof_end(c, PH_HEAT_SPMV);
        PFG_CHECK_LAUNCH(c);
        int done_it = 0;
        while (done_it < max_it) {
            const int n = std::min(8, max_it - done_it);
            for (int it = 0; it < n; ++it) {
                k_cg32_update<<<grid, BLOCK, 0, c->stream>>>(N, V, ld, kp);
                prof_begin(c, PH_HEAT_SPMV);
                k_cg32_spmv<<<grid, BLOCK, 0, c->stream>>>(N, rp, col, val32, V, ld, kp, max_it);
                prof_end(c, PH_HEAT_SPMV);
            }
            PFG_CHECK_LAUNCH(c);
            done_it += n;
            PFG_CUDA(c, cudaMemcpyAsync(h, kp.sc, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->stream));
            PFG_CUDA(c, cudaStreamSynchronize(c->stream));
            if (h[S_DONE] != 0.0) break;
        }
        st->krylov_iterations += (int)h[S_ITERS];
        if (h[S_DONE] == 2.0) break;  // breakdown
        k_heat_add_d<<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(N, V + V32_D * ld, x);
        PFG_CHECK_LAUNCH(c);
    }
    return heat_cg(c, x, x, st, ok, cap);
}

// HeatEqIncompNewton::solve through PicardAlgo::solve (PicardAlgo.cpp:31-95): without phase
// change one pass (runOnlyOnce); with it, the system is rebuilt from each iterate's temperatures
// (:131-138) until the residual is at most heat_min_res, failing (temperatures restored) after
// heat_max_iter + 1 passes or on a NaN residual.
template <int DIM>
int heat_dim(pfg_ctx* c, double dt, pfg_step_status* st) {
    const int N = c->N;
    const HeatConst k = heat_const(c, dt);
    double* T = ptr<double>(c->heat_t);  // the node states: the Picard iterate
    double* V = ptr<double>(c->heat_cg);
    const size_t ld = (size_t)std::max(N, 1);
    double* x = V + V_COUNT * ld;
    double* tprev = x + ld;
    double* xprev = tprev + ld;
    PFG_CUDA(c, cudaMemcpyAsync(tprev, T, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(xprev, T, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    heat_assemble<DIM>(c, k, tprev, T);
    PFG_CHECK_LAUNCH(c);
    const bool axf = c->prm.heat_residual == PFG_RES_AX_F;
    const int max_iter = c->prm.heat_max_iter;
    const CgPtrs kp = cg_ptrs(c);
    const int grid = std::max(1, std::min(c->max_grid, div_up(N, BLOCK)));
    double* h = c->h_scalars;
    double res = INFINITY;
    int it = 0;
    bool ok = true;
    st->dt = dt;
    while (res > c->prm.heat_min_res) {
        if (it > max_iter) {
            ok = false;
            break;
        }
        bool solved = false;
        const double cap = axf ? 0.1 * c->prm.heat_min_res : INFINITY;
        int rc = c->prm.precision == PFG_PREC_MIXED ? heat_cg_mixed(c, tprev, x, st, &solved, cap)
                                                    : heat_cg(c, tprev, x, st, &solved, cap);
        if (rc) return rc;
        if (!solved) {
            ok = false;
            break;
        }
        PFG_CUDA(c, cudaMemcpyAsync(T, x, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
        if (k.phase) {
            heat_assemble<DIM>(c, k, tprev, T);
            PFG_CHECK_LAUNCH(c);
        }
        k_heat_res<<<grid, BLOCK, 0, c->stream>>>(N, x, xprev, ptr<uint8_t>(c->flags), ptr<int>(c->nbr_ptr),
                                                   ptr<int>(c->nbr), ptr<double>(c->heat_val),
                                                   axf ? ptr<double>(c->heat_rhs) : nullptr, kp);
        PFG_CHECK_LAUNCH(c);
        PFG_CUDA(c, cudaMemcpyAsync(xprev, x, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
        PFG_CUDA(c, cudaMemcpyAsync(h, kp.sc, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        res = axf ? std::sqrt(h[S_NUM]) : (h[S_DEN] == 0.0 ? DBL_MAX : std::sqrt(h[S_NUM] / h[S_DEN]));
        ++it;
        if (std::isnan(res)) {
            ok = false;
            break;
        }
        if (!k.phase) break;
    }
    st->converged = ok ? 1 : 0;
    st->picard_iterations = it;
    st->residual = res;
    if (!ok) PFG_CUDA(c, cudaMemcpyAsync(T, tprev, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PFG_OK;
}

// ---- explicit heat step of problem BoussinesqWC (HeatEqWCompNewton) ----------------------
//
// HeatEqWCompNewton::solve (WCompNewton/HeatEquation.inl:137-158) inside the WC step, after the
// half-step prediction moved the nodes.  Element: for each element node i the lumped mass
//   ML_i = |e| sum_g w_g N_i(g) f_g,  f_g = cv rho_g, or (cv + dfl/dT(T_g) Lm) rho_g with phase
// change (getM with the factor of :51-66, then lump: the row sum of the consistent block), and
//   FTot_i = -dt (Le T)_i + ML_i T_i,  Le = |e| k_sum gradN^T gradN  (:285-299).
// Node: sums in ascending element order, the facet terms in facet order, the node conditions
// (:240-260), T = F / M into a second array (the facet terms read the neighbours' old
// temperatures), copied back.  dt is read from the step's device dt slot (slot 0).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_wch_elem(int E, int N, const int* __restrict__ conn,
                                                    const double* __restrict__ pos, const double* __restrict__ rho,
                                                    const double* __restrict__ T, const double* __restrict__ tdt,
                                                    HeatConst k, double* __restrict__ rec) {
    constexpr int NPE = DIM + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double dt = tdt[0];
    int nd[NPE];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    compute_geom<DIM>(pos, N, nd, g);
    double G[DIM][NPE];
    grad_n<DIM>(g, G);
    const double ae = g.detJ * k.refSize;
    double te[NPE], re[NPE], gt[DIM];
#pragma unroll
    for (int a = 0; a < NPE; ++a) {
        te[a] = T[nd[a]];
        re[a] = rho[nd[a]];
    }
#pragma unroll
    for (int f = 0; f < DIM; ++f) {
        double t = 0;
#pragma unroll
        for (int j = 0; j < NPE; ++j) t += G[f][j] * te[j];
        gt[f] = t;
    }
    double ml[NPE] = {};
    for (int q = 0; q < k.ng; ++q) {
        double Tg = 0, rg = 0;
#pragma unroll
        for (int a = 0; a < NPE; ++a) {
            Tg += k.gN[q][a] * te[a];
            rg += k.gN[q][a] * re[a];
        }
        const double f = k.phase ? (k.cv + dfl_dt(k, Tg) * k.lm) * rg : k.cv * rg;
#pragma unroll
        for (int i = 0; i < NPE; ++i) ml[i] += (f * k.gN[q][i]) * k.gw[q];
    }
    double* out = rec + (size_t)e * 2 * NPE;
#pragma unroll
    for (int i = 0; i < NPE; ++i) {
        double lt = 0;
#pragma unroll
        for (int f = 0; f < DIM; ++f) lt += G[f][i] * gt[f];
        const double m = ml[i] * ae;
        out[i] = m;
        out[NPE + i] = -dt * ((k.lsum * ae) * lt) + m * te[i];
    }
}

template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_wch_node(int N, int E, const int* __restrict__ ne_ptr,
                                                    const int* __restrict__ ne_elem,
                                                    const uint8_t* __restrict__ ne_loc, const int* __restrict__ conn,
                                                    const double* __restrict__ pos, const uint8_t* __restrict__ flags,
                                                    const uint8_t* __restrict__ hflags, const double* __restrict__ T,
                                                    const double* __restrict__ tbc, const double* __restrict__ rec,
                                                    HeatFacets hf, HeatConst k, const double* __restrict__ tdt,
                                                    double* __restrict__ tnew) {
    constexpr int NPE = DIM + 1;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const double dt = tdt[0];
    double m = 0, F = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; ++q) {
        const double* r = rec + (size_t)ne_elem[q] * 2 * NPE;
        const int i = ne_loc[q];
        m += r[i];
        F += r[NPE + i];
    }
    heat_facet_terms<DIM>(n, N, E, conn, pos, T, hf, k, dt, F);
    const uint8_t h = hflags[n];
    if ((flags[n] & F_FREE) && !(h & HT_T)) tnew[n] = T[n];
    else if (h & HT_T) tnew[n] = tbc[n];
    else tnew[n] = (1 / m) * F;
}

HeatFacets heat_facets(pfg_ctx* c) {
    HeatFacets hf;
    hf.ptr = ptr<int>(c->hf_ptr);
    hf.ent = ptr<int>(c->hf_ent);
    hf.fflags = ptr<uint8_t>(c->hf_fflags);
    hf.fnodes = ptr<int>(c->fc_nodes);
    hf.felem = ptr<int>(c->fc_elem);
    hf.q = c->has_heat_q ? ptr<double>(c->heat_q) : nullptr;
    hf.F = c->F;
    return hf;
}

template <int DIM>
int wc_heat_dim(pfg_ctx* c, const double* tdt) {
    const int N = c->N, E = c->E;
    const HeatConst k = heat_const(c, 0.0);
    double* rec = ptr<double>(c->wch_rec);
    double* T = ptr<double>(c->heat_t);
    double* tnew = ptr<double>(c->heat_rhs);
    prof_begin(c, PH_HEAT_ASSEMBLY);
    if (E > 0)
        k_wch_elem<DIM><<<div_up(E, BLOCK), BLOCK, 0, c->stream>>>(
            E, N, ptr<int>(c->conn), ptr<double>(c->pos), ptr<double>(c->ws) + (size_t)(DIM + 1) * N, T, tdt, k, rec);
    k_wch_node<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(
        N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn),
        ptr<double>(c->pos), ptr<uint8_t>(c->flags), ptr<uint8_t>(c->heat_flags), T, ptr<double>(c->heat_tbc), rec,
        heat_facets(c), k, tdt, tnew);
    PFG_CUDA(c, cudaMemcpyAsync(T, tnew, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
    prof_end(c, PH_HEAT_ASSEMBLY);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

}  // namespace

int heat_alloc(pfg_ctx* c) {
    const size_t N = std::max(c->N, 1), P = std::max(c->P, 1);
    int rc;
    if ((rc = ensure(c, c->heat_t, sizeof(double) * N)) || (rc = ensure(c, c->heat_flags, N)) ||
        (rc = ensure(c, c->heat_tbc, sizeof(double) * N)) || (rc = ensure(c, c->heat_val, sizeof(double) * P)) ||
        (rc = ensure(c, c->heat_rhs, sizeof(double) * N)) ||
        (rc = ensure(c, c->heat_cg, sizeof(double) * (V_COUNT + 3) * N)) ||
        (rc = ensure(c, c->heat_red, sizeof(double) * (3 * (size_t)std::max(c->max_grid, 1) + 64))) ||
        (rc = ensure(c, c->hf_ptr, sizeof(int) * (N + 1))) ||
        (rc = ensure(c, c->edata_df, sizeof(DF) * (3 + c->dim * (c->dim + 1)) * (size_t)std::max(c->E, 1))))
        return rc;
    if (c->prm.precision == PFG_PREC_MIXED &&
        ((rc = ensure(c, c->heat_cg32, sizeof(float) * (V32_COUNT * N + P))) ||
         (rc = ensure(c, c->heat_rhs32, sizeof(float) * N))))
        return rc;
    PFG_CUDA(c, cudaMemsetAsync(c->heat_t.p, 0, sizeof(double) * N, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(c->heat_flags.p, 0, N, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(c->heat_tbc.p, 0, sizeof(double) * N, c->stream));
    PFG_CUDA(c, cudaMemsetAsync(c->hf_ptr.p, 0, sizeof(int) * (N + 1), c->stream));
    PFG_CUDA(c, cudaMemsetAsync(c->heat_red.p, 0, sizeof(double) * (3 * (size_t)std::max(c->max_grid, 1) + 64),
                                c->stream));
    c->h_heat_flags.assign(c->N, 0);
    c->has_heat_bc = false;
    c->has_heat_q = false;
    c->heat_ready = true;
    c->heat_facets_dirty = true;
    return PFG_OK;
}

// Per-node lists of the facets that take a heat flux term (all their nodes carry the flag, or
// the free-surface flags for a facet whose nodes are all on the free surface, HeatEquation.inl:
// 319-335; Facet::isOnFreeSurface, Facet.cpp:249-255), in ascending facet order.
int heat_build_facets(pfg_ctx* c) {
    if (!c->heat_facets_dirty) return PFG_OK;
    const int N = c->N, F = c->has_facets ? c->F : 0, dim = c->dim;
    const int fsf = c->prm.heat_fs_flags & (HT_Q | HT_QH | HT_QR);
    std::vector<uint8_t> ff((size_t)std::max(F, 1), 0);
    std::vector<int> cnt((size_t)N + 1, 0);
    for (int f = 0; f < F; ++f) {
        bool fs = true;
        for (int d = 0; d < dim; ++d) fs = fs && (c->h_flags[c->h_facets[(size_t)d * F + f]] & F_FREE_SURFACE);
        int fl = HT_Q | HT_QH | HT_QR;
        for (int d = 0; d < dim; ++d) fl &= fs ? fsf : c->h_heat_flags[c->h_facets[(size_t)d * F + f]];
        ff[f] = (uint8_t)fl;
        if (fl)
            for (int d = 0; d < dim; ++d) cnt[c->h_facets[(size_t)d * F + f] + 1]++;
    }
    for (int n = 0; n < N; ++n) cnt[n + 1] += cnt[n];
    std::vector<int> ent((size_t)std::max(cnt[N], 1));
    std::vector<int> pos(cnt.begin(), cnt.end() - 1);
    for (int f = 0; f < F; ++f)
        if (ff[f])
            for (int d = 0; d < dim; ++d) ent[pos[c->h_facets[(size_t)d * F + f]]++] = f * 4 + d;
    int rc;
    if ((rc = ensure(c, c->hf_ent, sizeof(int) * ent.size())) || (rc = ensure(c, c->hf_fflags, ff.size())))
        return rc;
    PFG_CUDA(c, cudaMemcpyAsync(c->hf_ptr.p, cnt.data(), sizeof(int) * ((size_t)N + 1), cudaMemcpyHostToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->hf_ent.p, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(c->hf_fflags.p, ff.data(), ff.size(), cudaMemcpyHostToDevice, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    bool need_q = false;
    for (int f = 0; f < F; ++f) need_q |= (ff[f] & HT_Q) != 0;
    if (need_q && !c->has_heat_q) return fail(c, PFG_ERR_STATE, "heat facets with a Q flag need pfg_heat_set_flux");
    c->heat_facets_dirty = false;
    return PFG_OK;
}

int heat_step(pfg_ctx* c, double dt, pfg_step_status* st) {
    return c->dim == 2 ? heat_dim<2>(c, dt, st) : heat_dim<3>(c, dt, st);
}

// Jacobi-preconditioned CG (the Chronopoulos-Gear kernels above) on a scalar CSR system of n
// rows (rp, col, val; the diagonal among each row's entries), right-hand side b, from the guess
// in x (overwritten), to ||r|| <= max(rtol ||b||, atol) or max_it iterations.  V holds
// CG_VECTORS x n work values, red 3 max_grid + 64 partial sums and scalars.
int cg_solve(pfg_ctx* c, int n, const int* rp, const int* col, const double* val, const double* b, double* x,
             double* V, double* red, double rtol, double atol, int max_it, int* iters, bool* ok) {
    CgPtrs kp;
    kp.partials = red;
    kp.sc = red + 3 * (size_t)c->max_grid;
    kp.ticket = reinterpret_cast<unsigned*>(kp.sc + 32);
    const size_t ld = (size_t)std::max(n, 1);
    const int grid = std::max(1, std::min(c->max_grid, div_up(n, BLOCK)));
    max_it = std::max(1, max_it);
    k_cg_init<<<grid, BLOCK, 0, c->stream>>>(n, rp, col, val, b, x, V, ld, kp, rtol, atol, INFINITY);
    k_cg_spmv<1><<<grid, BLOCK, 0, c->stream>>>(n, rp, col, val, V, ld, kp, max_it);
    PFG_CHECK_LAUNCH(c);
    double* h = c->h_scalars;
    int done_it = 0;
    while (done_it < max_it) {
        const int m = std::min(8, max_it - done_it);
        for (int it = 0; it < m; ++it) {
            k_cg_update<<<grid, BLOCK, 0, c->stream>>>(n, x, V, ld, kp);
            k_cg_spmv<1><<<grid, BLOCK, 0, c->stream>>>(n, rp, col, val, V, ld, kp, max_it);
        }
        PFG_CHECK_LAUNCH(c);
        done_it += m;
        PFG_CUDA(c, cudaMemcpyAsync(h, kp.sc, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, c->stream));
        PFG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (h[S_DONE] != 0.0) break;
    }
    *ok = h[S_DONE] == 1.0;
    *iters = (int)h[S_ITERS];
    return PFG_OK;
}

// Host work before a BoussinesqWC step is launched or captured: heat buffers, the element
// records and the per-node facet lists.  *changed reports reallocated or rebuilt buffers (a
// captured step graph holding their old addresses must be dropped).
int wc_heat_prepare(pfg_ctx* c, bool* changed) {
    int rc;
    *changed = false;
    if (!c->heat_ready) {
        if ((rc = heat_alloc(c))) return rc;
        *changed = true;
    }
    const size_t need = sizeof(double) * 2 * (size_t)c->npe * std::max(c->E, 1);
    if (c->wch_rec.cap < need) {
        if ((rc = ensure(c, c->wch_rec, need))) return rc;
        *changed = true;
    }
    if (c->heat_facets_dirty) {
        if ((rc = heat_build_facets(c))) return rc;
        *changed = true;
    }
    return PFG_OK;
}

// Enqueue the explicit heat step of one BoussinesqWC step (graph-capturable).
int wc_heat_launch(pfg_ctx* c, const double* tdt) {
    return c->dim == 2 ? wc_heat_dim<2>(c, tdt) : wc_heat_dim<3>(c, tdt);
}

}  // namespace pfg
