// Surface tension on the free-surface facets, gathered at the nodes (header-only device code).
//
// Reference: the facet loops of m_applyBCPSPG (MomContEquationPSPG.inl:155-187) and
// MomEqWCompNewton::m_applyBC (MomEquation.inl:311-335), which add for every free-surface facet
// f of element e
//   FST = -gamma * sum_g w_g B_e^T T(P) P * detJ_f * refSize(dim-1)
// to the momentum rows of the dim+1 nodes of e (MatrixBuilder::getFST/getP/getT,
// MatricesBuilder.inl:166-214,:388-402; facet geometry Facet.cpp:15-77,:130-210).
// P is the tangential projector I - n n^T of the facet in Voigt order, B_e the element's
// strain-rate matrix.  FST does not vary over the facet, so the Gauss sum is the factor
// sum_g w_g, folded with gamma and refSize(dim-1) into FstArgs::coef.
//
// Layout: the host lists the nodes that some free-surface facet's element touches and, per
// listed node, its (facet, local index of the node in the facet's element) entries in
// ascending facet order (the reference's summation order).  k_fst, one thread per listed node,
// recomputes those entries from the current positions (one element Jacobian and one facet
// normal each) and writes the node's force to a dim x N array that is zero at every other
// node; the node kernels of the step add that array to their momentum rows.  No atomics, and
// the node kernels carry one extra load instead of the facet arithmetic (which would raise
// their register count even with gamma = 0).
#pragma once

#include "pfg_device.cuh"

namespace pfg {

struct FstArgs {
    const int* nodes;      // listed nodes; nullptr: no surface tension
    const int* nf_ptr;     // n_nodes + 1 offsets into nf_ent
    const int* nf_ent;     // facet * 4 + local index of the node in the facet's element
    const int* fnodes;     // dim x F facet nodes, fnodes[k * F + f]
    const int* felem;      // element of each facet
    int F, n_nodes;
    double coef;           // gamma * sum_g w_g (3-point facet rule) * refSize(dim - 1)
    float coef32;          // the same, for FP32 kernels
    // problem "Boussinesq" with DgammaDT: the factor gamma + DgammaDT (T_g - Tr) summed over the
    // facet Gauss points is sum_g w_g (gamma - DgammaDT Tr) + DgammaDT sum_g w_g T_g, and
    // sum_g w_g N_k(g) = sum_g w_g / dim for every facet node k of both 3-point rules, so the
    // facet coefficient is coef + tcoef * (sum of the facet's node temperatures)
    const double* T;       // node temperatures, or nullptr
    double tcoef;          // DgammaDT * sum_g w_g / dim * refSize(dim - 1)
};

// Coordinate differences x_a - x_b of an FP64 position array.
struct PosF64 {
    const double* x;
    int N;
    __device__ __forceinline__ double operator()(int a, int b, int d) const {
        return x[(size_t)d * N + a] - x[(size_t)d * N + b];
    }
};

// Adds the surface tension force of listed node j's facet entries to F (velocity components).
template <int DIM, class T, class Pos>
__device__ __forceinline__ void fst_gather(int j, int E, const FstArgs& fa, const int* __restrict__ conn,
                                           const Pos& dx, T (&F)[DIM]) {
    constexpr int NPE = DIM + 1;
    constexpr int NV = DIM == 2 ? 3 : 6;
    const int q1 = fa.nf_ptr[j + 1];
    for (int q = fa.nf_ptr[j]; q < q1; ++q) {
        const int ent = fa.nf_ent[q];
        const int f = ent >> 2, i = ent & 3;
        const int e = fa.felem[f];
        int nd[NPE];
        load_nodes<DIM>(conn, E, e, nd);
        // element shape gradients at node i: invJ from the Jacobian J[r][c] = x_{c+1} - x_0
        // (Element.cpp:15-135, MatricesBuilder.inl:92-127)
        T J[DIM][DIM];
#pragma unroll
        for (int r = 0; r < DIM; ++r)
#pragma unroll
            for (int cc = 0; cc < DIM; ++cc) J[r][cc] = dx(nd[cc + 1], nd[0], r);
        T g[DIM];  // dN_i/dx_f
        if constexpr (DIM == 2) {
            const T det = J[0][0] * J[1][1] - J[1][0] * J[0][1];
            const T inv[2][2] = {{J[1][1] / det, -J[0][1] / det}, {-J[1][0] / det, J[0][0] / det}};
#pragma unroll
            for (int fd = 0; fd < 2; ++fd) g[fd] = i == 0 ? -(inv[0][fd] + inv[1][fd]) : (i == 1 ? inv[0][fd] : inv[1][fd]);
        } else {
            const T det = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1]
                        - J[2][0] * J[1][1] * J[0][2] - J[2][1] * J[1][2] * J[0][0] - J[2][2] * J[1][0] * J[0][1];
            T inv[3][3];
            inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
            inv[0][1] = (J[2][1] * J[0][2] - J[2][2] * J[0][1]) / det;
            inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
            inv[1][0] = (J[2][0] * J[1][2] - J[1][0] * J[2][2]) / det;
            inv[1][1] = (J[0][0] * J[2][2] - J[2][0] * J[0][2]) / det;
            inv[1][2] = (J[1][0] * J[0][2] - J[0][0] * J[1][2]) / det;
            inv[2][0] = (J[1][0] * J[2][1] - J[2][0] * J[1][1]) / det;
            inv[2][1] = (J[2][0] * J[0][1] - J[0][0] * J[2][1]) / det;
            inv[2][2] = (J[0][0] * J[1][1] - J[1][0] * J[0][1]) / det;
#pragma unroll
            for (int fd = 0; fd < 3; ++fd)
                g[fd] = i == 0 ? -(inv[0][fd] + inv[1][fd] + inv[2][fd])
                               : (i == 1 ? inv[0][fd] : (i == 2 ? inv[1][fd] : inv[2][fd]));
        }
        // facet measure and unit normal (Facet::computeDetJ / computeNormal)
        T meas, nv[DIM];
        const int a = fa.fnodes[f], b = fa.fnodes[fa.F + f];
        if constexpr (DIM == 2) {
            const T ux = dx(b, a, 0), uy = dx(b, a, 1);
            const T len = sqrt(ux * ux + uy * uy);
            meas = len / 2;  // detJ of the facet on [-1, 1]
            nv[0] = uy / len;
            nv[1] = -ux / len;
        } else {
            const int c = fa.fnodes[2 * fa.F + f];
            T u[3], w[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                u[d] = dx(b, a, d);
                w[d] = dx(c, a, d);
            }
            const T c0 = u[1] * w[2] - u[2] * w[1], c1 = u[2] * w[0] - u[0] * w[2], c2 = u[0] * w[1] - u[1] * w[0];
            meas = sqrt(c0 * c0 + c1 * c1 + c2 * c2);  // detJ of the facet on the unit triangle
            nv[0] = c0 / meas;
            nv[1] = c1 / meas;
            nv[2] = c2 / meas;
        }
        // P (getP) and w = T(P) P (getT)
        T P[NV], tw[NV];
        if constexpr (DIM == 2) {
            P[0] = 1 - nv[0] * nv[0];
            P[1] = 1 - nv[1] * nv[1];
            P[2] = -nv[0] * nv[1];
            tw[0] = P[0] * P[0] * P[0] + P[2] * P[2] * P[1] + 2 * P[0] * P[2] * P[2];
            tw[1] = P[2] * P[2] * P[0] + P[1] * P[1] * P[1] + 2 * P[2] * P[1] * P[2];
            tw[2] = P[0] * P[2] * P[0] + P[2] * P[1] * P[1] + (P[0] * P[1] + P[2] * P[2]) * P[2];
        } else {
            P[0] = 1 - nv[0] * nv[0];
            P[1] = 1 - nv[1] * nv[1];
            P[2] = 1 - nv[2] * nv[2];
            P[3] = -nv[0] * nv[1];
            P[4] = -nv[0] * nv[2];
            P[5] = -nv[1] * nv[2];
            T Tm[6][6];
            Tm[0][0] = P[0] * P[0]; Tm[0][1] = P[3] * P[3]; Tm[0][2] = P[4] * P[4];
            Tm[0][3] = 2 * P[0] * P[3]; Tm[0][5] = 2 * P[4] * P[3]; Tm[0][4] = 2 * P[0] * P[4];
            Tm[1][0] = Tm[0][1]; Tm[1][1] = P[1] * P[1]; Tm[1][2] = P[5] * P[5];
            Tm[1][3] = 2 * P[3] * P[1]; Tm[1][5] = 2 * P[5] * P[1]; Tm[1][4] = 2 * P[3] * P[5];
            Tm[2][0] = Tm[0][2]; Tm[2][1] = Tm[1][2]; Tm[2][2] = P[2] * P[2];
            Tm[2][3] = 2 * P[5] * P[4]; Tm[2][5] = 2 * P[5] * P[2]; Tm[2][4] = 2 * P[2] * P[4];
            Tm[3][0] = P[0] * P[3]; Tm[3][1] = P[3] * P[1]; Tm[3][2] = P[4] * P[5];
            Tm[3][3] = P[0] * P[1] + P[3] * P[3]; Tm[3][5] = P[4] * P[1] + P[5] * P[3];
            Tm[3][4] = P[4] * P[3] + P[0] * P[5];
            Tm[5][0] = P[3] * P[4]; Tm[5][1] = P[5] * P[1]; Tm[5][2] = P[5] * P[2];
            Tm[5][3] = P[4] * P[1] + P[5] * P[3]; Tm[5][5] = P[1] * P[2] + P[5] * P[5];
            Tm[5][4] = P[5] * P[4] + P[3] * P[2];
            Tm[4][0] = P[0] * P[4]; Tm[4][1] = P[3] * P[5]; Tm[4][2] = P[2] * P[4];
            Tm[4][3] = P[4] * P[3] + P[0] * P[5]; Tm[4][5] = P[5] * P[4] + P[3] * P[2];
            Tm[4][4] = P[2] * P[0] + P[4] * P[4];
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                T s = 0;
#pragma unroll
                for (int k = 0; k < 6; ++k) s += Tm[r][k] * P[k];
                tw[r] = s;
            }
        }
        // rows of B^T w for node i (getB, MatricesBuilder.inl:129-164)
        T cf = sizeof(T) == sizeof(float) ? (T)fa.coef32 : (T)fa.coef;
        if (fa.T) {
            double ts = fa.T[a] + fa.T[b];
            if constexpr (DIM == 3) ts += fa.T[fa.fnodes[2 * fa.F + f]];
            cf = (T)(fa.coef + fa.tcoef * ts);
        }
        const T cm = cf * meas;
        if constexpr (DIM == 2) {
            F[0] -= cm * (g[0] * tw[0] + g[1] * tw[2]);
            F[1] -= cm * (g[1] * tw[1] + g[0] * tw[2]);
        } else {
            F[0] -= cm * (g[0] * tw[0] + g[1] * tw[3] + g[2] * tw[4]);
            F[1] -= cm * (g[1] * tw[1] + g[0] * tw[3] + g[2] * tw[5]);
            F[2] -= cm * (g[2] * tw[2] + g[0] * tw[4] + g[1] * tw[5]);
        }
    }
}

// Surface tension force of every listed node into out (dim x N; the other nodes keep 0).
template <int DIM, class T, class Pos>
__global__ void k_fst(FstArgs fa, int E, const int* __restrict__ conn, Pos dx, int N, T* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= fa.n_nodes) return;
    T F[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) F[d] = 0;
    fst_gather<DIM, T>(j, E, fa, conn, dx, F);
    const int n = fa.nodes[j];
#pragma unroll
    for (int d = 0; d < DIM; ++d) out[(size_t)d * N + n] = F[d];
}

// The facet term runs when gamma >= 1e-15, or (Boussinesq) DgammaDT >= 1e-15
// (MomContEquationPSPG.inl:157-158).
inline bool fst_on(const pfg_ctx* c) {
    return c->prm.gamma >= 1e-15 || (c->prm.boussinesq && c->prm.dgamma_dt >= 1e-15);
}

// Kernel argument block of the context (nodes = nullptr when the term is off or has no entries).
inline FstArgs fst_args(const pfg_ctx* c) {
    FstArgs a{};
    if (!fst_on(c) || c->n_fst_nodes == 0) return a;
    a.nodes = ptr<int>(c->nf_nodes);
    a.n_nodes = c->n_fst_nodes;
    a.nf_ptr = ptr<int>(c->nf_ptr);
    a.nf_ent = ptr<int>(c->nf_ent);
    a.fnodes = ptr<int>(c->fc_nodes);
    a.felem = ptr<int>(c->fc_elem);
    a.F = c->F;
    // 3-point facet rules (Mesh::getGaussWeight, Mesh.cpp:416-450), summed in order, and the
    // reference facet sizes (Mesh::getRefElementSize, Mesh.cpp:472-484)
    const double sumw = c->dim == 2 ? 5.0 / 18.0 + 8.0 / 18.0 + 5.0 / 18.0 : 1.0 / 3.0 + 1.0 / 3.0 + 1.0 / 3.0;
    const double ref = c->dim == 2 ? 2.0 : 0.5;
    a.coef = c->prm.gamma * sumw * ref;
    a.coef32 = (float)a.coef;
    if (c->prm.boussinesq && c->prm.dgamma_dt != 0.0) {
        a.T = ptr<double>(c->heat_t);
        a.coef = (c->prm.gamma - c->prm.dgamma_dt * c->prm.t_ref) * sumw * ref;
        a.tcoef = c->prm.dgamma_dt * sumw / c->dim * ref;
    }
    return a;
}

// The force array the node kernels add (nullptr when surface tension is off).
template <class T>
inline const T* fst_force(const pfg_ctx* c) {
    return (!fst_on(c) || c->n_fst_nodes == 0) ? nullptr : ptr<T>(c->fst_force);
}

}  // namespace pfg
