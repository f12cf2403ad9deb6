// PFEM per-time-step oracle: an FP64 CPU restatement of the reference's hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU library is compared
// against (tests/, __graft_entry__.smoke(), bench.py's cpu_baseline / --impl reference leg).
// No product code path links or calls it.
//
// Parity status: UNPINNED.  The reference (ImperatorS79/PFEM) ships no tests, golden
// vectors or fixtures, and it cannot be built here (Eigen, CGAL, gmsh, sol2 and Lua are
// absent).  This restatement follows the cited reference lines; its element matrices are
// additionally checked against closed forms (tests/golden/make_golden.py).
//
// Every function cites the reference file:line it restates.  Paths are relative to the
// reference project root.  OpenMP is used at the reference's own parallel sites; the
// serial loops (triplet collapse, RHS scatter, WC scatters) stay serial because their
// order defines the floating-point summation order.
//
// Layouts (shared with the GPU library):
//   positions  pos[d*N + n]                     (structure of arrays)
//   connectivity conn[k*E + e], k = 0..dim      (structure of arrays)
//   incompressible states q[f*N + n], f = 0..dim (v_0..v_{d-1}, p)   StatesFromToQ.hpp:9-34
//   WC states s[f*N + n], f = 0..2d+1 (v, p, rho, a)                 WCompNewton/Problem.cpp:18

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint8_t BOUND = 1, FREE_SURFACE = 2, FIXED = 4, DIRICHLET = 8;

// ---------------------------------------------------------------------------------------
// Gauss tables: srcs/mesh/Mesh.cpp:342-530 (values copied as the reference states them)
// ---------------------------------------------------------------------------------------
struct GaussTable {
    int n;
    double pts[4][3];
    double w[4];
    double sf[4][4];     // shape functions at each point (Mesh::getShapeFunctions)
    double refSize;
};

GaussTable gaussTable(int dim) {
    GaussTable t{};
    if (dim == 2) {
        t.n = 3;
        const double p[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}, {2.0 / 3.0, 1.0 / 6.0}};
        for (int g = 0; g < 3; ++g) {
            t.pts[g][0] = p[g][0];
            t.pts[g][1] = p[g][1];
            t.w[g] = 1.0 / 3.0;
            t.sf[g][0] = 1 - p[g][0] - p[g][1];
            t.sf[g][1] = p[g][0];
            t.sf[g][2] = p[g][1];
        }
        t.refSize = 0.5;
    } else {
        t.n = 4;
        const double a = 0.585410196624968, b = 0.138196601125011;
        const double p[4][3] = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
        for (int g = 0; g < 4; ++g) {
            for (int k = 0; k < 3; ++k) t.pts[g][k] = p[g][k];
            t.w[g] = 0.25;
            t.sf[g][0] = 1 - p[g][0] - p[g][1] - p[g][2];
            t.sf[g][1] = p[g][0];
            t.sf[g][2] = p[g][1];
            t.sf[g][3] = p[g][2];
        }
        t.refSize = 0.16666666666666666666666666666667;
    }
    return t;
}

// Small dense row-major matrix with runtime sizes up to 16x16.
struct Mat {
    int r = 0, c = 0;
    double a[16 * 16];
    Mat() {}
    Mat(int rr, int cc) : r(rr), c(cc) { std::memset(a, 0, sizeof(a)); }
    double& operator()(int i, int j) { return a[i * 16 + j]; }
    double operator()(int i, int j) const { return a[i * 16 + j]; }
};

Mat mul(const Mat& A, const Mat& B) {
    Mat C(A.r, B.c);
    for (int i = 0; i < A.r; ++i)
        for (int j = 0; j < B.c; ++j) {
            double s = 0;
            for (int k = 0; k < A.c; ++k) s += A(i, k) * B(k, j);
            C(i, j) = s;
        }
    return C;
}

Mat transpose(const Mat& A) {
    Mat T(A.c, A.r);
    for (int i = 0; i < A.r; ++i)
        for (int j = 0; j < A.c; ++j) T(j, i) = A(i, j);
    return T;
}

struct ElemGeom {
    double J[3][3];
    double invJ[3][3];
    double detJ;
};

struct PspgParams {
    double rho, mu, dt;
    double g[3];
    double gamma;      // surface tension coefficient (MomContEq "gamma")
    double tau0;       // Bingham yield stress (problem "Bingham"; 0 = Newtonian)
    double mReg;       // Bingham regularisation parameter
    // problem "Boussinesq" (MomContEquation.inl:34-37,164-171,193-199): body-force factor
    // rho (1 - alpha (T - Tr)) and PSPG gravity factor 1 - alpha (T - Tr) at each Gauss point,
    // T interpolated from the node temperatures (null: not Boussinesq)
    double alpha, Tr;
    const double* T;
    double dgammaDT;   // Boussinesq surface tension gamma + DgammaDT (T - Tr) (:174-179)
};

// HeatEqIncompNewton material (HeatEquation.inl:27-32) and the heat boundary-condition flags
struct HeatParams {
    double rho, cv, k;
    double h, Tinf, epsRad;
    int32_t fsFlags;   // flags of the free-surface tag (-2): HT_Q / HT_QH / HT_QR
    int32_t phaseChange;  // latent heat in the M factor (HeatEquation.inl:36-45, 60-66)
    double Tm, DT, Lm;    // melting temperature, melting range, latent heat
};

// d fl / dT of the liquid fraction, HeatEqIncompNewton::m_getDflDT (HeatEquation.inl:421-425)
double dFlDT(const HeatParams& p, double T) {
    const double d3 = p.DT * p.DT * p.DT;
    const double in = static_cast<double>(T > p.Tm - p.DT / 2) * static_cast<double>(T < p.Tm + p.DT / 2);
    return in * (-2 * 3 / d3 * T * T + 6 * 2 * p.Tm / d3 * T + (3 / (2 * p.DT) - 6 * p.Tm * p.Tm / d3));
}
constexpr uint8_t HT_T = 1, HT_Q = 2, HT_QH = 4, HT_QR = 8;

struct WcParams {
    double K0, K0p, rhoStar, mu;
    double g[3];
    int meduri;        // ContEq stabilization "Meduri" (1) or "None" (0)
    double sc;         // securityCoeff
    double maxDT;
    double gamma;      // surface tension coefficient (MomEq "gamma")
    int version;       // SolverWCompNewton id: 0 "CDS_dpdt", 1 "CDS_rho", 2 "CDS_drhodt"
};

// Problem "BoussinesqWC" (WCompNewton/Solver.cpp:72-146): MomEq material (MomEquation.inl:36-51)
// and HeatEqWCompNewton material (HeatEquation.inl:26-45).  Carman-Kozeny damping in the
// momentum equation and latent heat in the heat mass factor when phaseChange is set.
struct WcBqParams {
    double alpha, Tr, dgammaDT;
    int32_t phaseChange;   // MomEq: C, eps, Tm, DT given; HeatEq: Tm, DT, Lm given
    int32_t fsFlags;       // heat flags of the free-surface tag (-2)
    double C, eps, Tm, DT, Lm;
    double k, cv, h, Tinf, epsRad;
};

// Liquid fraction of MomEqWCompNewton::m_getFl (MomEquation.inl:377-381).
double flWC(double Tm, double DT, double T) {
    const double d3 = DT * DT * DT;
    return static_cast<double>(T > Tm - DT / 2) * static_cast<double>(T < Tm + DT / 2) *
               (-2 / d3 * T * T * T + 6 * Tm / d3 * T * T + (3 / (2 * DT) - 6 * Tm * Tm / d3) * T +
                (0.5 - 1.5 * Tm / DT + 2 * Tm * Tm * Tm / d3)) +
           static_cast<double>(T > Tm + DT / 2);
}

}  // namespace

struct OrcMesh {
    int dim, N, E, npe;
    std::vector<double> pos, posSave;
    std::vector<uint8_t> flags;
    std::vector<uint8_t> isFree;
    std::vector<int32_t> conn;
    std::vector<ElemGeom> geom;
    GaussTable gt;
    // facets of the alpha shape (Mesh::m_facetsList): dim nodes each (facets[k*F + f]) and the
    // element each belongs to (Facet::m_elementIndex)
    int F = 0;
    std::vector<int32_t> facets, facetElm;
    // assembled PSPG system, Eigen column-major (CSC) storage
    std::vector<int32_t> colptr, rowidx;
    std::vector<double> vals, b;
    // fractional step: M (velocity correction), MK_dt (velocity prediction), L (pressure) in
    // CSC storage with their right-hand sides, and the per-element D^T and L of the step
    struct Csc {
        std::vector<int32_t> colptr, rowidx;
        std::vector<double> vals;
    } fsM, fsMK, fsL;
    std::vector<double> fsbV, fsbP, fsbVc;
    std::vector<std::vector<double>> fsDT, fsLe;

    bool bound(int n) const { return flags[n] & BOUND; }
    bool fixed(int n) const { return flags[n] & FIXED; }
    bool dirichlet(int n) const { return (flags[n] & BOUND) && (flags[n] & DIRICHLET); }
    int node(int e, int k) const { return conn[(size_t)k * E + e]; }
    double x(int n, int d) const { return pos[(size_t)d * N + n]; }
};

namespace {

// Element::computeJ / computeDetJ / computeInvJ, srcs/mesh/Element.cpp:15-135
void computeGeometry(const OrcMesh& m, int e, ElemGeom& g) {
    std::memset(&g, 0, sizeof(g));
    if (m.dim == 2) {
        int n0 = m.node(e, 0), n1 = m.node(e, 1), n2 = m.node(e, 2);
        double x0 = m.x(n0, 0), x1 = m.x(n1, 0), x2 = m.x(n2, 0);
        double y0 = m.x(n0, 1), y1 = m.x(n1, 1), y2 = m.x(n2, 1);
        g.J[0][0] = x1 - x0; g.J[0][1] = x2 - x0;
        g.J[1][0] = y1 - y0; g.J[1][1] = y2 - y0;
        g.detJ = g.J[0][0] * g.J[1][1] - g.J[1][0] * g.J[0][1];
        g.invJ[0][0] = g.J[1][1] / g.detJ;
        g.invJ[0][1] = -g.J[0][1] / g.detJ;
        g.invJ[1][0] = -g.J[1][0] / g.detJ;
        g.invJ[1][1] = g.J[0][0] / g.detJ;
    } else {
        int nn[4] = {m.node(e, 0), m.node(e, 1), m.node(e, 2), m.node(e, 3)};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) g.J[r][c] = m.x(nn[c + 1], r) - m.x(nn[0], r);
        auto& J = g.J;
        g.detJ = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1]
               - J[2][0] * J[1][1] * J[0][2] - J[2][1] * J[1][2] * J[0][0] - J[2][2] * J[1][0] * J[0][1];
        double d = g.detJ;
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

// Mesh::updateNodesPosition* element loop, srcs/mesh/Mesh.cpp:1258-1264
void computeAllGeometry(OrcMesh& m) {
#pragma omp parallel for
    for (int e = 0; e < m.E; ++e) computeGeometry(m, e, m.geom[e]);
}

// MatrixBuilder::getGradN, srcs/simulation/matricesBuilder/MatricesBuilder.inl:92-127
Mat getGradN(int dim, const ElemGeom& g) {
    Mat G(dim, dim + 1);
    for (int r = 0; r < dim; ++r) {
        double s = 0;
        for (int k = 0; k < dim; ++k) s += g.invJ[k][r];
        G(r, 0) = -s;
        for (int k = 0; k < dim; ++k) G(r, k + 1) = g.invJ[k][r];
    }
    return G;
}

// MatrixBuilder::getB (Voigt strain rate), MatricesBuilder.inl:129-164
Mat getB(int dim, const Mat& G) {
    const int npe = dim + 1;
    if (dim == 2) {
        Mat B(3, 6);
        for (int j = 0; j < 3; ++j) {
            B(0, j) = B(2, 3 + j) = G(0, j);
            B(1, 3 + j) = B(2, j) = G(1, j);
        }
        return B;
    }
    Mat B(6, 12);
    for (int j = 0; j < npe; ++j) {
        B(0, j) = B(3, 4 + j) = B(4, 8 + j) = G(0, j);
        B(1, 4 + j) = B(3, j) = B(5, 8 + j) = G(1, j);
        B(2, 8 + j) = B(4, j) = B(5, 4 + j) = G(2, j);
    }
    return B;
}

// N row at Gauss point g and Ntilde (dim x dim*npe), MatricesBuilder.inl:5-84
Mat getNtilde(int dim, const GaussTable& t, int g) {
    Mat Nt(dim, dim * (dim + 1));
    for (int f = 0; f < dim; ++f)
        for (int j = 0; j <= dim; ++j) Nt(f, f * (dim + 1) + j) = t.sf[g][j];
    return Nt;
}

double nDot(const GaussTable& t, int g, const double* vals, int npe) {
    double s = 0;
    for (int j = 0; j < npe; ++j) s += t.sf[g][j] * vals[j];
    return s;
}

// getM with a per-Gauss-point factor, MatricesBuilder.inl:216-229
template <class F>
Mat getM(const OrcMesh& m, const ElemGeom& geo, F factor) {
    const int npe = m.npe;
    Mat M(npe, npe);
    for (int g = 0; g < m.gt.n; ++g) {
        double f = factor(g) * m.gt.w[g];
        for (int i = 0; i < npe; ++i)
            for (int j = 0; j < npe; ++j) M(i, j) += f * m.gt.sf[g][i] * m.gt.sf[g][j];
    }
    double s = geo.detJ * m.gt.refSize;
    for (int i = 0; i < npe; ++i)
        for (int j = 0; j < npe; ++j) M(i, j) *= s;
    return M;
}

// getK = |e| * (sum_g f w) * B^T Ddev B, MatricesBuilder.inl:276-290
Mat getK(const OrcMesh& m, const ElemGeom& geo, double factorSum, const Mat& B, const Mat& ddev) {
    Mat K = mul(mul(transpose(B), ddev), B);
    double s = geo.detJ * m.gt.refSize * factorSum;
    for (int i = 0; i < K.r; ++i)
        for (int j = 0; j < K.c; ++j) K(i, j) *= s;
    return K;
}

// getD = |e| * (sum_g f w N^T) m^T B, MatricesBuilder.inl:292-306
template <class F>
Mat getD(const OrcMesh& m, const ElemGeom& geo, F factor, const Mat& B) {
    const int npe = m.npe, dim = m.dim;
    double sumWNT[4] = {0, 0, 0, 0};
    for (int g = 0; g < m.gt.n; ++g) {
        double f = factor(g) * m.gt.w[g];
        for (int i = 0; i < npe; ++i) sumWNT[i] += f * m.gt.sf[g][i];
    }
    // m^T B : m = [1,...,1 (dim), 0, ...]
    double mB[12];
    for (int j = 0; j < dim * npe; ++j) {
        double s = 0;
        for (int k = 0; k < dim; ++k) s += B(k, j);
        mB[j] = s;
    }
    Mat D(npe, dim * npe);
    double s = geo.detJ * m.gt.refSize;
    for (int i = 0; i < npe; ++i)
        for (int j = 0; j < dim * npe; ++j) D(i, j) = s * sumWNT[i] * mB[j];
    return D;
}

// getC = |e| gradN^T (sum_g f w Ntilde_g), MatricesBuilder.inl:324-338
Mat getC(const OrcMesh& m, const ElemGeom& geo, double factor, const Mat& G) {
    const int npe = m.npe, dim = m.dim;
    Mat sumNW(dim, dim * npe);
    for (int g = 0; g < m.gt.n; ++g) {
        Mat Nt = getNtilde(dim, m.gt, g);
        for (int r = 0; r < dim; ++r)
            for (int c = 0; c < dim * npe; ++c) sumNW(r, c) += factor * Nt(r, c) * m.gt.w[g];
    }
    Mat C = mul(transpose(G), sumNW);
    double s = geo.detJ * m.gt.refSize;
    for (int i = 0; i < C.r; ++i)
        for (int j = 0; j < C.c; ++j) C(i, j) *= s;
    return C;
}

// getL = |e| (sum_g f w) gradN^T gradN, MatricesBuilder.inl:308-322
Mat getL(const OrcMesh& m, const ElemGeom& geo, double factorSum, const Mat& G) {
    Mat L = mul(transpose(G), G);
    double s = geo.detJ * m.gt.refSize * factorSum;
    for (int i = 0; i < L.r; ++i)
        for (int j = 0; j < L.c; ++j) L(i, j) *= s;
    return L;
}

// getF = |e| sum_g f w Ntilde_g^T vec, MatricesBuilder.inl:340-355
template <class F>
void getF(const OrcMesh& m, const ElemGeom& geo, F factor, const double* vec, double* out) {
    const int npe = m.npe, dim = m.dim;
    for (int i = 0; i < dim * npe; ++i) out[i] = 0;
    for (int g = 0; g < m.gt.n; ++g) {
        Mat Nt = getNtilde(dim, m.gt, g);
        double f = factor(g) * m.gt.w[g];
        for (int c = 0; c < dim * npe; ++c) {
            double s = 0;
            for (int r = 0; r < dim; ++r) s += Nt(r, c) * vec[r];
            out[c] += f * s;
        }
    }
    double s = geo.detJ * m.gt.refSize;
    for (int i = 0; i < dim * npe; ++i) out[i] *= s;
}

// getH = |e| sum_g f w gradN^T vec, MatricesBuilder.inl:372-386
template <class F>
void getH(const OrcMesh& m, const ElemGeom& geo, F factor, const Mat& G, const double* vec, double* out) {
    const int npe = m.npe, dim = m.dim;
    for (int i = 0; i < npe; ++i) out[i] = 0;
    for (int g = 0; g < m.gt.n; ++g) {
        const double f = factor(g);
        for (int i = 0; i < npe; ++i) {
            double s = 0;
            for (int r = 0; r < dim; ++r) s += G(r, i) * vec[r];
            out[i] += f * s * m.gt.w[g];
        }
    }
    double s = geo.detJ * m.gt.refSize;
    for (int i = 0; i < npe; ++i) out[i] *= s;
}

Mat ddevIncomp(int dim) {  // MomContEquation.inl:73-94 (file offsets of the .inl)
    int nv = dim == 2 ? 3 : 6;
    Mat D(nv, nv);
    for (int i = 0; i < dim; ++i) D(i, i) = 2;
    for (int i = dim; i < nv; ++i) D(i, i) = 1;
    return D;
}

Mat ddevWC(int dim) {  // WCompNewton/MomEquation.inl:63-83
    int nv = dim == 2 ? 3 : 6;
    Mat D(nv, nv);
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j) D(i, j) = (i == j) ? 4.0 / 3 : -2.0 / 3;
    for (int i = dim; i < nv; ++i) D(i, i) = 1;
    return D;
}

// Facet Gauss rule (nGPLD = 3, HeatEquation.inl:13-22): Mesh::getGaussPoints/getGaussWeight/
// getShapeFunctions/getRefElementSize of dimension d-1 (Mesh.cpp:342-530).
struct FacetGauss {
    double xi[3][2];
    double w[3];
    double sf[3][3];
    double ref;
};

FacetGauss facetGauss(int dim) {
    FacetGauss t{};
    if (dim == 2) {
        const double x[3] = {-std::sqrt(3.0 / 5.0), 0.0, std::sqrt(3.0 / 5.0)};
        const double w[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};
        for (int g = 0; g < 3; ++g) {
            t.xi[g][0] = x[g];
            t.w[g] = w[g];
            t.sf[g][0] = (1 - x[g]) / 2;
            t.sf[g][1] = (1 + x[g]) / 2;
        }
        t.ref = 2.0;
    } else {
        const double p[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}, {2.0 / 3.0, 1.0 / 6.0}};
        for (int g = 0; g < 3; ++g) {
            t.xi[g][0] = p[g][0];
            t.xi[g][1] = p[g][1];
            t.w[g] = 1.0 / 3.0;
            t.sf[g][0] = 1 - p[g][0] - p[g][1];
            t.sf[g][1] = p[g][0];
            t.sf[g][2] = p[g][1];
        }
        t.ref = 0.5;
    }
    return t;
}

// ---------------------------------------------------------------------------------------
// Surface tension on the facets
// ---------------------------------------------------------------------------------------
// Facet::computeJ / computeDetJ (srcs/mesh/Facet.cpp:15-77) and Facet::computeNormal
// (:130-210).  The normal's orientation (flipped away from the out node) is not restated:
// only n n^T enters the surface tension term.
void facetGeometry(const OrcMesh& m, int f, double& detJ, double n[3]) {
    const int a = m.facets[f], b = m.facets[(size_t)m.F + f];
    n[0] = n[1] = n[2] = 0;
    if (m.dim == 2) {
        const double J00 = (m.x(b, 0) - m.x(a, 0)) / 2, J10 = (m.x(b, 1) - m.x(a, 1)) / 2;
        detJ = std::sqrt(J00 * J00 + J10 * J10);
        n[0] = m.x(b, 1) - m.x(a, 1);
        n[1] = m.x(a, 0) - m.x(b, 0);
        const double norm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
        n[0] /= norm;
        n[1] /= norm;
    } else {
        const int c = m.facets[2 * (size_t)m.F + f];
        double u[3], w[3];
        for (int d = 0; d < 3; ++d) {
            u[d] = m.x(b, d) - m.x(a, d);
            w[d] = m.x(c, d) - m.x(a, d);
        }
        const double g0 = u[1] * w[2] - w[1] * u[2], g1 = u[2] * w[0] - w[2] * u[0], g2 = u[0] * w[1] - w[0] * u[1];
        detJ = std::sqrt(g0 * g0 + g1 * g1 + g2 * g2);
        n[0] = u[1] * w[2] - u[2] * w[1];
        n[1] = u[2] * w[0] - u[0] * w[2];
        n[2] = u[0] * w[1] - u[1] * w[0];
        const double norm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int d = 0; d < 3; ++d) n[d] /= norm;
    }
}

// MatrixBuilder::getP, MatricesBuilder.inl:166-190: the tangential projector I - n n^T in
// Voigt order (2D: 11, 22, 12; 3D: 11, 22, 33, 12, 13, 23).
Mat getP(int dim, const double n[3]) {
    if (dim == 2) {
        Mat P(3, 1);
        P(0, 0) = 1 - n[0] * n[0];
        P(1, 0) = 1 - n[1] * n[1];
        P(2, 0) = -n[0] * n[1];
        return P;
    }
    Mat P(6, 1);
    P(0, 0) = 1 - n[0] * n[0];
    P(1, 0) = 1 - n[1] * n[1];
    P(2, 0) = 1 - n[2] * n[2];
    P(3, 0) = -n[0] * n[1];
    P(4, 0) = -n[0] * n[2];
    P(5, 0) = -n[1] * n[2];
    return P;
}

// MatrixBuilder::getT, MatricesBuilder.inl:192-214 (entry by entry).
Mat getT(int dim, const Mat& Pm) {
    auto P = [&](int i) { return Pm(i, 0); };
    if (dim == 2) {
        Mat T(3, 3);
        T(0, 0) = P(0) * P(0); T(0, 1) = P(2) * P(2); T(0, 2) = 2 * P(0) * P(2);
        T(1, 0) = T(0, 1);     T(1, 1) = P(1) * P(1); T(1, 2) = 2 * P(2) * P(1);
        T(2, 0) = P(0) * P(2); T(2, 1) = P(2) * P(1); T(2, 2) = P(0) * P(1) + P(2) * P(2);
        return T;
    }
    Mat T(6, 6);
    T(0, 0) = P(0) * P(0); T(0, 1) = P(3) * P(3); T(0, 2) = P(4) * P(4);
    T(0, 3) = 2 * P(0) * P(3); T(0, 5) = 2 * P(4) * P(3); T(0, 4) = 2 * P(0) * P(4);
    T(1, 0) = T(0, 1); T(1, 1) = P(1) * P(1); T(1, 2) = P(5) * P(5);
    T(1, 3) = 2 * P(3) * P(1); T(1, 5) = 2 * P(5) * P(1); T(1, 4) = 2 * P(3) * P(5);
    T(2, 0) = T(0, 2); T(2, 1) = T(1, 2); T(2, 2) = P(2) * P(2);
    T(2, 3) = 2 * P(5) * P(4); T(2, 5) = 2 * P(5) * P(2); T(2, 4) = 2 * P(2) * P(4);
    T(3, 0) = P(0) * P(3); T(3, 1) = P(3) * P(1); T(3, 2) = P(4) * P(5);
    T(3, 3) = P(0) * P(1) + P(3) * P(3); T(3, 5) = P(4) * P(1) + P(5) * P(3); T(3, 4) = P(4) * P(3) + P(0) * P(5);
    T(5, 0) = P(3) * P(4); T(5, 1) = P(5) * P(1); T(5, 2) = P(5) * P(2);
    T(5, 3) = P(4) * P(1) + P(5) * P(3); T(5, 5) = P(1) * P(2) + P(5) * P(5); T(5, 4) = P(5) * P(4) + P(3) * P(2);
    T(4, 0) = P(0) * P(4); T(4, 1) = P(3) * P(5); T(4, 2) = P(2) * P(4);
    T(4, 3) = P(4) * P(3) + P(0) * P(5); T(4, 5) = P(5) * P(4) + P(3) * P(2); T(4, 4) = P(2) * P(0) + P(4) * P(4);
    return T;
}

// MatrixBuilder::getFST, MatricesBuilder.inl:388-402, with the constant factor gamma of
// setFSTcomputeFactor (IncompNewton/MomContEquation.inl:208-213, WCompNewton/MomEquation.inl:
// 141-146).  Three facet Gauss points (nGPLD = 3, MomContEquation.inl:17,22), weights of
// Mesh::getGaussWeight (Mesh.cpp:416-450), reference sizes of Mesh::getRefElementSize
// (Mesh.cpp:472-484).  FST[i + d*npe] is the force on velocity component d of element node i.
// With T (problem "Boussinesq") the factor is gamma + dgdt (T_g - Tr) at each facet Gauss point,
// T_g interpolated from the facet's node temperatures (MomContEquation.inl:174-179).
void getFST(const OrcMesh& m, int f, double gamma, double* FST, const double* Tn = nullptr, double dgdt = 0,
            double Tr = 0) {
    const int dim = m.dim, npe = m.npe;
    const FacetGauss fg = facetGauss(dim);
    const double* w = fg.w;
    const double refLD = fg.ref;
    const ElemGeom& geo = m.geom[m.facetElm[f]];
    Mat B = getB(dim, getGradN(dim, geo));
    double detJ, n[3];
    facetGeometry(m, f, detJ, n);
    Mat P = getP(dim, n);
    Mat T = getT(dim, P);
    Mat BtTP = mul(mul(transpose(B), T), P);
    for (int r = 0; r < dim * npe; ++r) FST[r] = 0;
    for (int g = 0; g < 3; ++g) {
        double fac = gamma;
        if (Tn) {
            double Tg = 0;
            for (int k = 0; k < dim; ++k) Tg += fg.sf[g][k] * Tn[m.facets[(size_t)k * m.F + f]];
            fac = gamma + dgdt * (Tg - Tr);
        }
        for (int r = 0; r < dim * npe; ++r) FST[r] -= fac * BtTP(r, 0) * w[g];
    }
    for (int r = 0; r < dim * npe; ++r) FST[r] *= detJ * refLD;
}

// The facet loops of m_applyBCPSPG (MomContEquationPSPG.inl:155-187; a facet counts when any
// of its nodes is on the free surface) and MomEqWCompNewton::m_applyBC (MomEquation.inl:
// 311-335; Facet::isOnFreeSurface, Facet.cpp:249-255: all of its nodes), adding each facet's
// FST to the velocity rows target[node + d*N] in facet order.
void addSurfaceTension(const OrcMesh& m, double gamma, bool anyNode, double* target, const double* T = nullptr,
                       double dgdt = 0, double Tr = 0) {
    if (gamma < 1e-15 && !(T && dgdt >= 1e-15)) return;
    const int dim = m.dim, npe = m.npe, N = m.N;
    double FST[12];
    for (int f = 0; f < m.F; ++f) {
        int cnt = 0;
        for (int k = 0; k < dim; ++k) cnt += (m.flags[m.facets[(size_t)k * m.F + f]] & FREE_SURFACE) ? 1 : 0;
        if (anyNode ? cnt == 0 : cnt < dim) continue;
        getFST(m, f, gamma, FST, T, dgdt, Tr);
        const int e = m.facetElm[f];
        for (int i = 0; i < npe; ++i)
            for (int d = 0; d < dim; ++d) target[m.node(e, i) + (size_t)d * N] += FST[i + d * npe];
    }
}

// MomContEqIncompNewton::m_computeTauPSPG, MomContEquationPSPG.inl:237-259
double computeTau(const OrcMesh& m, int e, const ElemGeom& geo, const PspgParams& p, const double* q) {
    const double h = std::sqrt(m.gt.refSize * geo.detJ / M_PI);
    double U = 0;
    for (int k = 0; k < m.npe; ++k) {
        int n = m.node(e, k);
        double nodeU = 0;
        for (int d = 0; d < m.dim; ++d) {
            double v = q[(size_t)d * m.N + n];
            nodeU += v * v;
        }
        U += std::sqrt(nodeU);
    }
    U /= (m.dim + 1);
    const double dt = p.dt;
    return 1 / std::sqrt((2 / dt) * (2 / dt) + (2 * U / h) * (2 * U / h)
                         + 9 * (4 * p.mu / (h * h * p.rho)) * (4 * p.mu / (h * h * p.rho)));
}

// Element matrix Ae ((d+1)npe)^2 and vector be of m_buildAbPSPG, MomContEquationPSPG.inl:26-53
void pspgElement(const OrcMesh& m, int e, const PspgParams& p, const double* qIter, const double* qPrev,
                 Mat& Ae, double* be) {
    const int dim = m.dim, npe = m.npe;
    const ElemGeom& geo = m.geom[e];
    const double dt = p.dt;
    double tau = computeTau(m, e, geo, p, qIter);
    Mat G = getGradN(dim, geo);
    Mat B = getB(dim, G);
    Mat Ms = getM(m, geo, [&](int) { return p.rho; });
    for (int i = 0; i < npe; ++i)
        for (int j = 0; j < npe; ++j) Ms(i, j) *= (1 / dt);
    // K factor (setKcomputeFactor, MomContEquation.inl:102-131): mu, or for a Bingham fluid
    // mu + tau0 (1 - exp(-mReg gd)) / gd with gd = sqrt(V^T B^T ddev B V) of the iterate
    double mue = p.mu;
    if (p.tau0 > 0) {
        Mat dd = ddevIncomp(dim);
        const int nv = dim * npe;
        double V[12];
        for (int f = 0; f < dim; ++f)
            for (int k = 0; k < npe; ++k) V[f * npe + k] = qIter[(size_t)f * m.N + m.node(e, k)];
        double gd2 = 0;
        for (int r = 0; r < B.r; ++r) {
            double eps = 0;
            for (int c = 0; c < nv; ++c) eps += B(r, c) * V[c];
            gd2 += eps * dd(r, r) * eps;
        }
        const double gd = std::sqrt(gd2);
        const double muEq = gd < 1e-15 ? p.tau0 * p.mReg : p.tau0 * (1 - std::exp(-p.mReg * gd)) / gd;
        mue = p.mu + muEq;
    }
    double sumW = 0;
    for (int g = 0; g < m.gt.n; ++g) sumW += mue * m.gt.w[g];
    Mat K = getK(m, geo, sumW, B, ddevIncomp(dim));
    Mat D = getD(m, geo, [](int) { return 1.0; }, B);
    Mat C = getC(m, geo, 1.0, G);
    for (int i = 0; i < C.r; ++i)
        for (int j = 0; j < C.c; ++j) C(i, j) *= (tau / dt);
    double lsum = 0;
    for (int g = 0; g < m.gt.n; ++g) lsum += (1 / p.rho) * m.gt.w[g];
    Mat L = getL(m, geo, lsum, G);
    double Fe[12], He[4];
    if (p.T) {
        double Te[4];
        for (int k = 0; k < npe; ++k) Te[k] = p.T[m.node(e, k)];
        auto boussinesq = [&](int g) { return 1 - p.alpha * (nDot(m.gt, g, Te, npe) - p.Tr); };
        getF(m, geo, [&](int g) { return p.rho * boussinesq(g); }, p.g, Fe);
        getH(m, geo, boussinesq, G, p.g, He);
    } else {
        getF(m, geo, [&](int) { return p.rho; }, p.g, Fe);
        getH(m, geo, [](int) { return 1.0; }, G, p.g, He);
    }
    for (int i = 0; i < npe; ++i) He[i] *= tau;

    const int nv = dim * npe, nt = (dim + 1) * npe;
    Ae = Mat(nt, nt);
    // [Me_dt + Ke, -De^T ; Ce_dt + De, tau*Le]
    for (int i = 0; i < nv; ++i)
        for (int j = 0; j < nv; ++j) {
            double md = ((i / npe) == (j / npe)) ? Ms(i % npe, j % npe) : 0.0;
            Ae(i, j) = md + K(i, j);
        }
    for (int i = 0; i < nv; ++i)
        for (int j = 0; j < npe; ++j) Ae(i, nv + j) = -D(j, i);
    for (int i = 0; i < npe; ++i)
        for (int j = 0; j < nv; ++j) Ae(nv + i, j) = C(i, j) + D(i, j);
    for (int i = 0; i < npe; ++i)
        for (int j = 0; j < npe; ++j) Ae(nv + i, nv + j) = tau * L(i, j);

    double vPrev[12];
    for (int f = 0; f < dim; ++f)
        for (int k = 0; k < npe; ++k) vPrev[f * npe + k] = qPrev[(size_t)f * m.N + m.node(e, k)];
    for (int i = 0; i < nv; ++i) {
        double s = 0;
        for (int j = 0; j < nv; ++j) {
            double md = ((i / npe) == (j / npe)) ? Ms(i % npe, j % npe) : 0.0;
            s += md * vPrev[j];
        }
        be[i] = Fe[i] + s;
    }
    for (int i = 0; i < npe; ++i) {
        double s = 0;
        for (int j = 0; j < nv; ++j) s += C(i, j) * vPrev[j];
        be[nv + i] = He[i] + s;
    }
}

struct Triplet {
    int32_t row, col;
    double val;
};

// Eigen's SparseMatrix::setFromTriplets: duplicates are summed in triplet order, storage is
// column-major with sorted row indices.  A stable sort by (col, row) keeps triplet order
// inside each duplicate group, then the group is summed left to right.
void toCsc(const std::vector<Triplet>& indexA, int R, std::vector<int32_t>& colptr, std::vector<int32_t>& rowidx,
           std::vector<double>& vals);

void setFromTriplets(OrcMesh& m, const std::vector<Triplet>& indexA, int R) {
    toCsc(indexA, R, m.colptr, m.rowidx, m.vals);
}

void toCsc(const std::vector<Triplet>& indexA, int R, std::vector<int32_t>& colptr, std::vector<int32_t>& rowidx,
           std::vector<double>& vals) {
    std::vector<uint32_t> order(indexA.size());
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        const Triplet &ta = indexA[a], &tb = indexA[b];
        return ta.col != tb.col ? ta.col < tb.col : ta.row < tb.row;
    });
    colptr.assign(R + 1, 0);
    rowidx.clear();
    vals.clear();
    rowidx.reserve(indexA.size() / 3);
    vals.reserve(indexA.size() / 3);
    for (size_t k = 0; k < order.size();) {
        const Triplet& t = indexA[order[k]];
        double s = t.val;
        size_t k2 = k + 1;
        while (k2 < order.size() && indexA[order[k2]].col == t.col && indexA[order[k2]].row == t.row)
            s += indexA[order[k2++]].val;
        rowidx.push_back(t.row);
        vals.push_back(s);
        colptr[t.col + 1]++;
        k = k2;
    }
    for (int c = 0; c < R; ++c) colptr[c + 1] += colptr[c];
}

// ---------------------------------------------------------------------------------------
// Heat equation (HeatEqIncompNewton), srcs/simulation/physics/IncompNewton/HeatEquation.inl
// ---------------------------------------------------------------------------------------
// Facet::computeNormal (Facet.cpp:130-210): the normal of facetGeometry turned away from the
// element's node that is not on the facet (Facet::getOutNode).
void orientedNormal(const OrcMesh& m, int f, double n[3]) {
    double detJ;
    facetGeometry(m, f, detJ, n);
    const int e = m.facetElm[f], a = m.facets[f];
    int out = -1;
    for (int k = 0; k < m.npe; ++k) {
        const int v = m.node(e, k);
        bool on = false;
        for (int i = 0; i < m.dim; ++i) on |= m.facets[(size_t)i * m.F + f] == v;
        if (!on) out = v;
    }
    double dot = 0;
    for (int d = 0; d < m.dim; ++d) dot += n[d] * (m.x(out, d) - m.x(a, d));
    if (dot > 0)
        for (int d = 0; d < m.dim; ++d) n[d] = -n[d];
}

// Element matrices of HeatEqIncompNewton::m_buildAb (HeatEquation.inl:240-246): Me with the
// factor cv rho (:54-59), with phase change (cv + dfl/dT(T_g) Lm) rho at each Gauss point, T_g
// from the node states Ts (:60-66), and Le = dt getL with the factor k (:70-74).
void heatElement(const OrcMesh& m, int e, const HeatParams& p, double dt, const double* Ts, Mat& Me, Mat& Le) {
    const ElemGeom& geo = m.geom[e];
    Mat G = getGradN(m.dim, geo);
    if (p.phaseChange) {
        double te[4];
        for (int k = 0; k < m.npe; ++k) te[k] = Ts[m.node(e, k)];
        Me = getM(m, geo, [&](int g) { return (p.cv + dFlDT(p, nDot(m.gt, g, te, m.npe)) * p.Lm) * p.rho; });
    } else {
        Me = getM(m, geo, [&](int) { return p.cv * p.rho; });
    }
    double ksum = 0;
    for (int g = 0; g < m.gt.n; ++g) ksum += p.k * m.gt.w[g];
    Le = getL(m, geo, ksum, G);
    for (int i = 0; i < Le.r; ++i)
        for (int j = 0; j < Le.c; ++j) Le(i, j) = dt * Le(i, j);
}

}  // namespace

extern "C" {

OrcMesh* orc_create(int dim, int N, const double* pos, const uint8_t* flags, int E, const int32_t* conn) {
    if ((dim != 2 && dim != 3) || N <= 0 || E < 0) return nullptr;
    OrcMesh* m = new OrcMesh();
    m->dim = dim;
    m->N = N;
    m->E = E;
    m->npe = dim + 1;
    m->pos.assign(pos, pos + (size_t)dim * N);
    m->posSave = m->pos;
    m->flags.assign(flags, flags + N);
    m->conn.assign(conn, conn + (size_t)(dim + 1) * E);
    m->isFree.assign(N, 1);
    for (size_t i = 0; i < m->conn.size(); ++i) m->isFree[m->conn[i]] = 0;
    m->geom.resize(E);
    m->gt = gaussTable(dim);
    computeAllGeometry(*m);
    return m;
}

void orc_destroy(OrcMesh* m) { delete m; }

// The facet list the alpha shape leaves behind (Mesh2D.cpp:199-244, Mesh3D.cpp:232-282):
// facets[k*F + f] (k < dim) and the element of each facet.  Returns 0, or -1 on bad input.
int orc_set_facets(OrcMesh* m, int F, const int32_t* facets, const int32_t* facetElm) {
    if (F < 0) return -1;
    for (int f = 0; f < F; ++f) {
        const int e = facetElm[f];
        if (e < 0 || e >= m->E) return -1;
        for (int k = 0; k < m->dim; ++k) {
            const int v = facets[(size_t)k * F + f];
            bool in = false;
            for (int i = 0; i < m->npe; ++i) in |= m->node(e, i) == v;
            if (!in) return -1;
        }
    }
    m->F = F;
    m->facets.assign(facets, facets + (size_t)m->dim * F);
    m->facetElm.assign(facetElm, facetElm + F);
    return 0;
}

// The surface tension forces alone (dim x N, field-major), with the PSPG facet rule
// (any_node != 0) or the WC one, at the current positions.
void orc_surface_tension(const OrcMesh* m, double gamma, int any_node, double* out) {
    std::fill(out, out + (size_t)m->dim * m->N, 0.0);
    addSurfaceTension(*m, gamma, any_node != 0, out);
}

int orc_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void orc_get_positions(const OrcMesh* m, double* out) { std::copy(m->pos.begin(), m->pos.end(), out); }

void orc_set_positions(OrcMesh* m, const double* in) {
    std::copy(in, in + m->pos.size(), m->pos.begin());
    computeAllGeometry(*m);
}

void orc_get_is_free(const OrcMesh* m, uint8_t* out) { std::copy(m->isFree.begin(), m->isFree.end(), out); }

// Element geometry export: J (9 per element, row-major 3x3), detJ, invJ (9 per element).
void orc_get_geometry(const OrcMesh* m, double* J, double* detJ, double* invJ) {
    for (int e = 0; e < m->E; ++e) {
        const ElemGeom& g = m->geom[e];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                J[9 * e + 3 * r + c] = g.J[r][c];
                invJ[9 * e + 3 * r + c] = g.invJ[r][c];
            }
        detJ[e] = g.detJ;
    }
}

// Mesh::saveNodesList / restoreNodesList (positions), srcs/mesh/Mesh.cpp:1019-1053
void orc_save_nodes(OrcMesh* m) { m->posSave = m->pos; }

void orc_restore_nodes(OrcMesh* m) {
    m->pos = m->posSave;
    computeAllGeometry(*m);
}

// Mesh::updateNodesPositionFromSave(Eigen::VectorXd), srcs/mesh/Mesh.cpp:1238-1277
void orc_update_positions_from_save(OrcMesh* m, const double* delta) {
    const int N = m->N;
#pragma omp parallel for
    for (int n = 0; n < N; ++n)
        if (!m->fixed(n))
            for (int d = 0; d < m->dim; ++d)
                m->pos[(size_t)d * N + n] = m->posSave[(size_t)d * N + n] + delta[(size_t)d * N + n];
    computeAllGeometry(*m);
}

// Mesh::updateNodesPosition(Eigen::VectorXd), srcs/mesh/Mesh.cpp:1101-1137
void orc_update_positions(OrcMesh* m, const double* delta) {
    const int N = m->N;
#pragma omp parallel for
    for (int n = 0; n < N; ++n)
        if (!m->fixed(n))
            for (int d = 0; d < m->dim; ++d) m->pos[(size_t)d * N + n] += delta[(size_t)d * N + n];
    computeAllGeometry(*m);
}

// Element matrix/vector for one element (for known-answer tests).
void orc_pspg_element(const OrcMesh* m, int e, const PspgParams* p, const double* qIter, const double* qPrev,
                      double* Ae, double* be) {
    Mat A;
    pspgElement(*m, e, *p, qIter, qPrev, A, be);
    for (int i = 0; i < A.r; ++i)
        for (int j = 0; j < A.c; ++j) Ae[i * A.c + j] = A(i, j);
}

// m_buildAbPSPG (MomContEquationPSPG.inl:6-146) followed, when apply_bc != 0, by
// m_applyBCPSPG (:148-235; surface tension when p->gamma >= 1e-15).  vbc holds the Dirichlet
// velocity of every node (dim x N field-major; read only at Dirichlet nodes), standing in
// for the Lua BoundaryV(pos, t + dt) call.  Returns nnz of the compressed matrix.
int orc_pspg_assemble(OrcMesh* m, const PspgParams* p, const double* qIter, const double* qPrev, const double* vbc,
                      int apply_bc) {
    const int dim = m->dim, npe = m->npe, N = m->N, E = m->E;
    const int R = (dim + 1) * N;
    const size_t tripletPerElm = (size_t)(dim + 1) * npe * (dim + 1) * npe;
    const size_t doubletPerElm = (size_t)(dim + 1) * npe;
    // default-constructed Eigen::Triplet is (0, 0, 0.0): unassigned slots keep it (:17)
    std::vector<Triplet> indexA(tripletPerElm * E, Triplet{0, 0, 0.0});
    std::vector<std::pair<int32_t, double>> indexb(doubletPerElm * E);
    m->b.assign(R, 0.0);

#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
        Mat Ae;
        double be[16];
        pspgElement(*m, e, *p, qIter, qPrev, Ae, be);
        size_t countA = 0, countb = 0;
        for (int i = 0; i < npe; ++i) {
            const int ni = m->node(e, i);
            const bool skipV = m->bound(ni) || m->isFree[ni];
            for (int j = 0; j < npe; ++j) {
                const int nj = m->node(e, j);
                for (int d1 = 0; d1 < dim; ++d1)
                    for (int d2 = 0; d2 <= dim; ++d2) {
                        if (!skipV)
                            indexA[tripletPerElm * e + countA] =
                                Triplet{ni + d1 * N, nj + d2 * N, Ae(i + d1 * npe, j + d2 * npe)};
                        countA++;
                    }
                for (int d2 = 0; d2 <= dim; ++d2) {
                    if (!m->isFree[ni])
                        indexA[tripletPerElm * e + countA] =
                            Triplet{ni + dim * N, nj + d2 * N, Ae(i + dim * npe, j + d2 * npe)};
                    countA++;
                }
            }
            for (int d = 0; d <= dim; ++d) {
                indexb[doubletPerElm * e + countb] = {ni + d * N, be[i + d * npe]};
                countb++;
            }
        }
    }
    // identity rows of free and bound nodes (:108-128)
    for (int n = 0; n < N; ++n) {
        if (m->isFree[n]) indexA.push_back(Triplet{n + dim * N, n + dim * N, 1.0});
        if (m->bound(n) || m->isFree[n])
            for (int d = 0; d < dim; ++d) indexA.push_back(Triplet{n + d * N, n + d * N, 1.0});
    }
    // setFromTriplets (:136)
    setFromTriplets(*m, indexA, R);
    // RHS scatter in doublet order (:140-144)
    for (const auto& d : indexb) m->b[d.first] += d.second;

    if (apply_bc) {
        // m_applyBCPSPG facet loop (:155-187)
        addSurfaceTension(*m, p->gamma, true, m->b.data(), p->T, p->dgammaDT, p->Tr);
        // m_applyBCPSPG node loop (:189-232)
        for (int n = 0; n < N; ++n) {
            if (m->isFree[n]) {
                m->b[n + dim * N] = 0;
                if (!m->bound(n))
                    for (int d = 0; d < dim; ++d) m->b[n + d * N] = qPrev[n + (size_t)d * N] + p->dt * p->g[d];
            }
            if (m->dirichlet(n)) {
                for (int d = 0; d < dim; ++d) {
                    const double r = vbc[(size_t)d * N + n];
                    const int col = n + d * N;
                    m->b[col] = r;
                    for (int k = m->colptr[col]; k < m->colptr[col + 1]; ++k) {
                        if (m->rowidx[k] == col) continue;
                        m->b[m->rowidx[k]] -= m->vals[k] * r;
                        m->vals[k] = 0;
                    }
                }
            }
        }
    }
    return (int)m->vals.size();
}

// HeatEqIncompNewton::m_buildAb (HeatEquation.inl:226-305) and m_applyBC (:307-394) for one
// Picard pass from T_prev, with the node states Ts (the M factor with phase change, the facet
// temperatures of Qh / Qr; null: Ts = T_prev).  hf[n]: HT_T (Dirichlet T = Tbc[n]), HT_Q / HT_QH / HT_QR (flux,
// convection, radiation on the facets whose nodes all carry the flag; a free-surface facet
// uses p->fsFlags).  qgp[(f*3 + g)*dim + d]: the prescribed flux vector at Gauss point g of
// facet f (the "Q" BC function; read only for HT_Q facets, may be null otherwise).  The
// system is left in colptr/rowidx/vals/b (orc_pspg_get).  Returns nnz.
int orc_heat_assemble(OrcMesh* m, const HeatParams* p, double dt, const double* Tprev, const uint8_t* hf,
                      const double* Tbc, const double* qgp, const double* Ts) {
    const int dim = m->dim, npe = m->npe, N = m->N, E = m->E;
    if (!Ts) Ts = Tprev;
    const size_t tripletPerElm = (size_t)dim * npe * npe + (size_t)dim * npe * dim * npe + 3 * (size_t)npe * dim * npe +
                                 (size_t)npe * npe;
    // default-constructed triplets (0, 0, 0.0) stay in the unassigned slots (:232-233)
    std::vector<Triplet> indexA(tripletPerElm * E, Triplet{0, 0, 0.0});
    // doubletPerElm slots per element, of which the first npe*E are written (:236,:283); the
    // rest stay (0, 0.0)
    std::vector<std::pair<int32_t, double>> indexb((size_t)(2 * dim * npe + 2 * npe) * E, {0, 0.0});
    m->b.assign(N, 0.0);
#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
        Mat Me, Le;
        heatElement(*m, e, *p, dt, Ts, Me, Le);
        double th[4];
        for (int k = 0; k < npe; ++k) th[k] = Tprev[m->node(e, k)];
        size_t countA = 0;
        for (int i = 0; i < npe; ++i) {
            const int ni = m->node(e, i);
            for (int j = 0; j < npe; ++j) {
                if (!(hf[ni] & HT_T)) {
                    if (!m->isFree[ni]) indexA[tripletPerElm * e + countA] = Triplet{ni, m->node(e, j), Me(i, j)};
                    countA++;
                    if (!m->isFree[ni]) indexA[tripletPerElm * e + countA] = Triplet{ni, m->node(e, j), Le(i, j)};
                    countA++;
                }
            }
            double s = 0;
            for (int j = 0; j < npe; ++j) s += Me(i, j) * th[j];
            indexb[(size_t)npe * e + i] = {ni, s};
        }
    }
    for (int n = 0; n < N; ++n)
        if ((hf[n] & HT_T) || m->isFree[n]) indexA.push_back(Triplet{n, n, 1.0});
    setFromTriplets(*m, indexA, N);
    for (const auto& d : indexb) m->b[d.first] += d.second;

    // facet loop (:315-375)
    const FacetGauss fg = facetGauss(dim);
    constexpr double sigma = 5.670374419e-8;
    for (int f = 0; f < m->F; ++f) {
        int nd[3];
        bool fs = true;
        for (int k = 0; k < dim; ++k) {
            nd[k] = m->facets[(size_t)k * m->F + f];
            fs = fs && (m->flags[nd[k]] & FREE_SURFACE);
        }
        bool bq = true, bqh = true, bqr = true;
        for (int k = 0; k < dim; ++k) {
            const int fl = fs ? p->fsFlags : hf[nd[k]];
            bq = bq && (fl & HT_Q);
            bqh = bqh && (fl & HT_QH);
            bqr = bqr && (fl & HT_QR);
        }
        if (!bq && !bqh && !bqr) continue;
        double detJ, nrm[3];
        facetGeometry(*m, f, detJ, nrm);
        double tf[3];
        for (int k = 0; k < dim; ++k) tf[k] = Ts[nd[k]];
        if (bq) {  // getQN, MatricesBuilder.inl:246-272
            orientedNormal(*m, f, nrm);
            double qn[3] = {0, 0, 0};
            for (int g = 0; g < 3; ++g) {
                double qdn = 0;
                for (int d = 0; d < dim; ++d) qdn += qgp[((size_t)f * 3 + g) * dim + d] * nrm[d];
                const double fact = qdn * fg.w[g];
                for (int k = 0; k < dim; ++k) qn[k] += fact * fg.sf[g][k];
            }
            for (int k = 0; k < dim; ++k) m->b[nd[k]] -= dt * (qn[k] * fg.ref * detJ);
        }
        for (int pass = 0; pass < 2; ++pass) {  // getSGamma, MatricesBuilder.inl:357-370 (:82-94)
            if (!(pass == 0 ? bqh : bqr)) continue;
            double sg[3] = {0, 0, 0};
            for (int g = 0; g < 3; ++g) {
                double T = 0;
                for (int k = 0; k < dim; ++k) T += fg.sf[g][k] * tf[k];
                const double fac = pass == 0 ? p->h * (T - p->Tinf)
                                             : sigma * p->epsRad * (T * T * T * T - p->Tinf * p->Tinf * p->Tinf * p->Tinf);
                for (int k = 0; k < dim; ++k) sg[k] += fac * fg.sf[g][k] * fg.w[g];
            }
            for (int k = 0; k < dim; ++k) m->b[nd[k]] -= dt * (sg[k] * (detJ * fg.ref));
        }
    }
    // node loop (:377-393)
    for (int n = 0; n < N; ++n) {
        if (m->isFree[n] && !(hf[n] & HT_T)) {
            m->b[n] = Tprev[n];
        } else if (hf[n] & HT_T) {
            const double r = Tbc[n];
            m->b[n] = r;
            for (int k = m->colptr[n]; k < m->colptr[n + 1]; ++k) {
                if (m->rowidx[k] == n) continue;
                m->b[m->rowidx[k]] -= m->vals[k] * r;
                m->vals[k] = 0;
            }
        }
    }
    return (int)m->vals.size();
}

// Facet::getPosFromGP (Facet.cpp:227-237) at the three heat Gauss points of every facet:
// out[(f*3 + g)*dim + d].  In 2D the facet Jacobian is half the edge (Facet.cpp:31-32) and the
// Gauss points lie in [-1, 1], so the positions are those of the reference, centred on node 0.
void orc_facet_gauss_positions(const OrcMesh* m, double* out) {
    const int dim = m->dim;
    const FacetGauss fg = facetGauss(dim);
    for (int f = 0; f < m->F; ++f) {
        const int a = m->facets[f], b = m->facets[(size_t)m->F + f];
        const int c = dim == 3 ? m->facets[2 * (size_t)m->F + f] : a;
        for (int g = 0; g < 3; ++g)
            for (int d = 0; d < dim; ++d) {
                double J0 = m->x(b, d) - m->x(a, d), J1 = 0;
                if (dim == 2) J0 /= 2;
                else J1 = m->x(c, d) - m->x(a, d);
                out[((size_t)f * 3 + g) * dim + d] = J0 * fg.xi[g][0] + J1 * fg.xi[g][1] + m->x(a, d);
            }
    }
}

// ---------------------------------------------------------------------------------------
// Fractional step (solver "FracStep"), IncompNewton/MomContEquationFracStep.inl:7-630.
//
// One Picard iteration: MK_dt v~ = bV (velocity prediction), L p = bP (pressure), M dv = bVc
// (velocity correction), v = v~ + dv.  The pressure system of the reference is singular (L has
// the factor 1, MomContEquation.inl:157-161; every non-free node keeps its Laplacian row and
// free-surface nodes only lose their right-hand side, :266-300): here each connected group of
// elements gets a gauge node (its smallest free-surface node, else its smallest node) whose row
// and column are treated as those of a free node (:303-325), i.e. p = 0 there.
// ---------------------------------------------------------------------------------------
struct FsParams {
    double rho, mu, dt, gammaFS;
    double g[3];
    double gamma;  // surface tension of the prediction's right-hand side (:207-243)
};

namespace {

void fsColumnIdentity(OrcMesh::Csc& A, int col) {  // column col: diagonal 1, the rest 0
    for (int k = A.colptr[col]; k < A.colptr[col + 1]; ++k) A.vals[k] = A.rowidx[k] == col ? 1.0 : 0.0;
}

}  // namespace

// m_buildMatFracStep (:7-197) and m_applyBCVAppStep (:199-260) at the current positions, with
// the previous step's velocities vPrev (d x N) and pressures pPrev (N); vbc the Dirichlet
// velocities at t + dt; gauge[n] = 1 for the pressure gauge nodes.
void orc_fs_build(OrcMesh* m, const FsParams* p, const double* vPrev, const double* pPrev, const double* vbc,
                  const uint8_t* gauge) {
    const int dim = m->dim, npe = m->npe, N = m->N, E = m->E;
    const double dt = p->dt;
    const int tM = dim * npe * npe, tMK = dim * npe * npe + dim * npe * dim * npe, tL = npe * npe;
    std::vector<Triplet> iM((size_t)tM * E, Triplet{0, 0, 0.0}), iMK((size_t)tMK * E, Triplet{0, 0, 0.0}),
        iL((size_t)tL * E, Triplet{0, 0, 0.0});
    const int dbl = 3 * dim * npe;
    std::vector<std::pair<int32_t, double>> ib((size_t)dbl * E, {0, 0.0});
    m->fsDT.assign(E, {});
    m->fsLe.assign(E, {});
    auto rowSkip = [&](int n) { return m->bound(n) || m->isFree[n]; };
    auto lSkip = [&](int n) { return m->isFree[n] || (gauge && gauge[n]); };
#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
        const ElemGeom& geo = m->geom[e];
        Mat G = getGradN(dim, geo);
        Mat B = getB(dim, G);
        Mat Ms = getM(*m, geo, [&](int) { return p->rho; });
        double sumMu = 0, sumL = 0;
        for (int g = 0; g < m->gt.n; ++g) {
            sumMu += p->mu * m->gt.w[g];
            sumL += 1.0 * m->gt.w[g];
        }
        Mat K = getK(*m, geo, sumMu, B, ddevIncomp(dim));
        Mat D = getD(*m, geo, [](int) { return 1.0; }, B);  // npe x dim*npe
        Mat Le = getL(*m, geo, sumL, G);
        double Fe[12];
        getF(*m, geo, [&](int) { return p->rho; }, p->g, Fe);
        std::vector<double>& DT = m->fsDT[e];
        DT.assign((size_t)dim * npe * npe, 0.0);  // D^T, (dim*npe) x npe row-major
        for (int r = 0; r < dim * npe; ++r)
            for (int c = 0; c < npe; ++c) DT[(size_t)r * npe + c] = D(c, r);
        std::vector<double>& LE = m->fsLe[e];
        LE.assign((size_t)npe * npe, 0.0);
        for (int i = 0; i < npe; ++i)
            for (int j = 0; j < npe; ++j) LE[(size_t)i * npe + j] = Le(i, j);
        double vP[12], pP[4];
        for (int d = 0; d < dim; ++d)
            for (int k = 0; k < npe; ++k) vP[d * npe + k] = vPrev[(size_t)d * N + m->node(e, k)];
        for (int k = 0; k < npe; ++k) pP[k] = pPrev[m->node(e, k)];
        double MvDt[12], DTp[12];
        for (int d = 0; d < dim; ++d)
            for (int i = 0; i < npe; ++i) {
                double s = 0;
                for (int j = 0; j < npe; ++j) s += (Ms(i, j) * (1 / dt)) * vP[d * npe + j];
                MvDt[d * npe + i] = s;
            }
        for (int r = 0; r < dim * npe; ++r) {
            double s = 0;
            for (int c = 0; c < npe; ++c) s += DT[(size_t)r * npe + c] * pP[c];
            DTp[r] = p->gammaFS * s;
        }
        size_t cM = 0, cMK = 0, cL = 0, cb = 0;
        for (int i = 0; i < npe; ++i) {
            const int ni = m->node(e, i);
            for (int j = 0; j < npe; ++j) {
                const int nj = m->node(e, j);
                for (int d = 0; d < dim; ++d) {
                    if (!rowSkip(ni)) {
                        iM[(size_t)tM * e + cM] = Triplet{ni + d * N, nj + d * N, Ms(i, j)};
                        iMK[(size_t)tMK * e + cMK] = Triplet{ni + d * N, nj + d * N, Ms(i, j) * (1 / dt)};
                    }
                    cM++;
                    cMK++;
                    for (int d2 = 0; d2 < dim; ++d2) {
                        if (!rowSkip(ni))
                            iMK[(size_t)tMK * e + cMK] = Triplet{ni + d * N, nj + d2 * N, K(i + d * npe, j + d2 * npe)};
                        cMK++;
                    }
                }
                if (!lSkip(ni)) iL[(size_t)tL * e + cL] = Triplet{ni, nj, Le(i, j)};
                cL++;
            }
            for (int d = 0; d < dim; ++d)
                if (!rowSkip(ni)) {
                    ib[(size_t)dbl * e + cb++] = {ni + d * N, Fe[i + d * npe]};
                    ib[(size_t)dbl * e + cb++] = {ni + d * N, MvDt[i + d * npe]};
                    ib[(size_t)dbl * e + cb++] = {ni + d * N, DTp[i + d * npe]};
                }
        }
    }
    for (int n = 0; n < N; ++n) {
        if (lSkip(n)) iL.push_back(Triplet{n, n, 1.0});
        if (rowSkip(n))
            for (int d = 0; d < dim; ++d) {
                iMK.push_back(Triplet{n + d * N, n + d * N, 1.0});
                iM.push_back(Triplet{n + d * N, n + d * N, 1.0});
            }
    }
    toCsc(iM, dim * N, m->fsM.colptr, m->fsM.rowidx, m->fsM.vals);
    toCsc(iMK, dim * N, m->fsMK.colptr, m->fsMK.rowidx, m->fsMK.vals);
    toCsc(iL, N, m->fsL.colptr, m->fsL.rowidx, m->fsL.vals);
    m->fsbV.assign((size_t)dim * N, 0.0);
    for (const auto& d : ib) m->fsbV[d.first] += d.second;
    // m_applyBCVAppStep: surface tension of facets with a free-surface node, then the nodes
    addSurfaceTension(*m, p->gamma, true, m->fsbV.data());
    for (int n = 0; n < N; ++n) {
        if (m->isFree[n] && !m->bound(n))
            for (int d = 0; d < dim; ++d) m->fsbV[n + (size_t)d * N] = vPrev[(size_t)d * N + n] + dt * p->g[d];
        if (m->dirichlet(n))
            for (int d = 0; d < dim; ++d) {
                const int c = n + d * N;
                const double r = vbc[(size_t)d * N + n];
                m->fsbV[c] = r;
                for (int k = m->fsMK.colptr[c]; k < m->fsMK.colptr[c + 1]; ++k) {
                    if (m->fsMK.rowidx[k] == c) continue;
                    m->fsbV[m->fsMK.rowidx[k]] -= m->fsMK.vals[k] * r;
                    m->fsMK.vals[k] = 0;
                }
            }
    }
    // m_applyBCPCorrStep (:303-325) on L: free nodes (and the gauge nodes)
    for (int n = 0; n < N; ++n)
        if (lSkip(n)) fsColumnIdentity(m->fsL, n);
    // m_applyBCVStep (:389-413) on M: free and bound nodes
    for (int n = 0; n < N; ++n)
        if (rowSkip(n))
            for (int d = 0; d < dim; ++d) fsColumnIdentity(m->fsM, n + d * N);
}

// m_buildMatPcorrStep (:262-301) with m_applyBCPCorrStep's right-hand side: bP.
void orc_fs_pressure_rhs(OrcMesh* m, const FsParams* p, const double* vTilde, const double* pPrev,
                         const uint8_t* gauge) {
    const int dim = m->dim, npe = m->npe, N = m->N, E = m->E;
    std::vector<std::pair<int32_t, double>> ib((size_t)2 * npe * E, {0, 0.0});
#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
        const std::vector<double>& DT = m->fsDT[e];
        const std::vector<double>& LE = m->fsLe[e];
        double vt[12], pP[4];
        for (int d = 0; d < dim; ++d)
            for (int k = 0; k < npe; ++k) vt[d * npe + k] = vTilde[(size_t)d * N + m->node(e, k)];
        for (int k = 0; k < npe; ++k) pP[k] = pPrev[m->node(e, k)];
        size_t cb = 0;
        for (int i = 0; i < npe; ++i) {
            double dv = 0, lp = 0;
            for (int r = 0; r < dim * npe; ++r) dv += DT[(size_t)r * npe + i] * vt[r];
            for (int j = 0; j < npe; ++j) lp += LE[(size_t)i * npe + j] * pP[j];
            const int ni = m->node(e, i);
            if (!m->isFree[ni] && !(m->flags[ni] & FREE_SURFACE)) {
                ib[(size_t)2 * npe * e + cb++] = {ni, -((p->rho / p->dt) * dv)};
                ib[(size_t)2 * npe * e + cb++] = {ni, p->gammaFS * lp};
            }
        }
    }
    m->fsbP.assign(N, 0.0);
    for (const auto& d : ib) m->fsbP[d.first] += d.second;
    for (int n = 0; n < N; ++n)
        if (m->isFree[n] || (gauge && gauge[n])) m->fsbP[n] = 0;
}

// m_buildMatVStep (:327-387) with m_applyBCVStep's right-hand side: bVc from dp = p - gammaFS p_prev.
void orc_fs_velocity_rhs(OrcMesh* m, const FsParams* p, const double* dP) {
    const int dim = m->dim, npe = m->npe, N = m->N, E = m->E;
    std::vector<std::pair<int32_t, double>> ib((size_t)dim * npe * E, {0, 0.0});
#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
        const std::vector<double>& DT = m->fsDT[e];
        double dp[4];
        for (int k = 0; k < npe; ++k) dp[k] = dP[m->node(e, k)];
        size_t cb = 0;
        for (int i = 0; i < npe; ++i) {
            const int ni = m->node(e, i);
            if (m->isFree[ni] || m->bound(ni)) continue;
            for (int d = 0; d < dim; ++d) {
                double s = 0;
                for (int c = 0; c < npe; ++c) s += DT[(size_t)(i + d * npe) * npe + c] * dp[c];
                ib[(size_t)dim * npe * e + cb++] = {ni + d * N, p->dt * s};
            }
        }
    }
    m->fsbVc.assign((size_t)dim * N, 0.0);
    for (const auto& d : ib) m->fsbVc[d.first] += d.second;
    for (int n = 0; n < N; ++n)
        if (m->isFree[n] || m->bound(n))
            for (int d = 0; d < dim; ++d) m->fsbVc[n + (size_t)d * N] = 0;
}

// which: 0 = MK_dt / bV, 1 = L / bP, 2 = M / bVc.  Returns nnz (arrays may be null).
int orc_fs_get(const OrcMesh* m, int which, int32_t* colptr, int32_t* rowidx, double* vals, double* b) {
    const OrcMesh::Csc& A = which == 0 ? m->fsMK : which == 1 ? m->fsL : m->fsM;
    const std::vector<double>& rhs = which == 0 ? m->fsbV : which == 1 ? m->fsbP : m->fsbVc;
    if (colptr) std::copy(A.colptr.begin(), A.colptr.end(), colptr);
    if (rowidx) std::copy(A.rowidx.begin(), A.rowidx.end(), rowidx);
    if (vals) std::copy(A.vals.begin(), A.vals.end(), vals);
    if (b) std::copy(rhs.begin(), rhs.end(), b);
    return (int)A.vals.size();
}

void orc_pspg_get(const OrcMesh* m, int32_t* colptr, int32_t* rowidx, double* vals, double* b) {
    if (colptr) std::copy(m->colptr.begin(), m->colptr.end(), colptr);
    if (rowidx) std::copy(m->rowidx.begin(), m->rowidx.end(), rowidx);
    if (vals) std::copy(m->vals.begin(), m->vals.end(), vals);
    if (b) std::copy(m->b.begin(), m->b.end(), b);
}

// ---------------------------------------------------------------------------------------
// Weakly compressible explicit step (CDS_dpdt), SolverWCompNewton::m_solveWCompNewtonNoT
// srcs/simulation/physics/WCompNewton/Solver.cpp:236-276 without the remesh at :266-272.
// s = [v (d), p, rho, a (d)] field-major.  vbc: Dirichlet velocities (d x N).
// ---------------------------------------------------------------------------------------
}  // extern "C"

namespace {

// HeatEqWCompNewton::solve (HeatEquation.inl:137-158): explicit, lumped mass.  m_buildSystem
// (:263-317): Me = getM with the factor cv rho_g ((cv + dfl/dT(T_g) Lm) rho_g with phase
// change, :51-66), lumped; Le = getL with the factor k; FTot = -dt Le T + Me T, summed over the
// elements in element order.  m_applyBC (:160-261): the flux facets (Q, Qh, Qr; all facet nodes
// flagged, free-surface facets use fsFlags), then free nodes without a T condition keep T and
// T-Dirichlet nodes take Tbc.  T <- invM F.
void wcHeatExplicit(OrcMesh* m, const WcBqParams* b, double dt, const double* rho, double* T, const uint8_t* hf,
                    const double* Tbc, const double* qgp) {
    const int dim = m->dim, npe = m->npe, N = m->N, E = m->E;
    HeatParams hp{};
    hp.cv = b->cv;
    hp.Tm = b->Tm;
    hp.DT = b->DT;
    std::vector<double> MeL((size_t)E * npe), FTe((size_t)E * npe);
#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
        const ElemGeom& geo = m->geom[e];
        double te[4], re[4];
        for (int k = 0; k < npe; ++k) {
            te[k] = T[m->node(e, k)];
            re[k] = rho[m->node(e, k)];
        }
        Mat Me = getM(*m, geo, [&](int g) {
            const double r = nDot(m->gt, g, re, npe);
            if (!b->phaseChange) return b->cv * r;
            return (b->cv + dFlDT(hp, nDot(m->gt, g, te, npe)) * b->Lm) * r;
        });
        Mat G = getGradN(dim, geo);
        double ksum = 0;
        for (int g = 0; g < m->gt.n; ++g) ksum += b->k * m->gt.w[g];
        Mat Le = getL(*m, geo, ksum, G);
        for (int i = 0; i < npe; ++i) {
            double lumped = 0, lt = 0;
            for (int j = 0; j < npe; ++j) {
                lumped += Me(i, j);
                lt += Le(i, j) * te[j];
            }
            MeL[(size_t)e * npe + i] = lumped;
            FTe[(size_t)e * npe + i] = -dt * lt + lumped * te[i];
        }
    }
    std::vector<double> invM(N, 0.0), F(N, 0.0);
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < npe; ++i) {
            invM[m->node(e, i)] += MeL[(size_t)e * npe + i];
            F[m->node(e, i)] += FTe[(size_t)e * npe + i];
        }
    for (int n = 0; n < N; ++n) invM[n] = 1 / invM[n];
    const FacetGauss fg = facetGauss(dim);
    constexpr double sigma = 5.670374419e-8;
    for (int f = 0; f < m->F; ++f) {
        int nd[3];
        bool fs = true;
        for (int k = 0; k < dim; ++k) {
            nd[k] = m->facets[(size_t)k * m->F + f];
            fs = fs && (m->flags[nd[k]] & FREE_SURFACE);
        }
        bool bq = true, bqh = true, bqr = true;
        for (int k = 0; k < dim; ++k) {
            const int fl = fs ? b->fsFlags : hf[nd[k]];
            bq = bq && (fl & HT_Q);
            bqh = bqh && (fl & HT_QH);
            bqr = bqr && (fl & HT_QR);
        }
        if (!bq && !bqh && !bqr) continue;
        double detJ, nrm[3];
        facetGeometry(*m, f, detJ, nrm);
        double tf[3];
        for (int k = 0; k < dim; ++k) tf[k] = T[nd[k]];
        if (bq) {  // getQN, MatricesBuilder.inl:246-272
            orientedNormal(*m, f, nrm);
            double qn[3] = {0, 0, 0};
            for (int g = 0; g < 3; ++g) {
                double qdn = 0;
                for (int d = 0; d < dim; ++d) qdn += qgp[((size_t)f * 3 + g) * dim + d] * nrm[d];
                const double fact = qdn * fg.w[g];
                for (int k = 0; k < dim; ++k) qn[k] += fact * fg.sf[g][k];
            }
            for (int k = 0; k < dim; ++k) F[nd[k]] -= dt * (qn[k] * fg.ref * detJ);
        }
        for (int pass = 0; pass < 2; ++pass) {  // getSGamma (h, then radiation)
            if (!(pass == 0 ? bqh : bqr)) continue;
            double sg[3] = {0, 0, 0};
            for (int g = 0; g < 3; ++g) {
                double Tg = 0;
                for (int k = 0; k < dim; ++k) Tg += fg.sf[g][k] * tf[k];
                const double fac = pass == 0 ? b->h * (Tg - b->Tinf)
                                             : sigma * b->epsRad * (Tg * Tg * Tg * Tg - b->Tinf * b->Tinf * b->Tinf * b->Tinf);
                for (int k = 0; k < dim; ++k) sg[k] += fac * fg.sf[g][k] * fg.w[g];
            }
            for (int k = 0; k < dim; ++k) F[nd[k]] -= dt * (sg[k] * (detJ * fg.ref));
        }
    }
    for (int n = 0; n < N; ++n) {
        if (m->isFree[n] && !(hf[n] & HT_T)) {
            F[n] = T[n];
            invM[n] = 1;
        } else if (hf[n] & HT_T) {
            F[n] = Tbc[n];
            invM[n] = 1;
        }
    }
    for (int n = 0; n < N; ++n) T[n] = invM[n] * F[n];
}

// One explicit step of m_solveWCompNewtonNoT (Solver.cpp:236-276) or, with bq, of
// m_solveBoussinesqWC (:278-320: the heat equation between the half-step prediction and the
// continuity equation; the momentum body force rho_g (1 - alpha (T_g - Tr)), the Carman-Kozeny
// term and the temperature-dependent surface tension, MomEquation.inl:105-132).
void wcStep(OrcMesh* m, const WcParams* p, const WcBqParams* bq, double dt, double* s, const double* vbc,
            const uint8_t* hf, const double* Tbc, const double* qgp) {
    const int dim = m->dim, npe = m->npe, N = m->N, E = m->E;
    double* v = s;
    double* P = s + (size_t)dim * N;
    double* rho = s + (size_t)(dim + 1) * N;
    double* a = s + (size_t)(dim + 2) * N;
    double* Tn = bq ? s + (size_t)(2 * dim + 2) * N : nullptr;

    // CDS_rho: ContEqWCompNewton::preCompute -> m_buildF0 (ContEquation.inl:171-175,
    // 194-230) before the nodes move: F0 = sum_e getM(factor 1) rho_e, consistent mass.
    std::vector<double> F0rho;
    if (p->version == 1) {
        std::vector<double> F0e((size_t)E * npe);
#pragma omp parallel for
        for (int e = 0; e < E; ++e) {
            Mat Me = getM(*m, m->geom[e], [](int) { return 1.0; });
            for (int i = 0; i < npe; ++i) {
                double f = 0;
                for (int j = 0; j < npe; ++j) f += Me(i, j) * rho[m->node(e, j)];
                F0e[(size_t)e * npe + i] = f;
            }
        }
        F0rho.assign(N, 0.0);
        for (int e = 0; e < E; ++e)
            for (int i = 0; i < npe; ++i) F0rho[m->node(e, i)] += F0e[(size_t)e * npe + i];
    }

    // v1/2 = v + dt/2 a ; x += dt v1/2 (:249-253, Mesh.cpp:1101-1137)
    std::vector<double> delta((size_t)dim * N);
#pragma omp parallel for
    for (int n = 0; n < N; ++n)
        for (int d = 0; d < dim; ++d) {
            v[(size_t)d * N + n] = v[(size_t)d * N + n] + 0.5 * dt * a[(size_t)d * N + n];
            delta[(size_t)d * N + n] = v[(size_t)d * N + n] * dt;
        }
    orc_update_positions(m, delta.data());
    if (bq) wcHeatExplicit(m, bq, dt, rho, Tn, hf, Tbc, qgp);

    // ContEqWCompNewton::m_buildSystemdpdt (ContEquation.inl:353-413) for CDS_dpdt: the D factor
    // K0 + K0' p_g and the mass times p; m_buildSystem (:232-302) for CDS_drhodt: the D factor
    // rho_g and the mass times rho; for CDS_rho only the lumped mass (F0 is m_buildF0's).
    const int ver = p->version;
    double* U = ver == 0 ? P : rho;  // the unknown of the continuity equation
    std::vector<double> MeL((size_t)E * npe), F0e((size_t)E * npe);
#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
        const ElemGeom& geo = m->geom[e];
        Mat Me = getM(*m, geo, [](int) { return 1.0; });
        double Ue[4], Ve[12];
        for (int k = 0; k < npe; ++k) Ue[k] = U[m->node(e, k)];
        for (int f = 0; f < dim; ++f)
            for (int k = 0; k < npe; ++k) Ve[f * npe + k] = v[(size_t)f * N + m->node(e, k)];
        Mat D;
        if (ver != 1) {
            Mat G = getGradN(dim, geo);
            Mat B = getB(dim, G);
            D = ver == 0 ? getD(*m, geo, [&](int g) { return p->K0 + p->K0p * nDot(m->gt, g, Ue, npe); }, B)
                         : getD(*m, geo, [&](int g) { return nDot(m->gt, g, Ue, npe); }, B);
        }
        for (int i = 0; i < npe; ++i) {
            double lumped = 0;
            for (int j = 0; j < npe; ++j) lumped += Me(i, j);
            MeL[(size_t)e * npe + i] = lumped;
            if (ver == 1) continue;
            double dv = 0;
            for (int j = 0; j < dim * npe; ++j) dv += D(i, j) * Ve[j];
            double f = -dt * dv;
            if (p->meduri) {
                double mp = 0;
                for (int j = 0; j < npe; ++j) mp += Me(i, j) * Ue[j];
                f += mp;
            } else {
                f += lumped * Ue[i];
            }
            F0e[(size_t)e * npe + i] = f;
        }
    }
    std::vector<double> invM(N, 0.0), F0(N, 0.0);
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < npe; ++i) {
            invM[m->node(e, i)] += MeL[(size_t)e * npe + i];
            if (ver != 1) F0[m->node(e, i)] += F0e[(size_t)e * npe + i];
        }
    if (ver == 1) F0 = F0rho;
    for (int n = 0; n < N; ++n) invM[n] = 1 / invM[n];
    if (ver == 0) {
        // m_applyBCdpdt (:334-351)
        for (int n = 0; n < N; ++n)
            if (m->isFree[n]) {
                F0[n] = 0;
                invM[n] = 1;
            }
        // p = invM F0 ; rho from Tait-Murnaghan (:139-146, :319-332)
#pragma omp parallel for
        for (int n = 0; n < N; ++n) {
            P[n] = invM[n] * F0[n];
            rho[n] = std::pow((p->K0p / p->K0) * P[n] + 1, 1 / p->K0p) * p->rhoStar;
        }
    } else {
        // m_applyBC (:177-192): free and free-surface nodes take rho*
        for (int n = 0; n < N; ++n)
            if (m->isFree[n] || (m->flags[n] & FREE_SURFACE)) {
                F0[n] = p->rhoStar;
                invM[n] = 1;
            }
        // rho = invM F0 ; p from Tait-Murnaghan (:150-166, :305-317)
#pragma omp parallel for
        for (int n = 0; n < N; ++n) {
            rho[n] = invM[n] * F0[n];
            P[n] = (p->K0 / p->K0p) * (std::pow(rho[n] / p->rhoStar, p->K0p) - 1);
        }
    }

    // MomEqWCompNewton::m_buildSystem, MomEquation.inl:229-302
    Mat ddev = ddevWC(dim);
    std::vector<double> MeD((size_t)E * dim * npe), FT((size_t)E * dim * npe);
#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
        const ElemGeom& geo = m->geom[e];
        double Pe[4], Re[4], Ve[12];
        for (int k = 0; k < npe; ++k) {
            Pe[k] = P[m->node(e, k)];
            Re[k] = rho[m->node(e, k)];
        }
        for (int f = 0; f < dim; ++f)
            for (int k = 0; k < npe; ++k) Ve[f * npe + k] = v[(size_t)f * N + m->node(e, k)];
        Mat G = getGradN(dim, geo);
        Mat B = getB(dim, G);
        Mat Mt = getM(*m, geo, [&](int g) { return nDot(m->gt, g, Re, npe); });
        double sumMu = 0;
        for (int g = 0; g < m->gt.n; ++g) sumMu += p->mu * m->gt.w[g];
        Mat K = getK(*m, geo, sumMu, B, ddev);
        Mat D = getD(*m, geo, [](int) { return 1.0; }, B);
        double Fe[12], Te[4];
        if (bq)
            for (int k = 0; k < npe; ++k) Te[k] = Tn[m->node(e, k)];
        getF(*m, geo, [&](int g) {
            const double r = nDot(m->gt, g, Re, npe);
            return bq ? r * (1 - bq->alpha * (nDot(m->gt, g, Te, npe) - bq->Tr)) : r;
        }, p->g, Fe);
        Mat M2(npe, npe);
        const bool ck = bq && bq->phaseChange;
        if (ck)
            M2 = getM(*m, geo, [&](int g) {
                const double fl = flWC(bq->Tm, bq->DT, nDot(m->gt, g, Te, npe));
                return bq->C * (1 - fl) * (1 - fl) / (fl * fl * fl + bq->eps);
            });
        for (int r = 0; r < dim * npe; ++r) {
            int i = r % npe;
            double lumped = 0;  // diagBlock + lump: row sum of the scalar block
            for (int j = 0; j < npe; ++j) lumped += Mt(i, j);
            MeD[(size_t)e * dim * npe + r] = lumped;
            double kv = 0;
            for (int c = 0; c < dim * npe; ++c) kv += K(r, c) * Ve[c];
            double dp = 0;
            for (int j = 0; j < npe; ++j) dp += D(j, r) * Pe[j];
            double ft = -kv + dp + Fe[r];
            if (ck) {  // - diagBlock(M2) V (MomEquation.inl:271-276)
                const int d = r / npe;
                double m2v = 0;
                for (int j = 0; j < npe; ++j) m2v += M2(i, j) * Ve[d * npe + j];
                ft -= m2v;
            }
            FT[(size_t)e * dim * npe + r] = ft;
        }
    }
    std::vector<double> invMv((size_t)dim * N, 0.0), F((size_t)dim * N, 0.0);
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < npe; ++i)
            for (int d = 0; d < dim; ++d) {
                int n = m->node(e, i);
                invMv[n + (size_t)d * N] += MeD[(size_t)e * dim * npe + i + d * npe];
                F[n + (size_t)d * N] += FT[(size_t)e * dim * npe + i + d * npe];
            }
    for (size_t k = 0; k < invMv.size(); ++k) invMv[k] = 1 / invMv[k];
    // m_applyBC (:305-374): facet loop (:311-335), then the node loop
    if (bq)
        addSurfaceTension(*m, p->gamma, false, F.data(), Tn, bq->dgammaDT, bq->Tr);
    else
        addSurfaceTension(*m, p->gamma, false, F.data());
    for (int n = 0; n < N; ++n) {
        if (m->isFree[n] && !m->bound(n)) {
            for (int d = 0; d < dim; ++d) {
                F[n + (size_t)d * N] = p->g[d];
                invMv[n + (size_t)d * N] = 1;
            }
        } else if (m->dirichlet(n)) {
            for (int d = 0; d < dim; ++d) {
                F[n + (size_t)d * N] = vbc[(size_t)d * N + n];
                invMv[n + (size_t)d * N] = 1;
            }
        }
    }
    // a = invM F ; v = v1/2 + dt/2 a (:216-222)
#pragma omp parallel for
    for (int n = 0; n < N; ++n)
        for (int d = 0; d < dim; ++d) {
            size_t k = n + (size_t)d * N;
            double acc = invMv[k] * F[k];
            a[k] = acc;
            v[k] = v[k] + 0.5 * dt * acc;
        }
}

}  // namespace

extern "C" {

void orc_wc_step(OrcMesh* m, const WcParams* p, double dt, double* s, const double* vbc) {
    wcStep(m, p, nullptr, dt, s, vbc, nullptr, nullptr, nullptr);
}

// BoussinesqWC step: s = [v (d), p, rho, a (d), T] field-major; hf heat flags per node, Tbc
// the T-Dirichlet values at t + dt, qgp the Q flux at the facet Gauss points (or null).
void orc_wc_bq_step(OrcMesh* m, const WcParams* p, const WcBqParams* bq, double dt, double* s, const double* vbc,
                    const uint8_t* hf, const double* Tbc, const double* qgp) {
    wcStep(m, p, bq, dt, s, vbc, hf, Tbc, qgp);
}

double wc_next_dt_impl(const OrcMesh* m, const WcParams* p, const WcBqParams* bq, const double* s);

// SolverWCompNewton::computeNextDT, WCompNewton/Solver.cpp:192-234 (adaptDT = true).
double orc_wc_next_dt(const OrcMesh* m, const WcParams* p, const double* s) { return wc_next_dt_impl(m, p, nullptr, s); }

// BoussinesqWC: the diffusion parameter is max(mu / rho, k / (cv rho)) (:215-219).
double orc_wc_bq_next_dt(const OrcMesh* m, const WcParams* p, const WcBqParams* bq, const double* s) {
    return wc_next_dt_impl(m, p, bq, s);
}

double wc_next_dt_impl(const OrcMesh* m, const WcParams* p, const WcBqParams* bq, const double* s) {
    const int dim = m->dim, N = m->N, E = m->E, npe = m->npe;
    const double* v = s;
    const double* P = s + (size_t)dim * N;
    const double* rho = s + (size_t)(dim + 1) * N;
    double dt2 = std::numeric_limits<double>::max();
#pragma omp parallel for reduction(min : dt2)
    for (int e = 0; e < E; ++e) {
        // Element::getRin, Element.cpp:226-294
        double he;
        const ElemGeom& geo = m->geom[e];
        double size = geo.detJ * m->gt.refSize;
        auto dist = [&](int a, int b) {
            double s2 = 0;
            for (int d = 0; d < dim; ++d) {
                double t = m->x(a, d) - m->x(b, d);
                s2 += t * t;
            }
            return std::sqrt(s2);
        };
        int n0 = m->node(e, 0), n1 = m->node(e, 1), n2 = m->node(e, 2);
        if (dim == 2) {
            double sp = (dist(n0, n1) + dist(n1, n2) + dist(n0, n2)) / 2;
            he = 2 * (size / sp);
        } else {
            int n3 = m->node(e, 3);
            auto X = [&](int n, int d) { return m->x(n, d); };
            auto nrm = [&](int a0, int a1, int a2) {  // |(a1-a0) x (a2-a0)|
                double ux = X(a1, 0) - X(a0, 0), uy = X(a1, 1) - X(a0, 1), uz = X(a1, 2) - X(a0, 2);
                double wx = X(a2, 0) - X(a0, 0), wy = X(a2, 1) - X(a0, 1), wz = X(a2, 2) - X(a0, 2);
                double cx = uy * wz - uz * wy, cy = uz * wx - ux * wz, cz = ux * wy - uy * wx;
                return std::sqrt(cx * cx + cy * cy + cz * cz);
            };
            double sum = nrm(n0, n1, n2) + nrm(n0, n3, n2) + nrm(n0, n1, n3) + nrm(n3, n1, n2);
            he = 2 * (6 * size / sum);
        }
        double maxSq = 0;
        for (int k = 0; k < npe; ++k) {
            int n = m->node(e, k);
            double c2 = (p->K0 + p->K0p * P[n]) / rho[n];
            double u2 = 0;
            for (int d = 0; d < dim; ++d) u2 += v[(size_t)d * N + n] * v[(size_t)d * N + n];
            double alpha = p->mu / rho[n];
            if (bq) alpha = std::max(alpha, bq->k / (bq->cv * rho[n]));  // HeatEq::getDiffusionParam
            maxSq = std::max(std::max(u2, c2), maxSq);
            maxSq = std::max(maxSq, 4 * alpha * alpha / (he * he));
        }
        dt2 = std::min(dt2, p->sc * p->sc * he * he / maxSq);
    }
    return std::min(std::sqrt(dt2), p->maxDT);
}

// ProbIncompNewton::getGlobalWrittableData("mass"): sum of element sizes,
// IncompNewton/Problem.cpp:173-189
double orc_volume(const OrcMesh* m) {
    double s = 0;
    for (int e = 0; e < m->E; ++e) s += m->geom[e].detJ * m->gt.refSize;
    return s;
}

// ProbWCompNewton::getGlobalWrittableData("mass"), WCompNewton/Problem.cpp:216-244
double orc_wc_mass(const OrcMesh* m, const double* s) {
    const double* rho = s + (size_t)(m->dim + 1) * m->N;
    double mass = 0;
    for (int e = 0; e < m->E; ++e) {
        double mid = 0;
        for (int k = 0; k < m->npe; ++k) mid += rho[m->node(e, k)];
        mid /= (double)m->npe;
        mass += mid * m->geom[e].detJ * m->gt.refSize;
    }
    return mass;
}

// MinMaxExtractor::update, extractors/MinMaxExtractor.cpp:28-62
double orc_tip(const OrcMesh* m, int coord, int wantMax) {
    double v = wantMax ? 0.0 : std::numeric_limits<double>::max();
    for (int n = 0; n < m->N; ++n)
        if (!m->bound(n) && !m->isFree[n])
            v = wantMax ? std::max(v, m->x(n, coord)) : std::min(v, m->x(n, coord));
    return v;
}

}  // extern "C"
