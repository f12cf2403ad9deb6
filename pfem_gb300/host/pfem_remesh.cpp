// Host remesh in C++ (libpfemremesh.so): Mesh::remesh (srcs/mesh/Mesh.cpp:919-926) with a
// Delaunay triangulation of its own where the reference calls CGAL.
//
// Delaunay: incremental Bowyer-Watson insertion into a triangulation of the points and an
// enclosing simplex, points in biased randomised order (rounds of doubling size, each sorted
// along a Morton curve), point location by a stochastic visibility walk from the last new
// simplex.  The cavity of a point is the set of simplices whose open circumball contains it;
// with exact predicates it is star-shaped from the point and its boundary faces are never
// coplanar with it, so every new simplex has positive volume, co-spherical ties included.
// Every simplex whose circumradius is at most alpha h has a ball empty of the far enclosing
// vertices, so the alpha complex does not depend on them.  Large perturbed 3D clouds are
// triangulated in overlapping cells on several threads (interior_by_cells), which yields the
// same interior simplices.
//
// Predicates: orientation and in-sphere determinants in double precision with a conservative
// error bound (1e-12 of the sum of the absolute values of their terms); when the bound does not
// decide the sign, the determinant is evaluated exactly in floating-point expansions (the
// Two-Sum, Two-Product, Grow-Expansion and Scale-Expansion algorithms of Shewchuk, "Adaptive
// precision floating-point arithmetic and fast robust geometric predicates", 1997).
//
// The alpha shape, the node additions and deletions and the boundary smoothing restate the
// reference's rules (cited per function) exactly as the Python host remesh does, so that on the
// same perturbation both produce the same mesh.
#include "../../include/pfem_remesh.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <new>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

struct pfr_mesh {
    int dim = 0;
    int n = 0, e = 0, f = 0;
    std::vector<double> pos;       // dim x n
    std::vector<uint8_t> flags;    // n
    std::vector<int32_t> conn;     // (dim+1) x e
    std::vector<int32_t> facets;   // dim x f
    std::vector<int32_t> facet_elm, facet_out;
    std::vector<int32_t> origin;   // n x (dim+1)
};

namespace {

thread_local std::string g_err;

constexpr uint8_t BOUND = 1, FREE_SURFACE = 2;

struct Failure : std::runtime_error {
    int code;
    Failure(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ---------------------------------------------------------------------------------------
// Exact arithmetic: nonoverlapping expansions, components in increasing magnitude, no zeros.
// ---------------------------------------------------------------------------------------
struct Ex {
    std::vector<double> c;
};

inline void two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    const double bv = x - a;
    const double av = x - bv;
    y = (a - av) + (b - bv);
}

inline void two_prod(double a, double b, double& x, double& y) {
    x = a * b;
    y = std::fma(a, b, -x);
}

Ex ex_diff(double a, double b) {
    double x, y;
    two_sum(a, -b, x, y);
    Ex r;
    if (y != 0) r.c.push_back(y);
    if (x != 0) r.c.push_back(x);
    return r;
}

// Grow-Expansion: e + b
void ex_grow(const std::vector<double>& e, double b, std::vector<double>& h) {
    h.clear();
    double q = b;
    for (double ei : e) {
        double x, y;
        two_sum(q, ei, x, y);
        if (y != 0) h.push_back(y);
        q = x;
    }
    if (q != 0) h.push_back(q);
}

Ex operator+(const Ex& e, const Ex& f) {
    Ex h = e;
    std::vector<double> tmp;
    for (double fj : f.c) {
        ex_grow(h.c, fj, tmp);
        h.c.swap(tmp);
    }
    return h;
}

Ex operator-(const Ex& e) {
    Ex r = e;
    for (double& x : r.c) x = -x;
    return r;
}

Ex operator-(const Ex& e, const Ex& f) { return e + (-f); }

// Scale-Expansion: e * b
Ex ex_scale(const Ex& e, double b) {
    Ex h;
    if (e.c.empty() || b == 0) return h;
    double q, hh;
    two_prod(e.c[0], b, q, hh);
    if (hh != 0) h.c.push_back(hh);
    for (size_t i = 1; i < e.c.size(); ++i) {
        double T, t, s, hs, q2, hq;
        two_prod(e.c[i], b, T, t);
        two_sum(q, t, s, hs);
        if (hs != 0) h.c.push_back(hs);
        two_sum(T, s, q2, hq);
        if (hq != 0) h.c.push_back(hq);
        q = q2;
    }
    if (q != 0) h.c.push_back(q);
    return h;
}

Ex operator*(const Ex& e, const Ex& f) {
    Ex r;
    for (double fj : f.c) r = r + ex_scale(e, fj);
    return r;
}

int ex_sign(const Ex& e) { return e.c.empty() ? 0 : (e.c.back() > 0 ? 1 : -1); }

constexpr double FILTER = 1e-12;

// ---------------------------------------------------------------------------------------
// Predicates.  orient<D>(p): sign of det[p1 - p0; ...; pD - p0] (positive: the simplex is
// positively oriented).  insphere<D>(p, q): positive when q lies inside the circumsphere of the
// positively oriented simplex p.
// ---------------------------------------------------------------------------------------
template <int D>
int orient(const double* const* p);

template <>
int orient<2>(const double* const* p) {
    const double a0 = p[1][0] - p[0][0], a1 = p[1][1] - p[0][1];
    const double b0 = p[2][0] - p[0][0], b1 = p[2][1] - p[0][1];
    const double l = a0 * b1, r = a1 * b0;
    const double det = l - r, perm = std::fabs(l) + std::fabs(r);
    if (std::fabs(det) > FILTER * perm) return det > 0 ? 1 : -1;
    const Ex A0 = ex_diff(p[1][0], p[0][0]), A1 = ex_diff(p[1][1], p[0][1]);
    const Ex B0 = ex_diff(p[2][0], p[0][0]), B1 = ex_diff(p[2][1], p[0][1]);
    return ex_sign(A0 * B1 - A1 * B0);
}

template <class T>
T det3(const T (&m)[3][3]) {
    return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}

double perm3(const double (&m)[3][3]) {
    auto a = [&](int i, int j) { return std::fabs(m[i][j]); };
    return a(0, 0) * (a(1, 1) * a(2, 2) + a(1, 2) * a(2, 1)) + a(0, 1) * (a(1, 0) * a(2, 2) + a(1, 2) * a(2, 0)) +
           a(0, 2) * (a(1, 0) * a(2, 1) + a(1, 1) * a(2, 0));
}

template <>
int orient<3>(const double* const* p) {
    double m[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) m[r][c] = p[r + 1][c] - p[0][c];
    const double det = det3(m), perm = perm3(m);
    if (std::fabs(det) > FILTER * perm) return det > 0 ? 1 : -1;
    Ex X[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) X[r][c] = ex_diff(p[r + 1][c], p[0][c]);
    return ex_sign(det3(X));
}

template <int D>
int insphere(const double* const* p, const double* q);

// 2D: det [[r_k, |r_k|^2]]_k with r_k = p_k - q, positive inside for counterclockwise p.
template <>
int insphere<2>(const double* const* p, const double* q) {
    double r[3][2], l[3];
    for (int k = 0; k < 3; ++k) {
        r[k][0] = p[k][0] - q[0];
        r[k][1] = p[k][1] - q[1];
        l[k] = r[k][0] * r[k][0] + r[k][1] * r[k][1];
    }
    double det = 0, perm = 0;
    for (int k = 0; k < 3; ++k) {
        const int i = (k + 1) % 3, j = (k + 2) % 3;  // cyclic minor: sign +
        const double m = r[i][0] * r[j][1] - r[i][1] * r[j][0];
        det += l[k] * m;
        perm += l[k] * (std::fabs(r[i][0] * r[j][1]) + std::fabs(r[i][1] * r[j][0]));
    }
    if (std::fabs(det) > FILTER * perm) return det > 0 ? 1 : -1;
    Ex R[3][2], L[3];
    for (int k = 0; k < 3; ++k) {
        R[k][0] = ex_diff(p[k][0], q[0]);
        R[k][1] = ex_diff(p[k][1], q[1]);
        L[k] = R[k][0] * R[k][0] + R[k][1] * R[k][1];
    }
    Ex E;
    for (int k = 0; k < 3; ++k) {
        const int i = (k + 1) % 3, j = (k + 2) % 3;
        E = E + L[k] * (R[i][0] * R[j][1] - R[i][1] * R[j][0]);
    }
    return ex_sign(E);
}

// 3D: det [[r_k, |r_k|^2]]_k expanded along the lift column; for a positively oriented tet
// (det[p1-p0; p2-p0; p3-p0] > 0) the determinant is negative when q lies inside.
template <>
int insphere<3>(const double* const* p, const double* q) {
    // the same determinant from the 2x2 minors of the x, y columns (fewer products)
    const double ax = p[0][0] - q[0], ay = p[0][1] - q[1], az = p[0][2] - q[2];
    const double bx = p[1][0] - q[0], by = p[1][1] - q[1], bz = p[1][2] - q[2];
    const double cx = p[2][0] - q[0], cy = p[2][1] - q[1], cz = p[2][2] - q[2];
    const double dx = p[3][0] - q[0], dy = p[3][1] - q[1], dz = p[3][2] - q[2];
    const double axby = ax * by, bxay = bx * ay, bxcy = bx * cy, cxby = cx * by, cxdy = cx * dy, dxcy = dx * cy;
    const double dxay = dx * ay, axdy = ax * dy, axcy = ax * cy, cxay = cx * ay, bxdy = bx * dy, dxby = dx * by;
    const double ab = axby - bxay, bc = bxcy - cxby, cd = cxdy - dxcy, da = dxay - axdy, ac = axcy - cxay,
                 bd = bxdy - dxby;
    const double abc = az * bc - bz * ac + cz * ab, bcd = bz * cd - cz * bd + dz * bc;
    const double cda = cz * da + dz * ac + az * cd, dab = dz * ab + az * bd + bz * da;
    const double al = ax * ax + ay * ay + az * az, bl = bx * bx + by * by + bz * bz;
    const double cl = cx * cx + cy * cy + cz * cz, dl = dx * dx + dy * dy + dz * dz;
    const double det = (dl * abc - cl * dab) + (bl * cda - al * bcd);
    const double abp = std::fabs(axby) + std::fabs(bxay), bcp = std::fabs(bxcy) + std::fabs(cxby);
    const double cdp = std::fabs(cxdy) + std::fabs(dxcy), dap = std::fabs(dxay) + std::fabs(axdy);
    const double acp = std::fabs(axcy) + std::fabs(cxay), bdp = std::fabs(bxdy) + std::fabs(dxby);
    const double perm = dl * (std::fabs(az) * bcp + std::fabs(bz) * acp + std::fabs(cz) * abp) +
                        cl * (std::fabs(dz) * abp + std::fabs(az) * bdp + std::fabs(bz) * dap) +
                        bl * (std::fabs(cz) * dap + std::fabs(dz) * acp + std::fabs(az) * cdp) +
                        al * (std::fabs(bz) * cdp + std::fabs(cz) * bdp + std::fabs(dz) * bcp);
    if (std::fabs(det) > FILTER * perm) return det < 0 ? 1 : -1;
    Ex R[4][3], L[4];
    for (int k = 0; k < 4; ++k) {
        for (int c = 0; c < 3; ++c) R[k][c] = ex_diff(p[k][c], q[c]);
        L[k] = R[k][0] * R[k][0] + R[k][1] * R[k][1] + R[k][2] * R[k][2];
    }
    Ex E;
    for (int k = 0; k < 4; ++k) {
        Ex m[3][3];
        for (int i = 0, rr = 0; i < 4; ++i) {
            if (i == k) continue;
            for (int c = 0; c < 3; ++c) m[rr][c] = R[i][c];
            ++rr;
        }
        const Ex t = L[k] * det3(m);
        E = ((k + 3) & 1) ? E - t : E + t;
    }
    return -ex_sign(E);
}

// ---------------------------------------------------------------------------------------
// Delaunay triangulation
// ---------------------------------------------------------------------------------------
inline uint64_t mix64(uint64_t z) {  // the SplitMix64 output function
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// U(-1, 1) for counter `k`: the perturbation of coordinate c of point i is jitter_unit(i*dim+c)
inline double jitter_unit(uint64_t k) {
    const uint64_t z = mix64((k + 1) * 0x9E3779B97F4A7C15ull);
    return 2.0 * (double)(z >> 11) * 0x1.0p-53 - 1.0;
}

template <int D>
class Delaunay {
public:
    static constexpr int V = D + 1;
    static constexpr int S = 2 * V;  // per simplex in T_: V vertices, then the V neighbours

    // pts: n points, D doubles each (interleaved)
    explicit Delaunay(std::vector<double> pts) : P_(std::move(pts)) { n_ = (int)(P_.size() / D); }

    void build() {
        add_super();
        std::vector<int> order = insertion_order();
        for (int p : order) insert(p);
    }

    int n_points() const { return n_; }
    int slots() const { return (int)alive_.size(); }
    bool alive(int t) const { return alive_[t] != 0; }
    bool real(int t) const {
        if (!alive_[t]) return false;
        for (int i = 0; i < V; ++i)
            if (T_[(size_t)t * S + i] >= n_) return false;
        return true;
    }
    int vert(int t, int i) const { return T_[(size_t)t * S + i]; }
    int nbr(int t, int i) const { return T_[(size_t)t * S + V + i]; }

private:
    std::vector<double> P_;
    int n_ = 0;
    std::vector<int> T_;  // simplex t: vertices T_[t*S + i], neighbour opposite i T_[t*S + V + i]
    std::vector<uint8_t> alive_;
    std::vector<int> free_;
    std::vector<int> mark_;
    int stamp_ = 0;
    int last_ = 0;
    uint64_t rng_ = 0x2545F4914F6CDD1Dull;
    // per insertion
    std::vector<int> stack_, cav_;
    struct Bnd {
        int c, j, nb;
    };
    std::vector<Bnd> bnd_;
    std::vector<uint64_t> hkey_;
    std::vector<int> hval_, hstamp_;

    const double* pt(int i) const { return &P_[(size_t)i * D]; }

    int alloc() {
        int t;
        if (!free_.empty()) {
            t = free_.back();
            free_.pop_back();
        } else {
            t = (int)alive_.size();
            alive_.push_back(0);
            T_.resize(T_.size() + S);
            mark_.push_back(0);
        }
        alive_[t] = 1;
        return t;
    }

    void add_super() {
        double lo[D], hi[D];
        for (int c = 0; c < D; ++c) lo[c] = hi[c] = n_ ? P_[c] : 0.0;
        for (int i = 0; i < n_; ++i)
            for (int c = 0; c < D; ++c) {
                lo[c] = std::min(lo[c], P_[(size_t)i * D + c]);
                hi[c] = std::max(hi[c], P_[(size_t)i * D + c]);
            }
        double ctr[D], R = 0;
        for (int c = 0; c < D; ++c) {
            ctr[c] = 0.5 * (lo[c] + hi[c]);
            R = std::max(R, hi[c] - lo[c]);
        }
        R = std::max(R, 1.0);
        const double s = 30 * R;
        if constexpr (D == 2) {
            const double dirs[3][2] = {{0.0, 1.0}, {-0.8660254037844386, -0.5}, {0.8660254037844386, -0.5}};
            for (auto& d : dirs)
                for (int c = 0; c < 2; ++c) P_.push_back(ctr[c] + s * d[c]);
        } else {
            const double dirs[4][3] = {{1, 1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
            for (auto& d : dirs)
                for (int c = 0; c < 3; ++c) P_.push_back(ctr[c] + s * d[c]);
        }
        const int t = alloc();
        for (int i = 0; i < V; ++i) {
            T_[(size_t)t * S + i] = n_ + i;
            T_[(size_t)t * S + V + i] = -1;
        }
        const double* q[V];
        for (int i = 0; i < V; ++i) q[i] = pt(n_ + i);
        if (orient<D>(q) < 0) std::swap(T_[(size_t)t * S + D - 1], T_[(size_t)t * S + D]);
        last_ = t;
    }

    std::vector<int> insertion_order() {
        std::vector<int> order(n_);
        std::iota(order.begin(), order.end(), 0);
        uint64_t s = 0x853C49E6748FEA9Bull;
        for (int i = n_ - 1; i > 0; --i) {  // Fisher-Yates with SplitMix64
            s += 0x9E3779B97F4A7C15ull;
            const int j = (int)(mix64(s) % (uint64_t)(i + 1));
            std::swap(order[i], order[j]);
        }
        // Morton codes
        double lo[D], hi[D];
        for (int c = 0; c < D; ++c) lo[c] = hi[c] = n_ ? P_[c] : 0.0;
        for (int i = 0; i < n_; ++i)
            for (int c = 0; c < D; ++c) {
                lo[c] = std::min(lo[c], P_[(size_t)i * D + c]);
                hi[c] = std::max(hi[c], P_[(size_t)i * D + c]);
            }
        constexpr int B = D == 2 ? 31 : 21;
        std::vector<uint64_t> code(n_);
        for (int i = 0; i < n_; ++i) {
            uint64_t m = 0;
            uint64_t q[D];
            for (int c = 0; c < D; ++c) {
                const double w = hi[c] > lo[c] ? (P_[(size_t)i * D + c] - lo[c]) / (hi[c] - lo[c]) : 0.0;
                q[c] = (uint64_t)std::min(std::max(w, 0.0) * (double)((1ull << B) - 1), (double)((1ull << B) - 1));
            }
            for (int b = B - 1; b >= 0; --b)
                for (int c = 0; c < D; ++c) m = (m << 1) | ((q[c] >> b) & 1u);
            code[i] = m;
        }
        // rounds [0, n/2^k), ..., [n/4, n/2), [n/2, n), each sorted along the curve
        std::vector<size_t> bounds;
        size_t b = (size_t)n_;
        while (b > 64) {
            bounds.push_back(b);
            b >>= 1;
        }
        bounds.push_back(b);
        bounds.push_back(0);
        std::reverse(bounds.begin(), bounds.end());
        for (size_t r = 0; r + 1 < bounds.size(); ++r)
            std::sort(order.begin() + bounds[r], order.begin() + bounds[r + 1],
                      [&](int a, int c) { return code[a] < code[c] || (code[a] == code[c] && a < c); });
        return order;
    }

    uint64_t next_rand() {
        rng_ += 0x9E3779B97F4A7C15ull;
        return mix64(rng_);
    }

    int locate(int p) {
        int t = last_;
        const double* q[V];
        for (long steps = 0;; ++steps) {
            if (steps > 64L * (long)alive_.size() + 1024) throw Failure(PFR_ERR_INTERNAL, "point location did not end");
            const int off = (int)(next_rand() % V);
            bool moved = false;
            for (int k = 0; k < V; ++k) {
                const int j = (off + k) % V;
                for (int i = 0; i < V; ++i) q[i] = pt(T_[(size_t)t * S + i]);
                q[j] = pt(p);
                if (orient<D>(q) < 0) {
                    const int nb = T_[(size_t)t * S + V + j];
                    if (nb < 0) throw Failure(PFR_ERR_INTERNAL, "point location left the enclosing simplex");
                    t = nb;
                    moved = true;
                    break;
                }
            }
            if (!moved) return t;
        }
    }

    bool in_conflict(int t, int p) const {
        const double* q[V];
        for (int i = 0; i < V; ++i) q[i] = pt(T_[(size_t)t * S + i]);
        return insphere<D>(q, pt(p)) > 0;
    }

    void insert(int p) {
        const int t0 = locate(p);
        for (int i = 0; i < V; ++i) {  // a duplicate of a vertex stays out of the triangulation
            const double* a = pt(T_[(size_t)t0 * S + i]);
            bool same = true;
            for (int c = 0; c < D; ++c) same = same && a[c] == pt(p)[c];
            if (same) return;
        }
        // stamps: 2s = in the cavity, 2s+1 = tested outside
        ++stamp_;
        const int in = 2 * stamp_, out = 2 * stamp_ + 1;
        stack_.clear();
        cav_.clear();
        bnd_.clear();
        stack_.push_back(t0);
        mark_[t0] = in;
        while (!stack_.empty()) {
            const int c = stack_.back();
            stack_.pop_back();
            cav_.push_back(c);
            for (int j = 0; j < V; ++j) {
                const int nb = T_[(size_t)c * S + V + j];
                if (nb < 0) {
                    bnd_.push_back({c, j, -1});
                    continue;
                }
                if (mark_[nb] == in) continue;
                if (mark_[nb] != out && in_conflict(nb, p)) {
                    mark_[nb] = in;
                    stack_.push_back(nb);
                } else {
                    mark_[nb] = out;
                    bnd_.push_back({c, j, nb});
                }
            }
        }
        // ridge table: each new simplex's faces through p, keyed by their other D-1 vertices
        size_t hs = 16;
        while (hs < 4 * bnd_.size() * D) hs <<= 1;
        if (hkey_.size() < hs) {
            hkey_.assign(hs, 0);
            hval_.assign(hs, 0);
            hstamp_.assign(hs, 0);
        }
        const size_t hmask = hs - 1;
        for (const Bnd& b : bnd_) {
            const int nt = alloc();
            mark_[nt] = 0;
            for (int i = 0; i < V; ++i) T_[(size_t)nt * S + i] = T_[(size_t)b.c * S + i];
            T_[(size_t)nt * S + b.j] = p;
            T_[(size_t)nt * S + V + b.j] = b.nb;
            if (b.nb >= 0)
                for (int i = 0; i < V; ++i)
                    if (T_[(size_t)b.nb * S + V + i] == b.c) {
                        T_[(size_t)b.nb * S + V + i] = nt;
                        break;
                    }
            for (int k = 0; k < V; ++k) {
                if (k == b.j) continue;
                uint64_t key;
                if constexpr (D == 2) {
                    const int o = 3 - k - b.j;
                    key = (uint64_t)(uint32_t)T_[(size_t)nt * S + o] + 1;
                } else {
                    int r[2], m = 0;
                    for (int i = 0; i < 4; ++i)
                        if (i != k && i != b.j) r[m++] = T_[(size_t)nt * S + i];
                    const uint32_t lo = (uint32_t)std::min(r[0], r[1]), hi = (uint32_t)std::max(r[0], r[1]);
                    key = (((uint64_t)hi << 32) | lo) + 1;
                }
                size_t h = (size_t)(mix64(key) & hmask);
                while (true) {
                    if (hstamp_[h] != stamp_) {
                        hstamp_[h] = stamp_;
                        hkey_[h] = key;
                        hval_[h] = nt * S + V + k;
                        break;
                    }
                    if (hkey_[h] == key) {
                        const int o = hval_[h];
                        T_[(size_t)nt * S + V + k] = o / S;
                        T_[o] = nt;
                        hkey_[h] = ~0ull;  // matched: a ridge joins exactly two new faces
                        break;
                    }
                    h = (h + 1) & hmask;
                }
            }
            last_ = nt;
        }
        for (int c : cav_) {
            alive_[c] = 0;
            free_.push_back(c);
        }
    }
};

// ---------------------------------------------------------------------------------------
// Small dense helpers on D x D systems
// ---------------------------------------------------------------------------------------
template <int D>
double det_rows(const double (&A)[D][D]) {
    if constexpr (D == 2)
        return A[0][0] * A[1][1] - A[0][1] * A[1][0];
    else
        return det3(A);
}

// Squared circumradius of a simplex from its edge vectors A (rows x_k - x_0): the centre c
// solves A c = |A_k|^2 / 2; flat simplices (|det A| <= 1e-12 (sum A^2)^(D/2)) get +inf.
template <int D>
double circumradius2(const double (&A)[D][D]) {
    double rhs[D], ss = 0;
    for (int k = 0; k < D; ++k) {
        double s = 0;
        for (int c = 0; c < D; ++c) s += A[k][c] * A[k][c];
        rhs[k] = 0.5 * s;
        ss += s;
    }
    const double det = det_rows<D>(A);
    if (!(std::fabs(det) > 1e-12 * std::pow(ss, D / 2.0))) return INFINITY;
    double c[D];
    for (int col = 0; col < D; ++col) {  // Cramer's rule
        double M[D][D];
        for (int r = 0; r < D; ++r)
            for (int cc = 0; cc < D; ++cc) M[r][cc] = cc == col ? rhs[r] : A[r][cc];
        c[col] = det_rows<D>(M) / det;
    }
    double r2 = 0;
    for (int k = 0; k < D; ++k) r2 += c[k] * c[k];
    return r2;
}

// Basic solution of the square system A x = b by Householder QR with column pivoting, the way
// the reference's colPivHouseholderQr().solve treats a rank-deficient A (Mesh.cpp:630,681): the
// pivots after the remaining columns' squared norms fall below (max column norm * eps)^2 (n-k)/n
// are dropped, their unknowns set to 0, the rest solved by back substitution.  The operations
// and their order are those of the Python host remesh's qr_basic_solve.
template <int D>
void qr_basic_solve(double (&A)[D][D], double (&b)[D], double (&x)[D]) {
    int perm[D];
    double norms[D];
    for (int j = 0; j < D; ++j) {
        perm[j] = j;
        double s = 0.0;
        for (int i = 0; i < D; ++i) s += A[i][j] * A[i][j];
        norms[j] = s;
    }
    double mx = 0.0;
    for (int j = 0; j < D; ++j) mx = std::max(mx, std::sqrt(norms[j]));
    const double e = mx * 2.220446049250313e-16;
    const double thresh = e * e / D;
    int nz = D;
    for (int k = 0; k < D; ++k) {
        int jb = k;
        for (int j = k + 1; j < D; ++j)
            if (norms[j] > norms[jb]) jb = j;
        if (nz == D && norms[jb] < thresh * (D - k)) nz = k;
        if (jb != k) {
            for (int i = 0; i < D; ++i) std::swap(A[i][k], A[i][jb]);
            std::swap(perm[k], perm[jb]);
            std::swap(norms[k], norms[jb]);
        }
        const double alpha = A[k][k];
        double sigma = 0.0;
        for (int i = k + 1; i < D; ++i) sigma += A[i][k] * A[i][k];
        if (sigma != 0.0) {
            const double nrm = std::sqrt(alpha * alpha + sigma);
            const double beta = alpha >= 0 ? -nrm : nrm;
            double v[D] = {};
            v[k] = 1.0;
            for (int i = k + 1; i < D; ++i) v[i] = A[i][k] / (alpha - beta);
            const double tau = (beta - alpha) / beta;
            for (int j = k + 1; j < D; ++j) {
                double w = A[k][j];
                for (int i = k + 1; i < D; ++i) w += v[i] * A[i][j];
                w *= tau;
                A[k][j] -= w;
                for (int i = k + 1; i < D; ++i) A[i][j] -= w * v[i];
            }
            double w = b[k];
            for (int i = k + 1; i < D; ++i) w += v[i] * b[i];
            w *= tau;
            b[k] -= w;
            for (int i = k + 1; i < D; ++i) b[i] -= w * v[i];
            A[k][k] = beta;
            for (int i = k + 1; i < D; ++i) A[i][k] = 0.0;
        }
        for (int j = k + 1; j < D; ++j) {
            double s = 0.0;
            for (int i = k + 1; i < D; ++i) s += A[i][j] * A[i][j];
            norms[j] = s;
        }
    }
    double c[D] = {};
    for (int k = nz - 1; k >= 0; --k) {
        double s = b[k];
        for (int j = k + 1; j < nz; ++j) s -= A[k][j] * c[j];
        c[k] = s / A[k][k];
    }
    for (int k = 0; k < D; ++k) x[k] = 0.0;
    for (int k = 0; k < nz; ++k) x[perm[k]] = c[k];
}

// Number of contiguous ranges parallel_ranges splits [0, n) into: up to 16, of 4096 items or more.
inline int range_count(int n) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    return (int)std::max<long long>(1, std::min<long long>(std::min<unsigned>(hw, 16u), n / 4096));
}

// Runs f(t, begin, end) for each of the range_count(n) contiguous ranges t of [0, n), one thread
// per range.
template <class F>
void parallel_ranges(int n, F&& f) {
    const int T = range_count(n);
    if (T <= 1) {
        f(0, 0, n);
        return;
    }
    // an exception in a worker is carried to this thread and rethrown after the joins
    std::vector<std::exception_ptr> err(T);
    auto run = [&](int t) {
        try {
            f(t, (int)((long long)n * t / T), (int)((long long)n * (t + 1) / T));
        } catch (...) {
            err[t] = std::current_exception();
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < T; ++t) th.emplace_back(run, t);
    run(0);
    for (auto& x : th) x.join();
    for (auto& e : err)
        if (e) std::rethrow_exception(e);
}

// Sorted distinct neighbours of each node (nodes sharing an element with it), CSR: the
// node-element incidence by a counting sort, then each range of nodes gathers its lists once
// into its own buffer (a repeated node is dropped by a per-node stamp) and sorts each list on its
// own; the buffers are concatenated in node order, so the lists do not depend on the thread count.
void neighbours(int N, int npe, int E, const int32_t* conn, std::vector<int>& ptr, std::vector<int>& idx) {
    std::vector<int> ep(N + 1, 0);
    for (int a = 0; a < npe; ++a)
        for (int e = 0; e < E; ++e) ++ep[conn[(size_t)a * E + e] + 1];
    for (int i = 0; i < N; ++i) ep[i + 1] += ep[i];
    std::vector<int> el(ep[N]), fill(ep.begin(), ep.end() - 1);
    for (int e = 0; e < E; ++e)
        for (int a = 0; a < npe; ++a) el[fill[conn[(size_t)a * E + e]]++] = e;
    std::vector<std::vector<int>> part(range_count(N));
    std::vector<int> cnt(N + 1, 0);
    parallel_ranges(N, [&](int t, int b, int e) {
        std::vector<int> seen(N, -1);  // seen[m] == n: m is already in node n's list
        std::vector<int>& out = part[t];
        for (int n = b; n < e; ++n) {
            const size_t s0 = out.size();
            seen[n] = n;
            for (int k = ep[n]; k < ep[n + 1]; ++k) {
                const int el_k = el[k];
                for (int a = 0; a < npe; ++a) {
                    const int m = conn[(size_t)a * E + el_k];
                    if (seen[m] != n) {
                        seen[m] = n;
                        out.push_back(m);
                    }
                }
            }
            std::sort(out.begin() + s0, out.end());
            cnt[n + 1] = (int)(out.size() - s0);
        }
    });
    ptr.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) ptr[i + 1] = ptr[i] + cnt[i + 1];
    idx.assign(ptr[N], 0);
    parallel_ranges(N, [&](int t, int b, int) { std::copy(part[t].begin(), part[t].end(), idx.begin() + ptr[b]); });
}

// ---------------------------------------------------------------------------------------
// Alpha shape (Mesh::triangulateAlphaShape2D/3D)
// ---------------------------------------------------------------------------------------
// vertex order of the face opposite vertex l of a positively oriented tet, as CGAL's
// vertex_triple_index orders it
constexpr int TRIPLE[4][3] = {{1, 3, 2}, {0, 2, 3}, {0, 3, 1}, {0, 1, 2}};

// Interior simplices of a large 3D cloud from independent triangulations of cells, in parallel.
//
// The perturbed points are split into K0 x K1 cells (K0 = round(sqrt K), K1 = floor(K / K0)) by
// quantiles, K0 slabs along the longest axis, each cut into K1 along the second longest (every
// point of space in exactly one cell's core box, half-open).  Each cell triangulates the points
// of its core box widened by a margin m >= 4 alpha h on those axes.  A tetrahedron is taken from
// the cell holding its centroid (computed from its vertices in ascending index, so every cell
// computes the same value), when it is interior.  This is the global alpha complex, with the
// interior flag of the neighbour across each face, under two conditions checked per cell:
//  * an interior tetrahedron of the global triangulation has its vertices within 2 alpha h of
//    its centroid, so a cell holds all of them and, its circumsphere being empty of every point,
//    the tetrahedron is in the cell's triangulation (which is unique for points in general
//    position); and a taken tetrahedron whose circumsphere lies inside the widened box is empty
//    of every point, so it is in the global triangulation;
//  * the neighbour across a face of a taken tetrahedron: if it is interior in the global
//    triangulation its vertices lie within 4 alpha h of the centroid and it is the cell's
//    neighbour too; if the cell's neighbour is interior with its circumsphere inside the widened
//    box it is the global one.
// A taken tetrahedron, or an interior neighbour of one, whose circumsphere leaves the widened box
// (a nearly flat tetrahedron of the perturbed points) voids the result: the caller then
// triangulates serially.  Cells run on up to 16 threads; their results are concatenated in cell
// order, so the output does not depend on the thread count.
bool interior_by_cells(const pfr_params& prm, int N, const double* pos, const std::vector<double>& pts, int K,
                       std::vector<int>& simp, std::vector<double>& vol, std::vector<uint8_t>& nbint) {
    constexpr int D = 3, V = 4;
    const double h = prm.hchar;
    const double alpha2 = (prm.alpha * h) * (prm.alpha * h);
    const double margin = 4.5 * prm.alpha * h + 10 * prm.jitter * h;
    double lo[D], hi[D];
    for (int c = 0; c < D; ++c) lo[c] = hi[c] = pts[c];
    for (int i = 0; i < N; ++i)
        for (int c = 0; c < D; ++c) {
            lo[c] = std::min(lo[c], pts[(size_t)i * D + c]);
            hi[c] = std::max(hi[c], pts[(size_t)i * D + c]);
        }
    int ax[D] = {0, 1, 2};
    std::sort(ax, ax + D, [&](int a, int b) { return hi[a] - lo[a] > hi[b] - lo[b] || (hi[a] - lo[a] == hi[b] - lo[b] && a < b); });
    const int a0 = ax[0], a1 = ax[1];
    int K0 = std::max(1, (int)std::lround(std::sqrt((double)K)));
    const int K1 = std::max(1, K / K0);
    struct Cell {
        double lo0, hi0, lo1, hi1;
    };
    std::vector<Cell> cells;
    std::vector<int> ord(N);
    std::iota(ord.begin(), ord.end(), 0);
    auto by = [&](int a) {
        return [&pts, a](int p, int q) {
            const double x = pts[(size_t)p * 3 + a], y = pts[(size_t)q * 3 + a];
            return x < y || (x == y && p < q);
        };
    };
    std::sort(ord.begin(), ord.end(), by(a0));
    for (int g = 0; g < K0; ++g) {
        const int b = (int)((long long)N * g / K0), e = (int)((long long)N * (g + 1) / K0);
        if (b >= e) continue;
        const double l0 = g == 0 ? -INFINITY : pts[(size_t)ord[b] * 3 + a0];
        const double h0 = g == K0 - 1 ? INFINITY : pts[(size_t)ord[e] * 3 + a0];
        std::vector<int> sub(ord.begin() + b, ord.begin() + e);
        std::sort(sub.begin(), sub.end(), by(a1));
        const int M = (int)sub.size();
        for (int k = 0; k < K1; ++k) {
            const int bb = (int)((long long)M * k / K1), ee = (int)((long long)M * (k + 1) / K1);
            if (bb >= ee) continue;
            const double l1 = k == 0 ? -INFINITY : pts[(size_t)sub[bb] * 3 + a1];
            const double h1 = k == K1 - 1 ? INFINITY : pts[(size_t)sub[ee] * 3 + a1];
            cells.push_back({l0, h0, l1, h1});
        }
    }
    const int C = (int)cells.size();
    struct Out {
        std::vector<int> simp;
        std::vector<double> vol;
        std::vector<uint8_t> nbint;
        bool ok = true;
        std::exception_ptr err;
    };
    std::vector<Out> outs(C);
    std::atomic<int> next{0};
    auto work = [&]() {
        for (int ci = next++; ci < C; ci = next++) try {
            const Cell& cl = cells[ci];
            Out& o = outs[ci];
            const double w0 = cl.lo0 - margin, W0 = cl.hi0 + margin, w1 = cl.lo1 - margin, W1 = cl.hi1 + margin;
            std::vector<int> gid;
            for (int i = 0; i < N; ++i) {
                const double x0 = pts[(size_t)i * 3 + a0], x1 = pts[(size_t)i * 3 + a1];
                if (x0 >= w0 && x0 < W0 && x1 >= w1 && x1 < W1) gid.push_back(i);
            }
            std::vector<double> lp(gid.size() * 3);
            for (size_t k = 0; k < gid.size(); ++k)
                for (int c = 0; c < 3; ++c) lp[k * 3 + c] = pts[(size_t)gid[k] * 3 + c];
            Delaunay<3> dt(std::move(lp));
            dt.build();
            const int S = dt.slots();
            // per slot, evaluated only for the simplices taken here and their neighbours: bit 0
            // evaluated, bit 1 interior (true positions), bit 2 its perturbed circumsphere lies in
            // the widened box
            std::vector<uint8_t> st(S, 0);
            auto eval = [&](int t) -> uint8_t {
                if (st[t]) return st[t];
                uint8_t r = 1;
                int v[V];
                for (int i = 0; i < V; ++i) v[i] = gid[dt.vert(t, i)];
                double A[D][D];
                for (int k = 0; k < D; ++k)
                    for (int c = 0; c < D; ++c) A[k][c] = pos[(size_t)c * N + v[k + 1]] - pos[(size_t)c * N + v[0]];
                const double m = std::fabs(det_rows<D>(A));
                if (circumradius2<D>(A) <= alpha2 && m > 0.0) {
                    r |= 2;
                    double B[D][D], rhs[D], ss = 0;
                    for (int k = 0; k < D; ++k) {
                        double sk = 0;
                        for (int c = 0; c < D; ++c) {
                            B[k][c] = pts[(size_t)v[k + 1] * 3 + c] - pts[(size_t)v[0] * 3 + c];
                            sk += B[k][c] * B[k][c];
                        }
                        rhs[k] = 0.5 * sk;
                        ss += sk;
                    }
                    const double det = det_rows<D>(B);
                    if (std::fabs(det) > 1e-12 * std::pow(ss, 1.5)) {  // else not inside
                        double cen[D];
                        for (int col = 0; col < D; ++col) {
                            double Mx[D][D];
                            for (int rr = 0; rr < D; ++rr)
                                for (int cc = 0; cc < D; ++cc) Mx[rr][cc] = cc == col ? rhs[rr] : B[rr][cc];
                            cen[col] = det_rows<D>(Mx) / det;
                        }
                        const double rad = std::sqrt(cen[0] * cen[0] + cen[1] * cen[1] + cen[2] * cen[2]) * (1 + 1e-9);
                        const double c0 = pts[(size_t)v[0] * 3 + a0] + cen[a0], c1 = pts[(size_t)v[0] * 3 + a1] + cen[a1];
                        if (c0 - rad > w0 && c0 + rad < W0 && c1 - rad > w1 && c1 + rad < W1) r |= 4;
                    }
                }
                return st[t] = r;
            };
            for (int t = 0; t < S && o.ok; ++t) {
                if (!dt.real(t)) continue;
                int v[V], sv[V];
                for (int i = 0; i < V; ++i) sv[i] = v[i] = gid[dt.vert(t, i)];
                std::sort(sv, sv + V);
                double ce0 = 0, ce1 = 0;
                for (int i = 0; i < V; ++i) {
                    ce0 += pts[(size_t)sv[i] * 3 + a0];
                    ce1 += pts[(size_t)sv[i] * 3 + a1];
                }
                ce0 *= 0.25;
                ce1 *= 0.25;
                if (!(ce0 >= cl.lo0 && ce0 < cl.hi0 && ce1 >= cl.lo1 && ce1 < cl.hi1)) continue;
                const uint8_t et = eval(t);
                if (!(et & 2)) continue;
                if (!(et & 4)) {
                    o.ok = false;
                    break;
                }
                uint8_t nbi[V];
                for (int l = 0; l < V; ++l) {
                    const int u = dt.nbr(t, l);
                    const uint8_t eu = u >= 0 && dt.real(u) ? eval(u) : 0;
                    nbi[l] = (eu & 2) != 0;
                    if (nbi[l] && !(eu & 4)) o.ok = false;
                }
                double A[D][D];
                for (int k = 0; k < D; ++k)
                    for (int c = 0; c < D; ++c) A[k][c] = pos[(size_t)c * N + v[k + 1]] - pos[(size_t)c * N + v[0]];
                double m = det_rows<D>(A);
                if (m < 0) {  // positive orientation on the true positions
                    std::swap(v[D - 1], v[D]);
                    std::swap(nbi[D - 1], nbi[D]);
                    m = -m;
                }
                for (int i = 0; i < V; ++i) {
                    o.simp.push_back(v[i]);
                    o.nbint.push_back(nbi[i]);
                }
                o.vol.push_back(m);
            }
        } catch (...) {  // carried to the calling thread
            outs[ci].err = std::current_exception();
        }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int T = (int)std::min<unsigned>(std::min<unsigned>(hw, 16u), (unsigned)C);
    std::vector<std::thread> th;
    for (int i = 1; i < T; ++i) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
    for (const Out& o : outs)
        if (o.err) std::rethrow_exception(o.err);
    simp.clear();
    vol.clear();
    nbint.clear();
    for (const Out& o : outs) {
        if (!o.ok) return false;
        simp.insert(simp.end(), o.simp.begin(), o.simp.end());
        vol.insert(vol.end(), o.vol.begin(), o.vol.end());
        nbint.insert(nbint.end(), o.nbint.begin(), o.nbint.end());
    }
    return true;
}

template <int D>
void alpha_shape(const pfr_params& prm, int N, const double* pos, const uint8_t* flags_in, pfr_mesh& out,
                 std::vector<int32_t>& node_origin) {
    constexpr int V = D + 1;
    const double h = prm.hchar;
    std::vector<double> pts((size_t)N * D);
    for (int i = 0; i < N; ++i)
        for (int c = 0; c < D; ++c) {
            double x = pos[(size_t)c * N + i];
            if (prm.jitter != 0) x += jitter_unit((uint64_t)i * D + c) * (prm.jitter * h);
            pts[(size_t)i * D + c] = x;
        }
    std::vector<int> simp;
    std::vector<double> vol;
    std::vector<uint8_t> interior, nbint;  // nbint: the neighbour across face l is interior
    int ns = 0;
    // large perturbed 3D clouds: interior simplices from cells triangulated in parallel (K fixed
    // by the node count, so the result does not depend on the machine); serially otherwise, or
    // when a cell's conditions fail
    const int K = std::min(16, N / 8192);
    bool by_cells = false;
    if constexpr (D == 3) {
        if (!prm.single_triangulation && prm.jitter > 0 && K >= 2 &&
            interior_by_cells(prm, N, pos, pts, K, simp, vol, nbint)) {
            by_cells = true;
            ns = (int)vol.size();
            interior.assign(ns, 1);
        }
    }
    if (!by_cells) {
    Delaunay<D> dt(std::move(pts));
    dt.build();

    // the simplices of the points (none with an enclosing vertex), in slot order
    const int S = dt.slots();
    std::vector<int> sid(S, -1);
    std::vector<int> nb;
    for (int t = 0; t < S; ++t)
        if (dt.real(t)) sid[t] = ns++;
    simp.resize((size_t)ns * V);
    nb.resize((size_t)ns * V);
    vol.resize(ns);
    interior.resize(ns);
    const double alpha2 = (prm.alpha * h) * (prm.alpha * h);
    for (int t = 0; t < S; ++t) {
        const int s = sid[t];
        if (s < 0) continue;
        int v[V], n[V];
        for (int i = 0; i < V; ++i) {
            v[i] = dt.vert(t, i);
            const int o = dt.nbr(t, i);
            n[i] = o >= 0 ? sid[o] : -1;
        }
        double A[D][D];
        for (int k = 0; k < D; ++k)
            for (int c = 0; c < D; ++c) A[k][c] = pos[(size_t)c * N + v[k + 1]] - pos[(size_t)c * N + v[0]];
        double m = det_rows<D>(A);
        if (m < 0) {  // positive orientation on the true positions: swap the last two vertices
            std::swap(v[D - 1], v[D]);
            std::swap(n[D - 1], n[D]);
            for (int c = 0; c < D; ++c) std::swap(A[D - 2][c], A[D - 1][c]);
            m = -m;
        }
        for (int i = 0; i < V; ++i) {
            simp[(size_t)s * V + i] = v[i];
            nb[(size_t)s * V + i] = n[i];
        }
        vol[s] = m;
        interior[s] = circumradius2<D>(A) <= alpha2 && m > 0.0;
    }
    nbint.resize((size_t)ns * V);
    for (int s = 0; s < ns; ++s)
        for (int l = 0; l < V; ++l) {
            const int o = nb[(size_t)s * V + l];
            nbint[(size_t)s * V + l] = o >= 0 && interior[o];
        }
    }
    std::vector<uint8_t> bound(N), wet(N, 0);
    for (int i = 0; i < N; ++i) bound[i] = (flags_in[i] & BOUND) != 0;
    std::vector<uint8_t> allbound(ns);
    for (int s = 0; s < ns; ++s) {
        bool ab = true;
        for (int i = 0; i < V; ++i) ab = ab && bound[simp[(size_t)s * V + i]];
        allbound[s] = ab;
        if (interior[s] && !ab)  // checkFaceDeletion: a node wetted by an interior simplex
            for (int i = 0; i < V; ++i) wet[simp[(size_t)s * V + i]] = 1;
    }
    std::vector<uint8_t> keep(ns);
    std::vector<int> eidx(ns, -1);
    int E = 0;
    for (int s = 0; s < ns; ++s) {
        bool anywet = false;
        for (int i = 0; i < V; ++i) anywet = anywet || wet[simp[(size_t)s * V + i]];
        bool del = interior[s] && allbound[s] && !anywet;
        if constexpr (D == 3) del = del || (interior[s] && allbound[s] && vol[s] / 6.0 < 0.02 * h * h * h);
        keep[s] = interior[s] && !del;
        if (keep[s]) eidx[s] = E++;
    }
    std::vector<int32_t> conn((size_t)V * E);
    for (int s = 0; s < ns; ++s)
        if (keep[s])
            for (int i = 0; i < V; ++i) conn[(size_t)i * E + eidx[s]] = simp[(size_t)s * V + i];
    // facets: regular faces of the alpha complex whose interior simplex was kept
    std::vector<int32_t> fv, felm, fout;
    for (int s = 0; s < ns; ++s) {
        if (!interior[s]) continue;
        for (int l = 0; l < V; ++l) {
            if (nbint[(size_t)s * V + l]) continue;
            if (!keep[s]) continue;
            const int* v = &simp[(size_t)s * V];
            if constexpr (D == 2) {
                fv.push_back(v[(l + 1) % 3]);
                fv.push_back(v[(l + 2) % 3]);
            } else {
                for (int k = 0; k < 3; ++k) fv.push_back(v[TRIPLE[l][k]]);
            }
            felm.push_back(eidx[s]);
            fout.push_back(v[l]);
        }
    }
    const int F = (int)felm.size();
    std::vector<uint8_t> flags(flags_in, flags_in + N);
    for (auto& f : flags) f &= (uint8_t)~FREE_SURFACE;
    for (int f = 0; f < F; ++f) {
        bool fb = true;
        for (int k = 0; k < D; ++k) fb = fb && bound[fv[(size_t)f * D + k]];
        if (!fb)
            for (int k = 0; k < D; ++k) flags[fv[(size_t)f * D + k]] |= FREE_SURFACE;
    }
    // flying nodes (Mesh::deleteFlyingNodes): in no element and not bound
    std::vector<int> remap(N);
    std::iota(remap.begin(), remap.end(), 0);
    node_origin.resize(N);
    std::iota(node_origin.begin(), node_origin.end(), 0);
    int Nn = N;
    if (prm.delete_flying_nodes) {
        std::vector<uint8_t> used(N, 0);
        for (int32_t x : conn) used[x] = 1;
        node_origin.clear();
        Nn = 0;
        for (int i = 0; i < N; ++i) {
            if (!used[i] && !bound[i]) {
                remap[i] = -1;
                continue;
            }
            remap[i] = Nn++;
            node_origin.push_back(i);
        }
    }
    out.dim = D;
    out.n = Nn;
    out.e = E;
    out.f = F;
    out.pos.resize((size_t)D * Nn);
    out.flags.resize(Nn);
    for (int k = 0; k < Nn; ++k) {
        const int i = node_origin[k];
        for (int c = 0; c < D; ++c) out.pos[(size_t)c * Nn + k] = pos[(size_t)c * N + i];
        out.flags[k] = flags[i];
    }
    out.conn.resize((size_t)V * E);
    for (size_t k = 0; k < conn.size(); ++k) out.conn[k] = remap[conn[k]];
    out.facets.resize((size_t)D * F);
    for (int f = 0; f < F; ++f)
        for (int k = 0; k < D; ++k) out.facets[(size_t)k * F + f] = remap[fv[(size_t)f * D + k]];
    out.facet_elm = felm;
    out.facet_out.resize(F);
    for (int f = 0; f < F; ++f) out.facet_out[f] = remap[fout[f]];
}

// ---------------------------------------------------------------------------------------
// Remesh steps before the triangulation
// ---------------------------------------------------------------------------------------
// Mesh::laplacianSmoothingBoundaries (Mesh.cpp:580-760): for every element with exactly D bound
// nodes, the non-bound node closer than h/3 to the wall facet is pushed h/3 along the facet
// normal (free-surface node) or moved to the mean of its neighbours.  Elements are visited in
// order and see earlier moves.
template <int D>
void smooth_boundaries(int N, int E, const int32_t* conn, const uint8_t* flags, double h, const std::vector<int>& ip,
                       const std::vector<int>& ix, std::vector<double>& pos) {
    constexpr int V = D + 1;
    auto X = [&](int c, int n) -> double& { return pos[(size_t)c * N + n]; };
    for (int e = 0; e < E; ++e) {
        int nb = 0, out = -1, fac[D];
        for (int a = 0; a < V; ++a) {
            const int n = conn[(size_t)a * E + e];
            if (flags[n] & BOUND) {
                if (nb < D) fac[nb] = n;
                ++nb;
            } else if (out < 0) {
                out = n;
            }
        }
        if (nb != D) continue;
        double P[D][D];
        for (int k = 0; k < D; ++k)
            for (int c = 0; c < D; ++c) P[k][c] = X(c, fac[k]);
        double normal[D] = {};
        double dist;
        bool axis = false;
        if constexpr (D == 2) {
            if (P[0][0] == P[1][0]) {
                normal[0] = 1;
                dist = std::fabs(P[0][0] - X(0, out));
                axis = true;
            } else if (P[0][1] == P[1][1]) {
                normal[1] = 1;
                dist = std::fabs(P[0][1] - X(1, out));
                axis = true;
            }
        } else {
            if (P[0][0] == P[1][0] && P[1][0] == P[2][0]) {
                normal[0] = 1;
                dist = std::fabs(P[0][0] - X(0, out));
                axis = true;
            } else if (P[0][1] == P[1][1] && P[1][1] == P[2][1]) {
                normal[1] = 1;
                dist = std::fabs(P[0][1] - X(1, out));
                axis = true;
            } else if (P[0][2] == P[1][2] && P[1][1] == P[2][2]) {  // the reference compares y with z here
                normal[2] = 1;
                dist = std::fabs(P[0][2] - X(2, out));
                axis = true;
            }
        }
        if (!axis) {  // the plane n . x = -1 through the facet nodes
            double M[D][D], b[D];
            for (int k = 0; k < D; ++k) {
                for (int c = 0; c < D; ++c) M[k][c] = P[k][c];
                b[k] = -1.0;
            }
            qr_basic_solve<D>(M, b, normal);
            double dot = 0.0, nn = 0.0;
            for (int c = 0; c < D; ++c) {
                dot += normal[c] * X(c, out);
                nn += normal[c] * normal[c];
            }
            dist = std::fabs(dot + 1) / std::sqrt(nn);
        }
        if (dist > h / 3) continue;
        if (flags[out] & FREE_SURFACE) {
            if constexpr (D == 2) {  // the sign with the raw normal, then normalised (Mesh.cpp:697-715)
                const double side = normal[0] * (X(0, out) - P[0][0]) + normal[1] * (X(1, out) - P[0][1]);
                if (side < 0) {
                    normal[0] = -normal[0];
                    normal[1] = -normal[1];
                }
                const double nn = std::sqrt(normal[0] * normal[0] + normal[1] * normal[1]);
                normal[0] = normal[0] / nn;
                normal[1] = normal[1] / nn;
            } else {  // normalised, then the sign (:716-734)
                const double nn = std::sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
                for (int c = 0; c < 3; ++c) normal[c] = normal[c] / nn;
                const double side = (X(0, out) - P[0][0]) * normal[0] + (X(1, out) - P[0][1]) * normal[1] +
                                    (X(2, out) - P[0][2]) * normal[2];
                if (side < 0)
                    for (int c = 0; c < 3; ++c) normal[c] = -normal[c];
            }
            for (int c = 0; c < D; ++c) X(c, out) += h / 3 * normal[c];
        } else {  // the mean of the neighbours, summed in order (:737-756)
            const int k0 = ip[out], k1 = ip[out + 1];
            for (int c = 0; c < D; ++c) {
                double acc = 0.0;
                for (int k = k0; k < k1; ++k) acc += X(c, ix[k]);
                X(c, out) = acc / (double)(k1 - k0);
            }
        }
    }
}

template <int D>
double simplex_size(const std::vector<double>& pos, int N, const int32_t* conn, int E, int e) {
    double A[D][D];
    for (int k = 0; k < D; ++k)
        for (int c = 0; c < D; ++c)
            A[k][c] = pos[(size_t)c * N + conn[(size_t)(k + 1) * E + e]] - pos[(size_t)c * N + conn[e]];
    return det_rows<D>(A) * (D == 2 ? 0.5 : 1.0 / 6.0);
}

template <int D>
void remesh_impl(const pfr_params& prm, int N, const double* pos_in, const uint8_t* flags_in, int E,
                 const int32_t* conn, pfr_mesh& out) {
    constexpr int V = D + 1;
    const double h = prm.hchar;
    for (size_t k = 0; k < (size_t)V * E; ++k)
        if (conn[k] < 0 || conn[k] >= N) throw Failure(PFR_ERR_INVALID, "connectivity index out of range");
    std::vector<double> pos(pos_in, pos_in + (size_t)D * N);
    std::vector<int> ip, ix;
    neighbours(N, V, E, conn, ip, ix);
    if (prm.laplacian_smoothing_boundaries) smooth_boundaries<D>(N, E, conn, flags_in, h, ip, ix, pos);

    // addNodes (Mesh.cpp:27-147): a node at the centroid of every element larger than
    // omega h^d, skipping elements with a free-surface node unless addOnFS
    std::vector<int> grow;
    const double hd = D == 2 ? h * h : h * h * h;
    for (int e = 0; e < E; ++e) {
        if (!(simplex_size<D>(pos, N, conn, E, e) > prm.omega * hd)) continue;
        if (!prm.add_on_fs) {
            bool on_fs = false;
            for (int a = 0; a < V; ++a) on_fs = on_fs || (flags_in[conn[(size_t)a * E + e]] & FREE_SURFACE);
            if (on_fs) continue;
        }
        grow.push_back(e);
    }
    const int N2 = N + (int)grow.size();
    std::vector<double> pos2((size_t)D * N2);
    std::vector<uint8_t> flags2(N2, 0);
    std::vector<int32_t> origin((size_t)N2 * V, -1);
    for (int c = 0; c < D; ++c)
        for (int i = 0; i < N; ++i) pos2[(size_t)c * N2 + i] = pos[(size_t)c * N + i];
    for (int i = 0; i < N; ++i) {
        flags2[i] = flags_in[i];
        origin[(size_t)i * V] = i;
    }
    for (size_t g = 0; g < grow.size(); ++g) {
        const int e = grow[g], n = N + (int)g;
        for (int c = 0; c < D; ++c) {
            double s = pos[(size_t)c * N + conn[e]];
            for (int a = 1; a < V; ++a) s += pos[(size_t)c * N + conn[(size_t)a * E + e]];
            pos2[(size_t)c * N2 + n] = s / (double)V;
        }
        for (int a = 0; a < V; ++a) origin[(size_t)n * V + a] = conn[(size_t)a * E + e];
    }

    // removeNodes (Mesh.cpp:928-1017): of two nodes closer than gamma h (half that when both are
    // on the free surface), one is deleted, never a bound node; nodes in no element are skipped
    std::vector<uint8_t> keep(N2, 1), used(N, 0), touched(N, 0), del(N, 0);
    for (size_t k = 0; k < (size_t)V * E; ++k) used[conn[k]] = 1;
    const double limit = prm.gamma * h;
    std::vector<uint8_t> close(ix.size());
    std::vector<uint8_t> any_close(N, 0);
    for (int i = 0; i < N; ++i)
        for (int k = ip[i]; k < ip[i + 1]; ++k) {
            const int j = ix[k];
            double s = 0;
            for (int c = 0; c < D; ++c) {
                const double d = pos2[(size_t)c * N2 + i] - pos2[(size_t)c * N2 + j];
                s += d * d;
            }
            const bool bothfs = (flags_in[i] & FREE_SURFACE) && (flags_in[j] & FREE_SURFACE);
            close[k] = std::sqrt(s) <= (bothfs ? 0.5 : 1.0) * limit;
            if (close[k]) any_close[i] = 1;
        }
    for (int i = 0; i < N; ++i) {
        if (!any_close[i] || del[i] || !used[i]) continue;
        const bool bi = flags_in[i] & BOUND, fi = flags_in[i] & FREE_SURFACE;
        for (int k = ip[i]; k < ip[i + 1]; ++k) {
            if (!close[k]) continue;
            const int j = ix[k];
            const bool bj = flags_in[j] & BOUND, fj = flags_in[j] & FREE_SURFACE;
            if (touched[j]) {
                if (bi || (fi && !fj)) continue;
                del[i] = 1;
            } else {
                if (bj || (fj && !fi)) continue;
                touched[i] = 1;
                del[j] = 1;
            }
        }
    }
    for (int i = 0; i < N; ++i) keep[i] = !del[i];
    // checkBoundingBox (Mesh.cpp:149-207)
    if (prm.has_bounding_box)
        for (int i = 0; i < N2; ++i)
            for (int c = 0; c < D; ++c) {
                const double x = pos2[(size_t)c * N2 + i];
                if (!(x >= prm.bounding_box[c] && x <= prm.bounding_box[D + c])) keep[i] = 0;
            }
    std::vector<int> idx;
    for (int i = 0; i < N2; ++i)
        if (keep[i]) idx.push_back(i);
    const int M = (int)idx.size();
    std::vector<double> pos3((size_t)D * M);
    std::vector<uint8_t> flags3(M);
    for (int k = 0; k < M; ++k) {
        for (int c = 0; c < D; ++c) pos3[(size_t)c * M + k] = pos2[(size_t)c * N2 + idx[k]];
        flags3[k] = flags2[idx[k]];
    }
    std::vector<int32_t> node_origin;
    alpha_shape<D>(prm, M, pos3.data(), flags3.data(), out, node_origin);
    out.origin.resize((size_t)out.n * V);
    for (int k = 0; k < out.n; ++k)
        for (int a = 0; a < V; ++a) out.origin[(size_t)k * V + a] = origin[(size_t)idx[node_origin[k]] * V + a];
}

int check_params(const pfr_params* p) {
    if (!p || (p->dim != 2 && p->dim != 3)) return PFR_ERR_INVALID;
    if (!(p->hchar > 0) || !(p->alpha > 0) || !(p->jitter >= 0) || !std::isfinite(p->jitter)) return PFR_ERR_INVALID;
    return PFR_OK;
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return PFR_OK;
    } catch (const Failure& e) {
        g_err = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_err = "out of host memory";
        return PFR_ERR_NOMEM;
    } catch (const std::exception& e) {
        g_err = e.what();
        return PFR_ERR_INTERNAL;
    }
}

}  // namespace

extern "C" {

PFR_API int pfr_default_params(int32_t dim, double hchar, pfr_params* p) {
    if (!p || (dim != 2 && dim != 3) || !(hchar > 0)) return PFR_ERR_INVALID;
    std::memset(p, 0, sizeof(*p));
    p->dim = dim;
    p->add_on_fs = 0;
    p->delete_flying_nodes = 1;
    p->laplacian_smoothing_boundaries = 1;
    p->hchar = hchar;
    p->alpha = 1.2;
    p->omega = 0.7;
    p->gamma = 0.2;
    p->jitter = dim == 3 ? 1e-6 : 0.0;
    return PFR_OK;
}

PFR_API int pfr_remesh(const pfr_params* p, int32_t n_nodes, const double* pos, const uint8_t* flags,
                       int32_t n_elems, const int32_t* conn, pfr_mesh** out) {
    if (out) *out = nullptr;
    int rc = check_params(p);
    if (rc || n_nodes < 0 || n_elems < 0 || !out || (n_nodes && (!pos || !flags)) || (n_elems && !conn)) {
        g_err = "pfr_remesh: bad arguments";
        return PFR_ERR_INVALID;
    }
    pfr_mesh* m = new (std::nothrow) pfr_mesh();
    if (!m) return PFR_ERR_NOMEM;
    rc = guarded([&] {
        if (p->dim == 2)
            remesh_impl<2>(*p, n_nodes, pos, flags, n_elems, conn, *m);
        else
            remesh_impl<3>(*p, n_nodes, pos, flags, n_elems, conn, *m);
    });
    if (rc) {
        delete m;
        return rc;
    }
    *out = m;
    return PFR_OK;
}

PFR_API int pfr_alpha_shape(const pfr_params* p, int32_t n_nodes, const double* pos, const uint8_t* flags,
                            pfr_mesh** out) {
    if (out) *out = nullptr;
    int rc = check_params(p);
    if (rc || n_nodes < 0 || !out || (n_nodes && (!pos || !flags))) {
        g_err = "pfr_alpha_shape: bad arguments";
        return PFR_ERR_INVALID;
    }
    pfr_mesh* m = new (std::nothrow) pfr_mesh();
    if (!m) return PFR_ERR_NOMEM;
    rc = guarded([&] {
        std::vector<int32_t> node_origin;
        if (p->dim == 2)
            alpha_shape<2>(*p, n_nodes, pos, flags, *m, node_origin);
        else
            alpha_shape<3>(*p, n_nodes, pos, flags, *m, node_origin);
        const int V = p->dim + 1;
        m->origin.assign((size_t)m->n * V, -1);
        for (int k = 0; k < m->n; ++k) m->origin[(size_t)k * V] = node_origin[k];
    });
    if (rc) {
        delete m;
        return rc;
    }
    *out = m;
    return PFR_OK;
}

PFR_API int pfr_mesh_counts(const pfr_mesh* m, int32_t* n_nodes, int32_t* n_elems, int32_t* n_facets) {
    if (!m) return PFR_ERR_INVALID;
    if (n_nodes) *n_nodes = m->n;
    if (n_elems) *n_elems = m->e;
    if (n_facets) *n_facets = m->f;
    return PFR_OK;
}

PFR_API int pfr_mesh_read(const pfr_mesh* m, double* pos, uint8_t* flags, int32_t* conn, int32_t* facets,
                          int32_t* facet_elm, int32_t* facet_out, int32_t* origin) {
    if (!m) return PFR_ERR_INVALID;
    if (pos) std::copy(m->pos.begin(), m->pos.end(), pos);
    if (flags) std::copy(m->flags.begin(), m->flags.end(), flags);
    if (conn) std::copy(m->conn.begin(), m->conn.end(), conn);
    if (facets) std::copy(m->facets.begin(), m->facets.end(), facets);
    if (facet_elm) std::copy(m->facet_elm.begin(), m->facet_elm.end(), facet_elm);
    if (facet_out) std::copy(m->facet_out.begin(), m->facet_out.end(), facet_out);
    if (origin) std::copy(m->origin.begin(), m->origin.end(), origin);
    return PFR_OK;
}

PFR_API void pfr_mesh_free(pfr_mesh* m) { delete m; }

PFR_API const char* pfr_last_error(void) { return g_err.c_str(); }

}  // extern "C"
