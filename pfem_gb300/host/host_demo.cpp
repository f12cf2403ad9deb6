// Drives libpfemgpu.so and libpfemremesh.so from C++ through pfem_host.hpp: a water column at
// rest in a box (walls left, bottom and right; open top), a few incompressible PSPG steps and a
// few weakly compressible steps; then a dam break meshed by the alpha shape and stepped with a
// remesh after every step (incompressible) or on the maxDT schedule (WC).  `host_demo remesh`
// runs only the host remesh checks (no GPU).  Prints one line per check and exits non-zero on
// failure.
//
//   g++ -std=c++17 -I include -I pfem_gb300/host pfem_gb300/host/host_demo.cpp
//       -L pfem_gb300 -lpfemgpu -lpfemremesh -Wl,-rpath,<dir of the libraries> -o host_demo
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pfem_host.hpp"

namespace {

struct Box {
    std::vector<double> pos;     // 2 x N
    std::vector<uint8_t> flags;  // N
    std::vector<int32_t> conn;   // 3 x E
    int N = 0;
};

// (nx+1) x (ny+1) lattice on [0, W] x [0, H], walls bound/fixed/Dirichlet, two positively
// oriented triangles per cell
Box make_box(int nx, int ny, double W, double H) {
    Box b;
    b.N = (nx + 1) * (ny + 1);
    b.pos.assign(2 * (size_t)b.N, 0.0);
    b.flags.assign(b.N, 0);
    auto id = [&](int i, int j) { return j * (nx + 1) + i; };
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            const int n = id(i, j);
            b.pos[n] = W * i / nx;
            b.pos[b.N + n] = H * j / ny;
            if (i == 0 || i == nx || j == 0) b.flags[n] = PFG_NODE_BOUND | PFG_NODE_FIXED | PFG_NODE_DIRICHLET;
            if (j == ny && i > 0 && i < nx) b.flags[n] = PFG_NODE_FREE_SURFACE;
        }
    std::vector<int32_t> a, c0, c1;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int p = id(i, j), q = id(i + 1, j), r = id(i + 1, j + 1), s = id(i, j + 1);
            a.push_back(p); c0.push_back(q); c1.push_back(r);
            a.push_back(p); c0.push_back(r); c1.push_back(s);
        }
    const size_t E = a.size();
    b.conn.resize(3 * E);
    for (size_t e = 0; e < E; ++e) {
        b.conn[e] = a[e];
        b.conn[E + e] = c0[e];
        b.conn[2 * E + e] = c1[e];
    }
    return b;
}

int fails = 0;
void expect(bool ok, const char* what, double value) {
    std::printf("%s %s %.6e\n", ok ? "ok" : "FAIL", what, value);
    if (!ok) ++fails;
}

// Node cloud of a 2D dam break: walls at spacing h (left, bottom, right of a W x Wh tank; bound,
// fixed, Dirichlet) and a cw x ch fluid column on the lattice offset by h, jittered by 0.1 h.
struct Cloud {
    std::vector<double> pos;
    std::vector<uint8_t> flags;
};
Cloud dam_break_cloud(double h, double W, double Wh, double cw, double ch) {
    std::vector<double> x, y;
    std::vector<uint8_t> f;
    const uint8_t wall = PFG_NODE_BOUND | PFG_NODE_FIXED | PFG_NODE_DIRICHLET;
    const int nh = (int)std::lround(Wh / h), nw = (int)std::lround(W / h);
    for (int j = nh; j >= 0; --j) x.push_back(0.0), y.push_back(h * j), f.push_back(wall);
    for (int i = 1; i <= nw; ++i) x.push_back(h * i), y.push_back(0.0), f.push_back(wall);
    for (int j = 1; j <= nh; ++j) x.push_back(W), y.push_back(h * j), f.push_back(wall);
    unsigned long long s = 12345;
    auto unif = [&]() {  // 64-bit LCG, top 53 bits
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return (double)(s >> 11) * 0x1.0p-53;
    };
    for (int i = 1; i <= (int)std::lround(cw / h); ++i)
        for (int j = 1; j <= (int)std::lround(ch / h); ++j) {
            x.push_back(h * i + (2 * unif() - 1) * 0.1 * h);
            y.push_back(h * j + (2 * unif() - 1) * 0.1 * h);
            f.push_back(0);
        }
    Cloud c;
    c.pos = x;
    c.pos.insert(c.pos.end(), y.begin(), y.end());
    c.flags = f;
    return c;
}

double min_measure(const pfem_gpu::Mesh& m) {
    const int n = m.nodes(), e = m.elements(), d = m.dim;
    double mn = 1e300;
    for (int k = 0; k < e; ++k) {
        double J[3][3];
        for (int a = 0; a < d; ++a)
            for (int c = 0; c < d; ++c)
                J[c][a] = m.pos[(size_t)c * n + m.conn[(size_t)(a + 1) * e + k]] - m.pos[(size_t)c * n + m.conn[k]];
        const double det = d == 2 ? J[0][0] * J[1][1] - J[0][1] * J[1][0]
                                  : J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                                        J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                                        J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        mn = std::min(mn, det);
    }
    return mn;
}

// host remesh only: the alpha shape of the cloud, then one remesh of the moved mesh
void remesh_checks() {
    const double h = 0.05;
    const Cloud c = dam_break_cloud(h, 4.0, 3.0, 1.0, 2.0);
    pfem_gpu::Remesher r(pfem_gpu::Remesher::defaults(2, h));
    pfem_gpu::Mesh m = r.alphaShape(c.pos, c.flags);
    int fs = 0;
    for (uint8_t f : m.flags) fs += (f & PFG_NODE_FREE_SURFACE) ? 1 : 0;
    expect(m.elements() > 1500 && m.nodes() == (int)c.flags.size(), "alpha shape elements", m.elements());
    expect(min_measure(m) > 0, "alpha shape positively oriented, min det", min_measure(m));
    expect(fs > 40, "free-surface nodes", fs);
    std::vector<double> moved = m.pos;
    unsigned long long s = 99;
    for (int i = 0; i < m.nodes(); ++i)
        if (!(m.flags[i] & PFG_NODE_BOUND))
            for (int d = 0; d < 2; ++d) {
                s = s * 6364136223846793005ull + 1442695040888963407ull;
                moved[(size_t)d * m.nodes() + i] += ((double)(s >> 11) * 0x1.0p-53 - 0.5) * 0.4 * h;
            }
    const pfem_gpu::Mesh m2 = r.remesh(m, moved);
    bool origins = true;
    for (int32_t o : m2.origin) origins = origins && o >= -1 && o < m.nodes();
    // the moved mesh gains centroid nodes in stretched elements and loses nodes of close pairs
    expect(origins && m2.nodes() > 0.8 * m.nodes() && m2.nodes() < 1.25 * m.nodes(), "remesh nodes", m2.nodes());
    expect(min_measure(m2) > 0, "remesh positively oriented, min det", min_measure(m2));
}

}  // namespace

int main(int argc, char** argv) {
    const double rho = 1000.0, g = 9.81, H = 0.5;
    const Box box = make_box(20, 10, 1.0, H);
    if (argc > 1 && std::strcmp(argv[1], "remesh") == 0) {
        try {
            remesh_checks();
        } catch (const std::exception& e) {
            std::printf("FAIL exception %s\n", e.what());
            return 2;
        }
        return fails ? 1 : 0;
    }
    try {
        // incompressible: hydrostatic column stays at rest
        pfg_params p;
        pfg_default_params(PFG_KIND_INCOMP_PSPG, 2, &p);
        pfem_gpu::SolverIncompNewton inc(p, 1e-3, 1e-3);
        inc.context().uploadMesh(box.pos, box.flags, box.conn);
        std::vector<double> q(3 * (size_t)box.N, 0.0);
        for (int n = 0; n < box.N; ++n) q[2 * (size_t)box.N + n] = rho * g * (H - box.pos[box.N + n]);
        inc.context().setStates(q);
        const double v0 = inc.context().volume();
        int ok = 0;
        for (int k = 0; k < 5; ++k) {
            ok += inc.solveOneTimeStep();
            inc.computeNextDT();
        }
        expect(ok == 5, "incompressible steps converged", ok);
        const std::vector<double> s = inc.context().states();
        double vmax = 0;
        for (int n = 0; n < 2 * box.N; ++n) vmax = std::max(vmax, std::fabs(s[n]));
        expect(vmax < 1e-3, "hydrostatic column stays at rest, max |v|", vmax);
        expect(std::fabs(inc.context().volume() - v0) < 1e-9 * v0, "volume", inc.context().volume());

        // weakly compressible: mass conservation over 100 explicit steps
        pfg_params pw;
        pfg_default_params(PFG_KIND_WC_CDS_DPDT, 2, &pw);
        pw.precision = PFG_PREC_MIXED;
        pfem_gpu::SolverWCompNewton wc(pw);
        wc.context().uploadMesh(box.pos, box.flags, box.conn);
        std::vector<double> w(6 * (size_t)box.N, 0.0);
        for (int n = 0; n < box.N; ++n) {
            const double pr = rho * g * (H - box.pos[box.N + n]);
            w[2 * (size_t)box.N + n] = pr;
            w[3 * (size_t)box.N + n] = pw.rho_star * std::pow(1 + pw.K0p / pw.K0 * pr, 1 / pw.K0p);
        }
        wc.context().setStates(w);
        wc.start();
        const double m0 = wc.context().mass();
        for (int k = 0; k < 100; ++k) {
            wc.solveOneTimeStep();
            wc.computeNextDT();
        }
        const double m1 = wc.context().mass();
        expect(std::fabs(m1 - m0) < 1e-6 * m0, "WC mass after 100 steps", m1);
        expect(wc.getTime() > 0 && wc.getTimeStep() > 0, "WC time", wc.getTime());

        // dam break with the host remesh: incompressible, remeshed after every step
        remesh_checks();
        const double h = 0.05;
        const Cloud cl = dam_break_cloud(h, 4.0, 3.0, 1.0, 2.0);
        pfem_gpu::Remesher rm(pfem_gpu::Remesher::defaults(2, h));
        pfem_gpu::Mesh mesh = rm.alphaShape(cl.pos, cl.flags);
        pfem_gpu::SolverIncompNewton db(p, 1e-3, 1e-3);
        db.context().uploadMesh(mesh.pos, mesh.flags, mesh.conn);
        std::vector<double> qd(3 * (size_t)mesh.nodes(), 0.0);
        for (int n = 0; n < mesh.nodes(); ++n)
            if (!(mesh.flags[n] & PFG_NODE_BOUND))
                qd[2 * (size_t)mesh.nodes() + n] = rho * g * std::max(0.0, 2.0 - mesh.pos[mesh.nodes() + n]);
        db.context().setStates(qd);
        db.setRemesher(&rm, &mesh);
        const double vd0 = db.context().volume();
        int okd = 0;
        for (int k = 0; k < 20; ++k) {
            okd += db.solveOneTimeStep();
            db.computeNextDT();
        }
        expect(okd == 20, "dam break steps with remesh converged", okd);
        expect(std::fabs(db.context().volume() - vd0) < 0.02 * vd0, "dam break volume", db.context().volume());
        expect(min_measure(mesh) > 0 && db.context().nodes() == mesh.nodes(), "remeshed mesh on the device",
               mesh.nodes());

        // WC dam break remeshed every maxDT
        pfem_gpu::Mesh wmesh = rm.alphaShape(cl.pos, cl.flags);
        pfg_params pw2;
        pfg_default_params(PFG_KIND_WC_CDS_DPDT, 2, &pw2);
        pw2.max_dt = 2e-4;
        pfem_gpu::SolverWCompNewton wr(pw2);
        wr.context().uploadMesh(wmesh.pos, wmesh.flags, wmesh.conn);
        std::vector<double> ws(6 * (size_t)wmesh.nodes(), 0.0);
        for (int n = 0; n < wmesh.nodes(); ++n) {
            const double pr = (wmesh.flags[n] & PFG_NODE_BOUND) ? 0.0 : rho * g * std::max(0.0, 2.0 - wmesh.pos[wmesh.nodes() + n]);
            ws[2 * (size_t)wmesh.nodes() + n] = pr;
            ws[3 * (size_t)wmesh.nodes() + n] = pw2.rho_star * std::pow(1 + pw2.K0p / pw2.K0 * pr, 1 / pw2.K0p);
        }
        wr.context().setStates(ws);
        wr.start();
        wr.setRemesher(&rm, &wmesh);
        const double wm0 = wr.context().mass();
        for (int k = 0; k < 300; ++k) wr.solveOneTimeStep();
        const std::vector<double> wsn = wr.context().states();
        bool finite = true;
        for (double v : wsn) finite = finite && std::isfinite(v);
        expect(wr.remeshes() > 0 && finite, "WC remeshes", wr.remeshes());
        expect(std::fabs(wr.context().mass() - wm0) < 0.02 * wm0, "WC mass with remesh", wr.context().mass());
    } catch (const std::exception& e) {
        std::printf("FAIL exception %s\n", e.what());
        return 2;
    }
    return fails ? 1 : 0;
}
