// Drives libpfemgpu.so from C++ through pfem_host.hpp: a water column at rest in a box (walls
// left, bottom and right; open top), a few incompressible PSPG steps and a few weakly
// compressible steps.  Prints one line per check and exits non-zero on failure.
//
//   g++ -std=c++17 -I include -I pfem_gb300/host pfem_gb300/host/host_demo.cpp
//       -L pfem_gb300 -lpfemgpu -Wl,-rpath,<dir of libpfemgpu.so> -o host_demo
#include <cmath>
#include <cstdio>
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

}  // namespace

int main() {
    const double rho = 1000.0, g = 9.81, H = 0.5;
    const Box box = make_box(20, 10, 1.0, H);
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
    } catch (const std::exception& e) {
        std::printf("FAIL exception %s\n", e.what());
        return 2;
    }
    return fails ? 1 : 0;
}
