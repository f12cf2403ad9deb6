// C++ host mirror of the reference's solver interface over the C ABIs of libpfemgpu.so and
// libpfemremesh.so.
//
//   pfem_gpu::Context                RAII owner of a pfg_ctx (one CUDA stream, device memory)
//   pfem_gpu::Mesh                   host arrays of a mesh (positions, flags, connectivity,
//                                    facets, state origins)
//   pfem_gpu::Remesher               Mesh::remesh / triangulateAlphaShape (srcs/mesh/Mesh.cpp:
//                                    919-926, Mesh2D.cpp:32-251, Mesh3D.cpp:36-286) in C++
//   pfem_gpu::SolverIncompNewton     solveOneTimeStep / computeNextDT of
//                                    srcs/simulation/physics/IncompNewton/Solver.cpp:216-247
//   pfem_gpu::SolverWCompNewton      solveOneTimeStep / computeNextDT of
//                                    srcs/simulation/physics/WCompNewton/Solver.cpp:192-276
//
// Errors follow the reference's conventions: configuration and API errors throw
// std::runtime_error (as SolTable::checkAndGet does); a numerical failure of an incompressible
// step returns false from solveOneTimeStep with the positions and states already restored, and
// computeNextDT then divides the time step.  With a Remesher attached (setRemesher), a solver
// rebuilds the mesh where the reference's does: after every successful incompressible step, and
// for WC once the time passes the next remeshing time (which then advances by maxDT).
// Header only; link libpfemgpu.so and libpfemremesh.so, include include/pfem_gpu.h and
// include/pfem_remesh.h.
#pragma once

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "pfem_gpu.h"
#include "pfem_remesh.h"

namespace pfem_gpu {

class Context {
  public:
    explicit Context(const pfg_params& p) {
        if (pfg_create(&p, &ctx_) != PFG_OK) throw std::runtime_error("pfg_create failed");
        params_ = p;
    }
    ~Context() {
        if (ctx_) pfg_destroy(ctx_);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    pfg_ctx* get() const { return ctx_; }
    const pfg_params& params() const { return params_; }
    int dim() const { return params_.dim; }

    void check(int rc, const char* what) const {
        if (rc != PFG_OK) throw std::runtime_error(std::string(what) + ": " + pfg_last_error(ctx_));
    }

    // positions dim x N (structure of arrays), one flag byte per node, (dim+1) x E connectivity
    void uploadMesh(const std::vector<double>& pos, const std::vector<uint8_t>& flags,
                    const std::vector<int32_t>& conn) {
        const int32_t n = (int32_t)flags.size();
        const int32_t e = (int32_t)(conn.size() / (dim() + 1));
        if (pos.size() != (size_t)dim() * n) throw std::runtime_error("uploadMesh: positions must be dim x N");
        check(pfg_upload_mesh(ctx_, n, pos.data(), flags.data(), e, conn.data()), "pfg_upload_mesh");
        nodes_ = n;
    }
    // boundary facets (dim x F nodes) and the element of each; needed after every uploadMesh
    // when params.gamma > 0 (surface tension)
    void uploadFacets(const std::vector<int32_t>& facets, const std::vector<int32_t>& facetElm) {
        if (facets.size() != (size_t)dim() * facetElm.size())
            throw std::runtime_error("uploadFacets: facets must be dim x F");
        check(pfg_upload_facets(ctx_, (int32_t)facetElm.size(), facets.data(), facetElm.data()), "pfg_upload_facets");
    }
    int nodes() const { return nodes_; }
    int statesPerNode() const {
        return params_.kind == PFG_KIND_INCOMP_PSPG ? params_.dim + 1 : 2 * params_.dim + 2;
    }
    // a remeshed domain with the node states (and temperatures) remapped on the device:
    // origin is N_new x width, the old nodes whose mean each new node takes (incompressible)
    void uploadMeshRemap(const std::vector<double>& pos, const std::vector<uint8_t>& flags,
                         const std::vector<int32_t>& conn, const std::vector<int32_t>& origin, int width) {
        const int32_t n = (int32_t)flags.size();
        const int32_t e = (int32_t)(conn.size() / (dim() + 1));
        if (pos.size() != (size_t)dim() * n || origin.size() != (size_t)n * width)
            throw std::runtime_error("uploadMeshRemap: positions must be dim x N and origin N x width");
        check(pfg_upload_mesh_remap(ctx_, n, pos.data(), flags.data(), e, conn.data(), origin.data(), width),
              "pfg_upload_mesh_remap");
        nodes_ = n;
    }
    void setStates(const std::vector<double>& q) {
        if (q.size() != (size_t)statesPerNode() * nodes_) throw std::runtime_error("setStates: wrong size");
        check(pfg_set_states(ctx_, q.data()), "pfg_set_states");
    }
    std::vector<double> states() const {
        std::vector<double> q((size_t)statesPerNode() * nodes_);
        check(pfg_get_states(ctx_, q.data()), "pfg_get_states");
        return q;
    }
    std::vector<double> positions() const {
        std::vector<double> x((size_t)dim() * nodes_);
        check(pfg_get_positions(ctx_, x.data()), "pfg_get_positions");
        return x;
    }
    double volume() const {
        double v = 0;
        check(pfg_volume(ctx_, &v), "pfg_volume");
        return v;
    }
    double mass() const {
        double m = 0;
        check(pfg_mass(ctx_, &m), "pfg_mass");
        return m;
    }
    // heat equation (HeatEqIncompNewton): node temperatures, BCs, one solve
    void setTemperature(const std::vector<double>& T) {
        if (T.size() != (size_t)nodes_) throw std::runtime_error("setTemperature: wrong size");
        check(pfg_set_temperature(ctx_, T.data()), "pfg_set_temperature");
    }
    std::vector<double> temperature() const {
        std::vector<double> T((size_t)nodes_);
        check(pfg_get_temperature(ctx_, T.data()), "pfg_get_temperature");
        return T;
    }
    void setHeatBC(const std::vector<uint8_t>& flags, const std::vector<double>& tDirichlet) {
        if (flags.size() != (size_t)nodes_ || (!tDirichlet.empty() && tDirichlet.size() != (size_t)nodes_))
            throw std::runtime_error("setHeatBC: wrong size");
        check(pfg_heat_set_bc(ctx_, flags.data(), tDirichlet.empty() ? nullptr : tDirichlet.data()),
              "pfg_heat_set_bc");
    }
    pfg_step_status heatStep(double dt) {
        pfg_step_status st{};
        check(pfg_heat_step(ctx_, dt, &st), "pfg_heat_step");
        return st;
    }
    // prescribed heat flux at the facet Gauss points, (F, 3, dim); empty clears it
    void setHeatFlux(const std::vector<double>& qGp) {
        check(pfg_heat_set_flux(ctx_, qGp.empty() ? nullptr : qGp.data()), "pfg_heat_set_flux");
    }
    // independent meshes back to back (instance i owns nodes [off[i], off[i+1])), mixed precision
    void setInstances(const std::vector<int32_t>& off, const std::vector<double>& rho, const std::vector<double>& mu) {
        const int32_t n = (int32_t)off.size() - 1;
        if (n < 1 || rho.size() != (size_t)n || mu.size() != (size_t)n)
            throw std::runtime_error("setInstances: offsets, rho and mu disagree");
        check(pfg_set_instances(ctx_, n, off.data(), rho.data(), mu.data()), "pfg_set_instances");
        instances_ = n;
    }
    // one time step per instance (dt[i] for instance i)
    std::vector<pfg_step_status> picardStepBatch(const std::vector<double>& dt) {
        if (dt.size() != (size_t)instances_) throw std::runtime_error("picardStepBatch: one dt per instance");
        std::vector<pfg_step_status> st((size_t)instances_);
        check(pfg_picard_step_batch(ctx_, dt.data(), st.data()), "pfg_picard_step_batch");
        return st;
    }
    std::vector<pfg_step_status> wcStepBatch(double dt, int nsteps) {
        std::vector<pfg_step_status> st((size_t)instances_);
        check(pfg_wc_step_batch(ctx_, dt, nsteps, st.data()), "pfg_wc_step_batch");
        return st;
    }
    // launch shapes of the mixed form's tunable kernels (zero fields keep their value)
    void setTuning(const pfg_tuning& t) { check(pfg_set_tuning(ctx_, &t), "pfg_set_tuning"); }
    pfg_tuning tuning() const {
        pfg_tuning t{};
        check(pfg_get_tuning(ctx_, &t), "pfg_get_tuning");
        return t;
    }

  private:
    pfg_ctx* ctx_ = nullptr;
    pfg_params params_{};
    int nodes_ = 0;
    int instances_ = 1;
};

// Host arrays of a mesh, as pfr_remesh / pfr_alpha_shape return them.
struct Mesh {
    int dim = 2;
    std::vector<double> pos;       // dim x N
    std::vector<uint8_t> flags;    // N (PFG_NODE_* bits, free surface from the triangulation)
    std::vector<int32_t> conn;     // (dim+1) x E, positively oriented
    std::vector<int32_t> facets;   // dim x F boundary facets
    std::vector<int32_t> facetElm; // F: the element of each facet
    std::vector<int32_t> facetOut; // F: the element's node off the facet
    std::vector<int32_t> origin;   // N x (dim+1): old nodes whose states each node takes, -1 padded
    int nodes() const { return (int)flags.size(); }
    int elements() const { return (int)(conn.size() / (dim + 1)); }
    int facetCount() const { return (int)facetElm.size(); }
};

// Mesh::remesh and Mesh::triangulateAlphaShape through libpfemremesh.so.
class Remesher {
  public:
    explicit Remesher(const pfr_params& p) : p_(p) {}
    static pfr_params defaults(int dim, double hchar) {
        pfr_params p;
        if (pfr_default_params(dim, hchar, &p) != PFR_OK) throw std::runtime_error("pfr_default_params failed");
        return p;
    }
    const pfr_params& params() const { return p_; }

    // the initial mesh of a node cloud (positions dim x N, flags with PFG_NODE_BOUND set on walls)
    Mesh alphaShape(const std::vector<double>& pos, const std::vector<uint8_t>& flags) const {
        const int32_t n = (int32_t)flags.size();
        if (pos.size() != (size_t)p_.dim * n) throw std::runtime_error("alphaShape: positions must be dim x N");
        pfr_mesh* m = nullptr;
        check(pfr_alpha_shape(&p_, n, pos.data(), flags.data(), &m), "pfr_alpha_shape");
        return take(m);
    }

    // one remesh of `cur` whose nodes moved to `pos` (dim x N)
    Mesh remesh(const Mesh& cur, const std::vector<double>& pos) const {
        if (pos.size() != (size_t)p_.dim * cur.nodes()) throw std::runtime_error("remesh: positions must be dim x N");
        pfr_mesh* m = nullptr;
        check(pfr_remesh(&p_, cur.nodes(), pos.data(), cur.flags.data(), cur.elements(), cur.conn.data(), &m),
              "pfr_remesh");
        return take(m);
    }

    // remesh the context's mesh in place: positions from the device; incompressible states (and
    // temperatures) remapped on the device, WC states (and BoussinesqWC temperatures) remapped
    // here (their mean over the origins).  Per-node inputs (Dirichlet values, heat boundary
    // conditions) belong to the old node numbering: set them again after a remesh.
    void remesh(Context& ctx, Mesh& cur) const {
        Mesh next = remesh(cur, ctx.positions());
        const int w = p_.dim + 1;
        if (ctx.params().kind == PFG_KIND_INCOMP_PSPG) {
            ctx.uploadMeshRemap(next.pos, next.flags, next.conn, next.origin, w);
        } else {
            // WC states (and, for BoussinesqWC, the temperatures) remapped here: each new node
            // takes the mean of its origins' values, summed in origin order
            const int n_old = cur.nodes(), n = next.nodes();
            auto remap = [&](const std::vector<double>& q, int nf) {
                std::vector<double> out((size_t)nf * n);
                for (int f = 0; f < nf; ++f)
                    for (int j = 0; j < n; ++j) {
                        const int32_t* o = &next.origin[(size_t)j * w];
                        double s = 0.0;
                        int cnt = 0;
                        for (int k = 0; k < w && o[k] >= 0; ++k, ++cnt) s += q[(size_t)f * n_old + o[k]];
                        out[(size_t)f * n + j] = s / cnt;
                    }
                return out;
            };
            const std::vector<double> q = remap(ctx.states(), ctx.statesPerNode());
            const bool heat = ctx.params().boussinesq != 0;
            const std::vector<double> T = heat ? remap(ctx.temperature(), 1) : std::vector<double>();
            ctx.uploadMesh(next.pos, next.flags, next.conn);
            ctx.setStates(q);
            if (heat) ctx.setTemperature(T);
        }
        if (next.facetCount() && (ctx.params().gamma >= 1e-15 || ctx.params().dgamma_dt >= 1e-15))
            ctx.uploadFacets(next.facets, next.facetElm);
        cur = std::move(next);
    }

  private:
    static void check(int rc, const char* what) {
        if (rc != PFR_OK) throw std::runtime_error(std::string(what) + ": " + pfr_last_error());
    }
    Mesh take(pfr_mesh* m) const {
        Mesh r;
        r.dim = p_.dim;
        int32_t n = 0, e = 0, f = 0;
        pfr_mesh_counts(m, &n, &e, &f);
        r.pos.resize((size_t)p_.dim * n);
        r.flags.resize(n);
        r.conn.resize((size_t)(p_.dim + 1) * e);
        r.facets.resize((size_t)p_.dim * f);
        r.facetElm.resize(f);
        r.facetOut.resize(f);
        r.origin.resize((size_t)n * (p_.dim + 1));
        pfr_mesh_read(m, r.pos.data(), r.flags.data(), r.conn.data(), r.facets.data(), r.facetElm.data(),
                      r.facetOut.data(), r.origin.data());
        pfr_mesh_free(m);
        return r;
    }
    pfr_params p_;
};

// SolverIncompNewton with the PSPG solve on the GPU.
class SolverIncompNewton {
  public:
    SolverIncompNewton(const pfg_params& p, double initialDT, double maxDT, bool adaptDT = true,
                       double coeffDTincrease = 1.5, double coeffDTDecrease = 2.0)
        : ctx_(p), dt_(initialDT), maxDT_(maxDT), adapt_(adaptDT), inc_(coeffDTincrease), dec_(coeffDTDecrease) {}

    Context& context() { return ctx_; }
    double getTimeStep() const { return dt_; }
    double getTime() const { return time_; }
    const pfg_step_status& lastStatus() const { return st_; }

    // remesh after every successful step (the solver keeps pointers: both must outlive it)
    void setRemesher(const Remesher* r, Mesh* mesh) {
        remesher_ = r;
        mesh_ = mesh;
    }

    // m_solveIncompNewtonNoT: the Picard solve; on success the time advances and, with a
    // Remesher attached, the mesh is rebuilt (Mesh::remesh, Solver.cpp:233-236)
    bool solveOneTimeStep() {
        ctx_.check(pfg_picard_step(ctx_.get(), dt_, &st_), "pfg_picard_step");
        ok_ = st_.converged != 0;
        if (ok_) {
            time_ += dt_;
            if (remesher_) remesher_->remesh(ctx_, *mesh_);
        }
        return ok_;
    }

    void computeNextDT() {
        if (!ok_) {
            if (!adapt_) throw std::runtime_error("solving the precedent time step was not successful!");
            dt_ /= dec_;
        } else if (adapt_) {
            dt_ = std::min(maxDT_, dt_ * inc_);
        }
    }

  private:
    Context ctx_;
    double dt_, maxDT_;
    bool adapt_;
    double inc_, dec_;
    double time_ = 0;
    bool ok_ = true;
    pfg_step_status st_{};
    const Remesher* remesher_ = nullptr;
    Mesh* mesh_ = nullptr;
};

// SolverWCompNewton with the explicit step and its CFL time step on the GPU.
class SolverWCompNewton {
  public:
    explicit SolverWCompNewton(const pfg_params& p) : ctx_(p) {}

    Context& context() { return ctx_; }
    double getTimeStep() const { return st_.dt; }
    double getTime() const { return st_.time; }

    // after an upload and setStates: seed the device-side time and CFL step; the first
    // remeshing time is maxDT (the intent of the commented-out initialisation, Solver.cpp:63-66)
    void start(double time = 0.0) {
        double dt = 0;
        ctx_.check(pfg_next_dt(ctx_.get(), &dt), "pfg_next_dt");
        ctx_.check(pfg_set_time(ctx_.get(), time, dt), "pfg_set_time");
        st_.dt = dt;
        st_.time = time;
        nextRemesh_ = time + ctx_.params().max_dt;
    }

    // remesh on the reference's schedule (the solver keeps pointers: both must outlive it)
    void setRemesher(const Remesher* r, Mesh* mesh) {
        remesher_ = r;
        mesh_ = mesh;
    }
    int remeshes() const { return remeshes_; }

    // m_solveWCompNewtonNoT: one explicit step with the device-side CFL dt (computeNextDT
    // runs on the device after every step); once the time passes the next remeshing time the
    // mesh is rebuilt and that time advances by maxDT (Solver.cpp:264-272)
    bool solveOneTimeStep() {
        ctx_.check(pfg_wc_step(ctx_.get(), 0.0, 1, &st_), "pfg_wc_step");
        if (remesher_ && st_.time > nextRemesh_) {
            remesher_->remesh(ctx_, *mesh_);
            double dt = 0;
            ctx_.check(pfg_next_dt(ctx_.get(), &dt), "pfg_next_dt");
            ctx_.check(pfg_set_time(ctx_.get(), st_.time, dt), "pfg_set_time");
            st_.dt = dt;
            nextRemesh_ += ctx_.params().max_dt;
            ++remeshes_;
        }
        return true;
    }
    void computeNextDT() {}

  private:
    Context ctx_;
    pfg_step_status st_{};
    const Remesher* remesher_ = nullptr;
    Mesh* mesh_ = nullptr;
    double nextRemesh_ = 0;
    int remeshes_ = 0;
};

}  // namespace pfem_gpu
