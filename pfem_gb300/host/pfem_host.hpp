// C++ host mirror of the reference's solver interface over the C ABI of libpfemgpu.so.
//
//   pfem_gpu::Context                RAII owner of a pfg_ctx (one CUDA stream, device memory)
//   pfem_gpu::SolverIncompNewton     solveOneTimeStep / computeNextDT of
//                                    srcs/simulation/physics/IncompNewton/Solver.cpp:216-247
//   pfem_gpu::SolverWCompNewton      solveOneTimeStep / computeNextDT of
//                                    srcs/simulation/physics/WCompNewton/Solver.cpp:192-276
//
// Errors follow the reference's conventions: configuration and API errors throw
// std::runtime_error (as SolTable::checkAndGet does); a numerical failure of an incompressible
// step returns false from solveOneTimeStep with the positions and states already restored, and
// computeNextDT then divides the time step.  Remeshing stays with the caller: after it, call
// uploadMesh with the new arrays and setStates with the remapped node states.
// Header only; link libpfemgpu.so and include include/pfem_gpu.h.
#pragma once

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "pfem_gpu.h"

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

    // m_solveIncompNewtonNoT: the Picard solve; on success the time advances (the caller
    // remeshes and re-uploads, as Mesh::remesh follows in the reference)
    bool solveOneTimeStep() {
        ctx_.check(pfg_picard_step(ctx_.get(), dt_, &st_), "pfg_picard_step");
        ok_ = st_.converged != 0;
        if (ok_) time_ += dt_;
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
};

// SolverWCompNewton with the explicit step and its CFL time step on the GPU.
class SolverWCompNewton {
  public:
    explicit SolverWCompNewton(const pfg_params& p) : ctx_(p) {}

    Context& context() { return ctx_; }
    double getTimeStep() const { return st_.dt; }
    double getTime() const { return st_.time; }

    // after an upload and setStates: seed the device-side time and CFL step
    void start(double time = 0.0) {
        double dt = 0;
        ctx_.check(pfg_next_dt(ctx_.get(), &dt), "pfg_next_dt");
        ctx_.check(pfg_set_time(ctx_.get(), time, dt), "pfg_set_time");
        st_.dt = dt;
        st_.time = time;
    }

    // m_solveWCompNewtonNoT: one explicit step with the device-side CFL dt (computeNextDT
    // runs on the device after every step)
    bool solveOneTimeStep() {
        ctx_.check(pfg_wc_step(ctx_.get(), 0.0, 1, &st_), "pfg_wc_step");
        return true;
    }
    void computeNextDT() {}

  private:
    Context ctx_;
    pfg_step_status st_{};
};

}  // namespace pfem_gpu
