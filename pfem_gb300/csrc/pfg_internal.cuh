// Internal declarations of the PFEM GB300 library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/pfem_gpu.h"

namespace pfg {

constexpr uint8_t F_BOUND = PFG_NODE_BOUND;
constexpr uint8_t F_FREE_SURFACE = PFG_NODE_FREE_SURFACE;
constexpr uint8_t F_FIXED = PFG_NODE_FIXED;
constexpr uint8_t F_DIRICHLET = PFG_NODE_DIRICHLET;
constexpr uint8_t F_FREE = PFG_NODE_FREE;

// Upper bound on distinct neighbours (including itself) of one node.  Delaunay meshes have
// mean valence ~6 (2D) / ~14 (3D); the cap leaves room for badly shaped post-remesh stars.
constexpr int MAX_NBR = 128;

// Device error word bits (ctx->d_err).
constexpr int ERR_NBR_OVERFLOW = 1;
constexpr int ERR_KRYLOV_BREAKDOWN = 2;
constexpr int ERR_NONFINITE = 4;

// Gauss-point tables of the element rules (Mesh::getGaussPoints/Weight/ShapeFunctions,
// srcs/mesh/Mesh.cpp:342-530) and the sums the closed-form element kernels need.
struct GaussConst {
    int n;            // points
    double w[4];      // weights
    double N[4][4];   // N[g][i]
    double MM[4][4];  // sum_g w_g N_i N_j
    double s[4];      // sum_g w_g N_i
    double sumw;      // sum_g w_g
    double refSize;   // reference element size
};

// Grow-only device buffer.
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
};

struct Reducer;  // fwd

// One coarse level of the node-aggregation multigrid (pfg_mg.cu): block CSR with (d+1)^2
// FP32 blocks and node-major (d+1)-vectors.
struct MgLevel {
    int n = 0, nnzb = 0;
    DBuf agg;              // finer-level node -> aggregate (this level's node), -1 = none
    DBuf mem_ptr, mem;     // members of each aggregate, ascending
    DBuf bptr, bcol, bdiag;
    DBuf gptr, glist;      // Galerkin gather list of each block (finer-level block ids)
    DBuf val, binv;        // blocks, diagonal-block inverses
    DBuf x, xb, b;         // cycle vectors
};

// One front of the device sparse LU (pfg_lu.cu).
struct LuFront {
    int nv, nb;          // own / boundary nodes
    int node_off;        // into lu_nodes (V then B)
    int rec_off, n_rec;  // assembly records
    int child_off, n_child;
    int map_off;         // B's local indices in the parent's front
    int piv_off;         // m pivots
    long long mat_off;   // dense n x n matrix (row-major)
    long long vec_off;   // n-vector of the solve
};

}  // namespace pfg

struct pfg_ctx {
    pfg_params prm{};
    pfg_tuning tune{};  // launch shapes of the tunable mixed-form kernels (pfg_set_tuning)
    int dim = 0, npe = 0;
    int N = 0, E = 0;
    int R = 0;          // incompressible unknowns (dim+1)*N
    int nstates = 0;    // per-node states of the kind
    bool has_mesh = false;
    bool has_system = false;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    size_t bytes_in_use = 0;

    // mesh
    pfg::DBuf pos, pos_save, flags, conn;
    // node -> element incidence (ascending element per node)
    pfg::DBuf ne_ptr, ne_elem, ne_loc;
    pfg::DBuf inc_slot;    // (e, local i) -> position of that incidence in the node-major lists
    // node adjacency (sorted, includes the node) and the node-pair list
    pfg::DBuf nbr_ptr, nbr, pair_node;
    int P = 0;
    // mixed PSPG: element list of each off-diagonal node pair (slot(e)*16 + i*4 + j, ascending e)
    pfg::DBuf pe_ptr, pe_item;
    pfg::DBuf pe_pair;        // the pair of each item (item-parallel pair assembly)
    pfg::DBuf pe_pos;         // each item as (position in the row's incidences) * 16 + i * 4 + j
    long long n_items = 0;    // pair element items, E (d+1) d
    // mixed assembly: slot of each element in the element-major data (elements ordered by their
    // smallest node) and the slot of each incidence's element
    pfg::DBuf el_slot, ne_slot;
    pfg::DBuf conn_s;  // connectivity in slot order
    // CSR system
    pfg::DBuf row_ptr, col, val, val32, diag_pos, rhs;
    int64_t nnz = 0;
    // element data of the plain FP64 form [detJ, tau, gradN, ksum] (structure of arrays), and a
    // double-float copy used by the heat assembly alone.  edata is overwritten by the heat
    // assembly (k_heat_geom stores the heat layout in it): every reader's own assembly rewrites
    // it first, so no reader may carry it across a heat step.  The mixed form keeps its element
    // data in mx_ed_aos, which no other assembly writes.
    pfg::DBuf edata, edata_df;
    // incompressible states
    pfg::DBuf q, q_prev, q_iter_prev, vbc;
    // Krylov workspace
    pfg::DBuf kv;          // 10 vectors of R doubles
    pfg::DBuf kv32;        // FP32 workspace (mixed precision)
    pfg::DBuf binv;        // node-block Jacobi inverses, (dim+1)^2 x N
    pfg::DBuf red;         // reduction partials + scalars + counters
    pfg::DBuf err_word;    // int device error word
    // WC
    pfg::DBuf ws;          // states (2d+2)*N of the working precision
    pfg::DBuf wc_el;       // element -> node partial values
    pfg::DBuf wc_dt;       // [dt_next, time, dt_min_bits]
    pfg::DBuf stage;       // FP64 staging for host<->device precision conversion
    int wc_pending = 0;    // steps enqueued since the last synchronize
    int wc_cur = 0;        // mixed form: current half of the ping-pong v/p state
    double host_time = 0.0;
    // host mirrors for validation
    std::vector<uint8_t> h_flags;
    // pinned host scratch for scalar readbacks
    double* h_scalars = nullptr;
    int max_grid = 0;      // blocks for grid-stride loops (multiple of the SM count)
    int num_sms = 0;
    // phase timers
    bool prof = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<int> marks;  // (phase, ev_start, ev_stop) triples
    double phase_ms[PFG_NUM_PHASES] = {};
    long long phase_n[PFG_NUM_PHASES] = {};
    long long spmv_pairs = 0;             // node pairs read by the timed Krylov SpMV launches
    long long spmv_list_pairs = 0;        // node pairs of the instances the next launch covers
    std::vector<long long> h_inst_pairs;  // node pairs per instance
    // WC: FP64 element partials, per-node CFL quantities, captured step graphs [fixed, adaptive]
    pfg::DBuf wc_eld, wc_nodal;
    // WC mixed form, batched: number of instances (1 = a single mesh) and per-instance
    // [mu, mu sum_g w_g]; the node -> instance map shares node_inst with the PSPG form
    int n_wc_inst = 1;
    pfg::DBuf wc_inst;
    cudaGraphExec_t wc_graph[2] = {nullptr, nullptr};
    // mixed-precision PSPG: FP32 block inverses, instance tables (segments of nodes,
    // per-instance ints / doubles / FP32 Krylov scalars), reduction partials, counters
    pfg::DBuf binv32, node_inst, mx_seg, mx_ii, mx_id, mx_sc, mx_part, mx_cnt, mx_scale, mx_list;
    // mixed PSPG assembly and residual: FP32 row scales, per-instance FP32 / double-float
    // coefficients, double-float copies of the iterate (Dirichlet values substituted), of the
    // previous velocities, of the temperatures and of the positions and iterate velocities (the
    // element prep's inputs), and the element records of A_e x (one 32-byte record of d+1
    // double-float values per element node)
    pfg::DBuf mx_scale32, mx_f32, mx_xdf, mx_vpdf, mx_tdf, mx_rec, mx_gdf;
    pfg::DBuf mx_ed_aos;  // element data element-major (high, then low parts) for the gathering kernels
    pfg::DBuf mx_vsum;    // per element: sums of the previous velocities over its nodes (double-float)
    int n_inst = 0, n_seg = 0;
    cudaGraphExec_t mx_graph[2] = {nullptr, nullptr};  // one chunk of BiCGSTAB iterations [FP32, FP64]
    std::vector<int> h_mx_ii;
    std::vector<double> h_mx_id;
    std::vector<float> h_mx_f32;
    // surface tension: facets (dim x F nodes, element of each), the nodes their elements touch
    // with each one's (facet, local node of the facet's element) entries, and the force array
    // (dim x N, FP64 or FP32 by the kind's precision)
    pfg::DBuf fc_nodes, fc_elem, nf_nodes, nf_ptr, nf_ent, fst_force;
    int F = 0;
    int n_fst_nodes = 0;
    bool has_facets = false;
    std::vector<int32_t> h_conn;
    // multigrid preconditioner of the mixed correction solves: coarse levels (n_mg in use) and
    // the level-0 cycle vectors
    std::vector<pfg::MgLevel> mg;
    int n_mg = 0;
    pfg::DBuf mg_x0;
    pfg::DBuf mg_in64;     // FP64 correction solves: FP32 scaled input and output of the cycle
    pfg::DBuf val16;       // bfloat16 copy of the node-pair blocks (level-0 multigrid sweeps)
    // heat equation: node temperatures, BC flags and Dirichlet values, the scalar system over
    // the node pairs (values in pair order, right-hand side), CG vectors, reductions, the
    // per-node lists of heat facets (facet * 4 + facet-local node) with each facet's flux
    // flags, and the flux vectors at the facet Gauss points
    pfg::DBuf heat_t, heat_flags, heat_tbc, heat_val, heat_rhs, heat_cg, heat_red;
    pfg::DBuf heat_cg32, heat_rhs32;  // mixed precision: FP32 CG vectors and matrix values, FP32 residual
    pfg::DBuf hf_ptr, hf_ent, hf_fflags, heat_q;
    pfg::DBuf wch_rec;  // BoussinesqWC heat step: per element node lumped mass and right-hand side
    // fractional step: gauge nodes, the velocity matrix (CSR), L and M (node-pair layout), work
    // vectors, CG vectors and partial sums
    pfg::DBuf fs_gauge, fs_rp, fs_col, fs_val, fs_lval, fs_mval, fs_vec, fs_cg, fs_red;
    bool heat_ready = false;  // heat buffers allocated (and zeroed) for the current mesh
    bool has_heat_bc = false, has_heat_q = false;
    bool heat_facets_dirty = true;  // the per-node heat facet lists need rebuilding
    std::vector<uint8_t> h_heat_flags;
    std::vector<int32_t> h_facets, h_facet_elm;
    // device sparse LU of the plain form (PFG_LINSOLVE_LU): fronts, their nodes, assembly
    // records, children, boundary maps, pivots, dense front matrices and solve vectors, the
    // fronts of each tree level (deepest first; small ones batched, large ones blocked)
    pfg::DBuf lu_front, lu_nodes, lu_recs, lu_kids, lu_maps, lu_piv, lu_mat, lu_vec, lu_list, lu_r, lu_one;
    bool lu_ready = false;
    int lu_fronts = 0;
    size_t lu_factor_bytes = 0;
    std::vector<std::vector<int>> lu_levels, lu_large;
    std::vector<std::pair<int, int>> lu_small;
    std::vector<pfg::LuFront> h_lu_front;
};

namespace pfg {

// ---- allocation / error helpers (pfg_api.cu) -----------------------------------------
int fail(pfg_ctx* c, int code, const char* fmt, ...);
int cuda_fail(pfg_ctx* c, cudaError_t e, const char* what);
int ensure(pfg_ctx* c, DBuf& b, size_t bytes);
void release(DBuf& b);

template <class T>
inline T* ptr(const DBuf& b) {
    return static_cast<T*>(b.p);
}

#define PFG_CUDA(ctx, call)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return pfg::cuda_fail(ctx, e_, #call); \
    } while (0)

#define PFG_CHECK_LAUNCH(ctx) PFG_CUDA(ctx, cudaGetLastError())

// ---- phase timers (pfg_api.cu) ---------------------------------------------------------
enum Phase : int {
    PH_WC_PREDICT = 0,
    PH_WC_CONT_ELEM,
    PH_WC_CONT_NODE,
    PH_WC_MOM_ELEM,
    PH_WC_MOM_NODE,
    PH_WC_DT,
    PH_PSPG_ELEM,
    PH_PSPG_RHS,
    PH_PSPG_PAIRS,
    PH_KRYLOV_ITER,
    PH_RESIDUAL,
    PH_POSITIONS,
    PH_KRYLOV_SPMV,
    PH_MG_CYCLE,
    PH_MG_SETUP,
    PH_HEAT_ASSEMBLY,
    PH_HEAT_SPMV
};
void prof_begin(pfg_ctx* c, int phase);
void prof_end(pfg_ctx* c, int phase);
int prof_flush(pfg_ctx* c);

// ---- scans (pfg_mesh.cu) ---------------------------------------------------------------
// Exclusive prefix sum of n ints into out (n+1 entries; out[n] = total).  Uses tmp space.
int scan_exclusive(pfg_ctx* c, const int* in, int* out, int n, DBuf& tmp);

// ---- mesh build (pfg_mesh.cu) --------------------------------------------------------
int build_topology(pfg_ctx* c);

// ---- constants (pfg_api.cu) ----------------------------------------------------------
GaussConst gauss_const(int dim);
void upload_constants(int dim);

// ---- PSPG (pfg_pspg.cu) --------------------------------------------------------------
int pspg_alloc(pfg_ctx* c);
int pspg_assemble(pfg_ctx* c, double dt, const double* d_qiter, const double* d_qprev, bool apply_bc);
int pspg_elem_prep(pfg_ctx* c, double dt, const double* d_qiter);
// ---- fractional step (pfg_fracstep.cu) ----
int fs_alloc(pfg_ctx* c);
int fs_picard_step(pfg_ctx* c, double dt, pfg_step_status* st);
int pspg_update_positions(pfg_ctx* c, double dt, const double* d_q);
int pspg_residual(pfg_ctx* c, const double* d_q, double* res_out);
int picard_step(pfg_ctx* c, double dt, pfg_step_status* st);
int compute_geometry(pfg_ctx* c, double* d_detJ, double* d_invJ);
int volume(pfg_ctx* c, double* out);
int tip(pfg_ctx* c, int coord, int want_max, double* out);

// ---- Krylov (pfg_krylov.cu) ----------------------------------------------------------
int krylov_alloc(pfg_ctx* c);
// Solve A x = b (x in/out, device).  Returns iterations in *iters and ||b - A x|| in *res.
int bicgstab(pfg_ctx* c, double* d_x, int* iters, double* res);
int spmv_residual_norm(pfg_ctx* c, const double* d_x, double* res);

// ---- sparse LU, the plain form's direct solver (pfg_lu.cu) ------------------------------
int lu_solve(pfg_ctx* c, double* x, int* refine_sweeps);
void lu_release(pfg_ctx* c);

// ---- mixed-precision PSPG (pfg_pspg_mixed.cu) -----------------------------------------
int mx_alloc(pfg_ctx* c);
// ---- heat equation (pfg_heat.cu) ----
int heat_alloc(pfg_ctx* c);
int heat_build_facets(pfg_ctx* c);
int heat_step(pfg_ctx* c, double dt, pfg_step_status* st);
int wc_heat_prepare(pfg_ctx* c, bool* changed);
constexpr int CG_VECTORS = 6;  // work vectors of cg_solve
int cg_solve(pfg_ctx* c, int n, const int* rp, const int* col, const double* val, const double* b, double* x,
             double* V, double* red, double rtol, double atol, int max_it, int* iters, bool* ok);
int wc_heat_launch(pfg_ctx* c, const double* tdt);
int mx_set_instances(pfg_ctx* c, int n_inst, const int* node_off, const double* rho, const double* mu);
int mx_picard_step(pfg_ctx* c, const double* dts, pfg_step_status* st);
void mx_release_graph(pfg_ctx* c);

// ---- multigrid preconditioner (pfg_mg.cu) ---------------------------------------------
int mg_setup(pfg_ctx* c);
int mg_numeric(pfg_ctx* c);
void mg_apply(pfg_ctx* c, const float* b, float* out);
void mg_release(pfg_ctx* c);

// ---- WC (pfg_wc.cu) -------------------------------------------------------------------
int wc_alloc(pfg_ctx* c);
void wc_release_graphs(pfg_ctx* c);
int wc_set_states(pfg_ctx* c, const double* h);
int wc_get_states(pfg_ctx* c, double* h);
int wc_steps(pfg_ctx* c, double dt, int nsteps, pfg_step_status* st);
int wc_enqueue(pfg_ctx* c, double dt, int nsteps);
int wc_sync(pfg_ctx* c, pfg_step_status* st);
int wc_sync_batch(pfg_ctx* c, pfg_step_status* st);
int wc_next_dt(pfg_ctx* c, double* dt);
int wc_mass(pfg_ctx* c, double* out);
int wc_set_time(pfg_ctx* c, double time, double next_dt);
int wc_dirichlet_changed(pfg_ctx* c);
int wc_sync_positions(pfg_ctx* c);
// mixed form (pfg_wc_mixed.cu)
size_t wcm_state_bytes(pfg_ctx* c);
size_t wcm_elem_bytes(pfg_ctx* c);
int wcm_launch_step(pfg_ctx* c, bool adapt);
int wcm_positions_in(pfg_ctx* c);
int wcm_positions_out(pfg_ctx* c);
int wcm_set_states(pfg_ctx* c, const double* h);
int wcm_get_states(pfg_ctx* c, double* h);
int wcm_state_to_stage(pfg_ctx* c);
int wcm_vbc_refresh(pfg_ctx* c);
int wcm_next_dt(pfg_ctx* c);
int wcm_set_instances(pfg_ctx* c, int n_inst, const int* node_off, const double* mu);

}  // namespace pfg
