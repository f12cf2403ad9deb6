/*
 * pfem_gpu.h - C ABI of the GB300 PFEM per-time-step solve library (libpfemgpu.so).
 *
 * The library replaces the per-step work behind the reference's solver classes
 * (ImperatorS79/PFEM, paths relative to its project root):
 *
 *   Solver::solveOneTimeStep / computeNextDT      srcs/simulation/Solver.hpp:53,56
 *   Equation::solve / preCompute                  srcs/simulation/Equation.hpp:65,68
 *   Mesh geometry + position updates              srcs/mesh/Mesh.hpp:46-267
 *
 * A host-side solver subclass (C++, C or any FFI) keeps the reference's time loop and its
 * remeshing; after every remesh it hands this library the new connectivity and node arrays.
 *
 * Conventions
 *   - Every entry point returns an int status: 0 (PFG_OK) or a negative PFG_ERR_* code.
 *     Nothing throws across the ABI; pfg_last_error() gives the message of the last failure.
 *   - Numerical failure of a step (Picard not converged, NaN) is NOT an error code: it is
 *     reported in pfg_step_status.converged = 0, mirroring the reference's `bool` return
 *     (PicardAlgo.cpp:55-66,79-86).  The library then restores the saved node positions and
 *     states itself, like Mesh::restoreNodesList.
 *   - One context per host thread; each context owns one CUDA stream and all of its device
 *     memory.  Calls on one context must not overlap.
 *   - All host arrays are plain pointers: positions and fields are structure-of-arrays
 *     ("field-major"): x[d*N + n]; element connectivity conn[k*E + e], k = 0..dim.
 *   - The library never calls back into the host.
 */
#ifndef PFEM_GPU_H
#define PFEM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PFG_API __attribute__((visibility("default")))

/* ---- status codes ---------------------------------------------------------------- */
#define PFG_OK 0
#define PFG_ERR_INVALID (-1)     /* bad argument (sizes, indices, null pointers)          */
#define PFG_ERR_CUDA (-2)        /* a CUDA call failed                                     */
#define PFG_ERR_NOMEM (-3)       /* device allocation failed or HBM budget exceeded        */
#define PFG_ERR_STATE (-4)       /* call out of order (e.g. step before mesh upload)       */
#define PFG_ERR_UNSUPPORTED (-5) /* option not implemented for this configuration          */
#define PFG_ERR_DEVICE (-6)      /* a kernel reported an internal error (e.g. valence cap) */

/* ---- node flags (one byte per node) ------------------------------------------------ */
#define PFG_NODE_BOUND 1u        /* Node::isBound           srcs/mesh/Node.hpp:101        */
#define PFG_NODE_FREE_SURFACE 2u /* Node::isOnFreeSurface                                  */
#define PFG_NODE_FIXED 4u        /* Node::isFixed: position never updated                 */
#define PFG_NODE_DIRICHLET 8u    /* bound node whose tag has a velocity BC
                                    (Solver::m_bcTagFlags bit 0, Solver.hpp:78)            */
#define PFG_NODE_FREE 16u        /* output only: node in no element (Node::isFree)        */

/* ---- configuration --------------------------------------------------------------- */
typedef enum {
    PFG_KIND_INCOMP_PSPG = 0,  /* SolverIncompNewton, id "PSPG", problem IncompNewtonNoT  */
    PFG_KIND_WC_CDS_DPDT = 1   /* SolverWCompNewton, id "CDS_dpdt", problem WCompNewtonNoT */
} pfg_kind;

typedef enum {
    PFG_PREC_FP64 = 0,         /* plain form: FP64 everywhere                              */
    PFG_PREC_MIXED = 1         /* FP32 assembly/Krylov/state, FP64 geometry, refinement
                                  residual and global sums                                 */
} pfg_precision;

typedef enum {
    PFG_LINSOLVE_BICGSTAB = 0, /* Jacobi-preconditioned BiCGSTAB                           */
    PFG_LINSOLVE_LU = 1        /* device sparse LU (plain form; reference: Eigen SparseLU) */
} pfg_linsolve;

typedef enum {
    PFG_PC_BLOCK_JACOBI = 0,   /* node-block Jacobi                                         */
    PFG_PC_MULTIGRID = 1       /* node-aggregation multigrid V-cycle (mixed precision only;
                                  the FP64 form uses node-block Jacobi)                     */
} pfg_preconditioner;

/* Arithmetic of the mixed form's FP32 system (the correction solves' operator). */
typedef enum {
    PFG_ASM_FP32 = 0,        /* FP32 element arithmetic and FP32 sums                      */
    PFG_ASM_DOUBLE_FLOAT = 1 /* double-float element arithmetic, rounded to FP32 once       */
} pfg_assembly;

typedef enum {
    PFG_RES_AX_F = 0,          /* ||A q - b||_2            MomContEquationPSPG.inl:366-371 */
    PFG_RES_U = 1,             /* relative velocity change                        :319-342 */
    PFG_RES_U_P = 2,           /* max(rel. velocity change, rel. pressure change) :343-364 */
    PFG_RES_T = 3              /* heat: relative temperature change  HeatEquation.inl:153-180 */
} pfg_residual;

typedef struct pfg_params {
    int32_t dim;               /* 2 (triangles) or 3 (tetrahedra)                          */
    int32_t kind;              /* pfg_kind                                                 */
    int32_t precision;         /* pfg_precision                                            */
    int32_t linear_solver;     /* pfg_linsolve (incompressible only)                       */
    double gravity[3];         /* bodyForce                                                */
    double mu;                 /* dynamic viscosity (both kinds)                           */
    /* incompressible (MomContEq): */
    double rho;
    int32_t picard_max_iter;   /* maxIter                                                  */
    int32_t residual;          /* pfg_residual                                             */
    double picard_min_res;     /* minRes                                                   */
    int32_t krylov_max_iter;   /* per linear solve (mixed: per correction solve)           */
    int32_t refine_max_iter;   /* mixed: refinement sweeps per linear solve (0 = 30)       */
    double krylov_rel_tol;     /* stop when ||r|| <= max(rel_tol*||b||, abs_tol)           */
    double krylov_abs_tol;
    /* weakly compressible (ContEq + MomEq): */
    double K0, K0p, rho_star;  /* Tait-Murnaghan                                           */
    double security_coeff;     /* securityCoeff (CFL)                                      */
    double max_dt;             /* maxDT                                                    */
    int32_t meduri;            /* ContEq stabilization: 1 = "Meduri", 0 = "None"           */
    int32_t pad1;
    /* resources: */
    size_t hbm_budget_bytes;   /* 0 = no limit                                             */
    /* mixed precision, incompressible: */
    double inner_rel_tol;      /* FP32 correction solve stops at this fraction of its
                                  starting residual (0 = 1e-4; defaults: 1e-3 in 2D,
                                  5e-4 in 3D); a sweep that needs less to meet the linear
                                  solve's tolerance stops at 0.2 of the remaining reduction
                                  (at most 0.01)                                            */
    /* both kinds: */
    double gamma;              /* surface tension coefficient (MomContEq / MomEq "gamma");
                                  >= 1e-15 adds the facet term of m_applyBCPSPG
                                  (MomContEquationPSPG.inl:155-187) / MomEq::m_applyBC
                                  (MomEquation.inl:311-335) and needs pfg_upload_facets    */
    /* mixed precision, incompressible: */
    int32_t preconditioner;    /* pfg_preconditioner of the FP32 correction solves         */
    int32_t assembly;          /* pfg_assembly: arithmetic of the FP32 system's node blocks
                                  (the refinement residual is double-float either way)    */
    /* incompressible, Bingham fluid (problem "Bingham", MomContEquation.inl:54-58,102-121):
       tau0 > 0 makes the viscosity mu + tau0 (1 - exp(-m_reg gd)) / gd per element, gd the
       strain-rate norm of the Picard iterate                                             */
    double tau0;               /* yield stress (0 = Newtonian)                             */
    double m_reg;              /* regularisation parameter mReg                            */
    /* incompressible, heat equation (HeatEqIncompNewton, IncompNewton/HeatEquation.inl:27-32;
       problems "Conduction" and "Boussinesq"); used by pfg_heat_step:                      */
    double heat_k;             /* thermal conductivity k                                   */
    double heat_cv;            /* specific heat cv (the heat mass factor is cv rho)        */
    double heat_h;             /* convection coefficient h of the Qh facets                */
    double heat_t_inf;         /* ambient temperature Tinf of the Qh / Qr facets           */
    double heat_eps_rad;       /* emissivity epsRad of the Qr facets                       */
    int32_t heat_fs_flags;     /* pfg_heat_flag bits of the free-surface tag: PFG_HEAT_Q,
                                  PFG_HEAT_QH, PFG_HEAT_QR (FreeSurfaceQ / Qh / Qr)        */
    int32_t boussinesq;        /* 1: problem "Boussinesq" (MomContEquation.inl:164-199): the
                                  PSPG body force uses rho (1 - alpha (T - Tr)) and the
                                  pressure-row gravity term 1 - alpha (T - Tr) at each
                                  Gauss point, T the node temperatures                     */
    double alpha_t;            /* thermal expansion coefficient alpha                      */
    double t_ref;              /* reference temperature Tr                                 */
    double dgamma_dt;          /* Boussinesq: surface tension gamma + dgamma_dt (T - Tr) at
                                  the facet Gauss points (DgammaDT, MomContEquation.inl:
                                  174-179); the facet term runs when gamma or dgamma_dt is
                                  >= 1e-15 (MomContEquationPSPG.inl:157-158)              */
    /* heat equation Picard loop (HeatEq maxIter / minRes / residual) and phase change
       (HeatEquation.inl:36-45, 60-66, 421-425): with heat_phase_change the mass factor is
       (cv + dfl/dT(T) Lm) rho at the element Gauss points and each heat step iterates       */
    int32_t heat_max_iter;     /* maxIter                                                  */
    int32_t heat_residual;     /* PFG_RES_T or PFG_RES_AX_F                                */
    double heat_min_res;       /* minRes                                                   */
    int32_t heat_phase_change; /* 1: latent heat (Tm, DT, Lm given)                       */
    int32_t pad3;
    double heat_tm;            /* melting temperature Tm                                   */
    double heat_dt_melt;       /* melting range DT                                         */
    double heat_lm;            /* latent heat Lm                                           */
    /* weakly compressible problem "BoussinesqWC" (kind PFG_KIND_WC_CDS_DPDT with boussinesq =
       1, plain FP64 precision; WCompNewton/Solver.cpp:72-146, 278-320): every step runs the
       explicit lumped-mass heat step of HeatEqWCompNewton (heat_k, heat_cv with the node
       densities, the heat boundary conditions and facets of pfg_heat_set_bc / _set_flux; with
       heat_phase_change the latent heat heat_lm) between the half-step prediction and the
       continuity equation; the momentum body force uses rho (1 - alpha_t (T - t_ref)), the
       surface tension gamma + dgamma_dt (T - t_ref), and with heat_phase_change the
       Carman-Kozeny damping C (1 - fl)^2 / (fl^3 + eps) of MomEquation.inl:122-130 (fl the
       liquid fraction over heat_tm, heat_dt_melt); the CFL diffusion parameter is
       max(mu / rho, k / (cv rho)).  The temperatures are pfg_set_temperature's.              */
    double ck_c;               /* Carman-Kozeny constant C                                 */
    double ck_eps;             /* Carman-Kozeny eps                                        */
    /* incompressible, solver "FracStep" (MomContEquationFracStep.inl:7-630; plain FP64 form,
       residual PFG_RES_U or PFG_RES_U_P): per Picard iteration the velocity prediction
       (M/dt + K) v~ = F + M/dt v_prev + gamma_fs D^T p_prev, the pressure L p = -(rho/dt) D v~
       + gamma_fs L p_prev and the correction M dv = dt D^T (p - gamma_fs p_prev), each an SPD
       system solved by Jacobi CG to the Krylov tolerances.  As written in the reference, L is
       singular (free-surface nodes keep their Laplacian rows with a zero right-hand side): the
       smallest free-surface node of each connected group of elements (else its smallest node)
       is pinned to p = 0; fs_pressure_dirichlet = 1 pins every free-surface node instead.      */
    double gamma_fs;           /* gammaFS in [0, 1]                                        */
    int32_t frac_step;         /* 1: fractional step instead of PSPG                       */
    int32_t fs_pressure_dirichlet;
    /* weakly compressible, the continuity equation's form (the SolverWCompNewton id,
       WCompNewton/Solver.cpp:22-23; ContEquation.inl:123-302): pfg_wc_version.  The density
       forms run in the plain FP64 form.                                                     */
    int32_t wc_version;
    int32_t pad4;
} pfg_params;

/* Continuity forms of the weakly compressible solver. */
typedef enum {
    PFG_WC_DPDT = 0,           /* "CDS_dpdt": p from the lumped mass, D factor K0 + K0' p, free
                                  nodes p = 0; rho from Tait-Murnaghan                       */
    PFG_WC_RHO = 1,            /* "CDS_rho": rho = (lumped mass after the move)^-1 times the
                                  consistent mass before it times rho                        */
    PFG_WC_DRHODT = 2          /* "CDS_drhodt": rho from the lumped mass, D factor rho;
                                  both density forms: free and free-surface nodes take rho*,
                                  p from Tait-Murnaghan                                      */
} pfg_wc_version;

/* Heat boundary-condition flags per node (the reference's tag flags of HeatEq's BC table,
 * IncompNewton/Solver.cpp:132-170): T Dirichlet, Q prescribed flux, Qh convection, Qr
 * radiation.  A facet takes a flux term when all its nodes carry the flag; a free-surface
 * facet uses pfg_params.heat_fs_flags instead (HeatEquation.inl:319-335). */
typedef enum pfg_heat_flag {
    PFG_HEAT_T = 1,
    PFG_HEAT_Q = 2,
    PFG_HEAT_QH = 4,
    PFG_HEAT_QR = 8
} pfg_heat_flag;

typedef struct pfg_step_status {
    int32_t converged;         /* 1 = step accepted (reference: solveOneTimeStep() true)   */
    int32_t picard_iterations; /* Picard solves performed                                  */
    int32_t krylov_iterations; /* total Krylov iterations in the step                      */
    int32_t steps_done;        /* WC: explicit steps completed                             */
    double residual;           /* last Picard residual                                     */
    double dt;                 /* time step used by the last step                          */
    double time;               /* device-side simulated time after the call                */
    int32_t fp64_solves;       /* mixed incompressible: 1 when the correction solves ran in
                                  FP64 (FP32 ones stopped contracting for this mesh)       */
    int32_t pad0;
} pfg_step_status;

typedef struct pfg_ctx pfg_ctx;

/* Fill *p with the reference's dam-break defaults for `kind` and `dim`.
 * (damBreakKoshizukaIncomp.lua / damBreakKoshizukaComp.lua, examples/2D/damBreakKoshizuka) */
PFG_API int pfg_default_params(int32_t kind, int32_t dim, pfg_params* p);

/* Create a context on the current CUDA device.  Replaces the construction of the
 * Solver/Equation pair: SolverIncompNewton::SolverIncompNewton (IncompNewton/Solver.cpp:12-193)
 * and SolverWCompNewton::SolverWCompNewton (WCompNewton/Solver.cpp:15-165). */
PFG_API int pfg_create(const pfg_params* params, pfg_ctx** out);
PFG_API int pfg_destroy(pfg_ctx* ctx);
PFG_API const char* pfg_last_error(const pfg_ctx* ctx);   /* never NULL */

/* Hand the library a (re)meshed domain.  Replaces what Mesh::remesh leaves behind
 * (Mesh.cpp:919-926; triangulateAlphaShape2D/3D, Mesh2D.cpp:32-251, Mesh3D.cpp:36-286):
 * positions (dim x N), node flags, and (dim+1) x E positively oriented elements.  Rebuilds
 * the node-element incidence, node adjacency and the sparsity pattern on the device.
 * Node states are reset to zero; set them with pfg_set_states afterwards. */
PFG_API int pfg_upload_mesh(pfg_ctx* ctx, int32_t n_nodes, const double* pos, const uint8_t* flags,
                            int32_t n_elems, const int32_t* conn);
/* pfg_upload_mesh keeping the node states on the device (incompressible contexts): new node j
 * takes the states (and temperature) of origin[j*width + 0], or the mean of the valid entries
 * origin[j*width + k] (-1 padded; the centroid node Mesh::addNodes creates takes the mean of its
 * element's nodes, Mesh.cpp:59-67).  The table comes from the host remesh; the states never
 * cross to the host.  width <= 4. */
PFG_API int pfg_upload_mesh_remap(pfg_ctx* ctx, int32_t n_nodes, const double* pos, const uint8_t* flags,
                                  int32_t n_elems, const int32_t* conn, const int32_t* origin, int32_t width);

/* The boundary facets of the uploaded mesh (Mesh::m_facetsList, built by the alpha shape in
 * Mesh2D.cpp:199-244 / Mesh3D.cpp:232-282): facets[k*F + f] (k < dim) are the nodes of facet
 * f and facet_elm[f] the element it belongs to (Facet::m_elementIndex).  Needed, after every
 * pfg_upload_mesh, when params.gamma >= 1e-15: the surface tension term is evaluated on the
 * facets that touch the free surface (PFG_NODE_FREE_SURFACE).  Every facet node must be a node
 * of its element. */
PFG_API int pfg_upload_facets(pfg_ctx* ctx, int32_t n_facets, const int32_t* facets, const int32_t* facet_elm);

/* Node states, field-major.  Incompressible: (dim+1)*N values [v_0..v_{d-1}, p]
 * (getQFromNodesStates / setNodesStatesfromQ, StatesFromToQ.hpp:9-34).
 * WC: (2*dim+2)*N values [v, p, rho, a] (WCompNewton/Problem.cpp:18). */
PFG_API int pfg_set_states(pfg_ctx* ctx, const double* states);
PFG_API int pfg_get_states(pfg_ctx* ctx, double* states);
PFG_API int pfg_get_positions(pfg_ctx* ctx, double* pos);          /* dim*N */
/* Replace the node positions (dim*N) and keep the connectivity and the states, as
 * Mesh::restoreNodesList does with a saved node list (Mesh.cpp:1019-1053), or for a host that
 * moves nodes without remeshing. */
PFG_API int pfg_set_positions(pfg_ctx* ctx, const double* pos);
PFG_API int pfg_get_flags(pfg_ctx* ctx, uint8_t* flags);           /* N, PFG_NODE_FREE set */

/* Dirichlet velocities V_bc(pos, t + dt) of n Dirichlet nodes, values[d*n + i] (field-major
 * over the listed nodes).  Stands in for the Lua BoundaryV calls of m_applyBCPSPG
 * (MomContEquationPSPG.inl:206-231) and MomEqWCompNewton::m_applyBC (MomEquation.inl:355-371).
 * Nodes not listed keep their previous value (initially 0). */
PFG_API int pfg_set_dirichlet(pfg_ctx* ctx, int32_t n, const int32_t* nodes, const double* values);

/* One incompressible PSPG time step: MomContEqIncompNewton::solve + PicardAlgo::solve
 * (MomContEquation.inl:287-309 [.inl offsets], PicardAlgo.cpp:31-95,
 * MomContEquationPSPG.inl:261-373).  On non-convergence the positions and states are
 * restored and status->converged = 0.
 * precision = PFG_PREC_MIXED: FP32 assembly and FP32 correction solves, with every residual
 * (refinement and Picard) evaluated in FP64 from the element formulas; the linear solves stop
 * on the same FP64 residual test as the plain form. */
PFG_API int pfg_picard_step(pfg_ctx* ctx, double dt, pfg_step_status* status);

/* Device memory currently held by the context, in bytes (for admission control by callers
 * that run several contexts under one HBM budget). */
PFG_API int pfg_device_bytes(const pfg_ctx* ctx, size_t* bytes);

/* Batches (mixed precision, incompressible): the uploaded mesh is the union of n_inst
 * independent meshes stored back to back, instance i owning nodes
 * [node_offsets[i], node_offsets[i+1]) and only elements among them.  rho[i], mu[i] are the
 * instance's fluid parameters (gamma is shared).  No reference counterpart: the reference runs
 * one Problem per process; this replaces n_inst independent SolverIncompNewton objects.
 * Also for weakly compressible contexts in mixed precision (pfg_wc_step_batch): there mu[i] is
 * per instance, rho[i] must equal rho_star, and surface tension is not available. */
PFG_API int pfg_set_instances(pfg_ctx* ctx, int32_t n_inst, const int32_t* node_offsets, const double* rho,
                              const double* mu);
/* One Picard time step of every instance at once (instance i with time step dt[i]); each
 * instance converges, fails and restores on its own, exactly as pfg_picard_step would
 * alone.  status[i] receives instance i's result. */
PFG_API int pfg_picard_step_batch(pfg_ctx* ctx, const double* dt, pfg_step_status* status);

/* nsteps weakly compressible CDS_dpdt steps (WCompNewton/Solver.cpp:236-276 without the
 * remesh).  dt > 0 uses that fixed step for every step; dt <= 0 uses the device-side CFL step
 * of computeNextDT (WCompNewton/Solver.cpp:192-234), which is refreshed after every step.
 * Returns after all steps with a single host synchronisation. */
PFG_API int pfg_wc_step(pfg_ctx* ctx, double dt, int32_t nsteps, pfg_step_status* status);

/* Batched weakly compressible steps (mixed precision): after pfg_set_instances on a WC context,
 * every instance steps at once with its own CFL time step (dt <= 0) or the shared fixed dt,
 * each exactly as it would alone; status[i] receives instance i's dt and time.  The reference
 * runs one Problem per process; this replaces n_inst independent SolverWCompNewton objects. */
PFG_API int pfg_wc_step_batch(pfg_ctx* ctx, double dt, int32_t nsteps, pfg_step_status* status);

/* Asynchronous form of pfg_wc_step: enqueues nsteps steps on the context's stream and returns
 * without waiting.  pfg_synchronize waits for all enqueued work and fills the status (dt and
 * time of the last step).  Lets a caller keep the GPU busy while it prepares other work. */
PFG_API int pfg_wc_step_async(pfg_ctx* ctx, double dt, int32_t nsteps);
PFG_API int pfg_synchronize(pfg_ctx* ctx, pfg_step_status* status);
/* The CUDA stream (cudaStream_t) every kernel of this context is launched on, for callers
 * that order their own GPU work against the library's. */
PFG_API int pfg_get_stream(pfg_ctx* ctx, void** stream);

/* CFL time step of the current WC state (SolverWCompNewton::computeNextDT). */
PFG_API int pfg_next_dt(pfg_ctx* ctx, double* dt);
/* CFL time step computed without allocating any device memory.  This entry point has no
 * counterpart in the reference; it serves callers that may not call cudaMalloc when they need
 * a time step (a host application whose pool allocator owns all device memory, a time loop
 * running under another component's stream capture, a plugin that only receives device
 * pointers).  Same result as pfg_next_dt on an FP64 weakly compressible context, computed from
 * caller-owned device arrays: d_conn ((dim+1) x E int32), d_pos (dim x N), d_states
 * ((2 dim + 2) x N, [v, p, rho, a]); the step goes to the device double *d_dt.  Uses
 * params->dim, K0, K0p, mu, security_coeff, max_dt.  Work is enqueued on `stream`
 * (cudaStream_t, NULL = default stream); the caller synchronises.  Scratch is one static device
 * array for at most 1,048,576 nodes (16 MiB, held by every device that loads the library until
 * exit); larger meshes return PFG_ERR_INVALID.  All calls share that array, so calls that
 * overlap on the GPU race.  The first call on a device looks up the array's address and should
 * come before any stream capture; that address is kept for the life of the process, so do not
 * call cudaDeviceReset (or otherwise destroy and recreate the device's primary context) between
 * calls.  The caller owns the validation of d_conn: every index must lie in [0, n_nodes), and
 * none is checked here (checking would need a device pass of its own).  As in the reference's
 * loop, where std::min drops a NaN candidate (WCompNewton/Solver.cpp:222), an element with a
 * NaN state or position is skipped by the minimum, so the step stays finite; a caller that must
 * detect a non-finite state checks the states themselves (pfg_next_dt behaves the same way). */
PFG_API int pfg_wc_next_dt_noalloc(const pfg_params* params, int32_t n_nodes, int32_t n_elems,
                                   const int32_t* d_conn, const double* d_pos, const double* d_states,
                                   double* d_dt, void* stream);

/* Device-side time-step seed for pfg_wc_step(dt <= 0) (Solver::m_initialDT). */
PFG_API int pfg_set_time(pfg_ctx* ctx, double time, double next_dt);

/* Global sums and extractor values, reduced on the device in FP64:
 *   volume  = sum |e|                    (ProbIncompNewton mass, IncompNewton/Problem.cpp:173-189)
 *   mass    = sum |e| * mean(rho)        (ProbWCompNewton mass, WCompNewton/Problem.cpp:216-244)
 *   tip     = max/min coordinate over non-bound, non-free nodes (MinMaxExtractor.cpp:28-62) */
PFG_API int pfg_volume(pfg_ctx* ctx, double* volume);
PFG_API int pfg_mass(pfg_ctx* ctx, double* mass);
PFG_API int pfg_tip(pfg_ctx* ctx, int32_t coord, int32_t want_max, double* value);

/* ---- inspection (parity tests) ---------------------------------------------------- */
/* Assemble the PSPG system at the current positions: element tau from q_iter, right-hand
 * side from q_prev (m_buildAbPSPG, MomContEquationPSPG.inl:6-146), then, when apply_bc != 0,
 * m_applyBCPSPG (:148-235).  NULL q_iter / q_prev use the current device states. */
PFG_API int pfg_pspg_assemble(pfg_ctx* ctx, double dt, const double* q_iter, const double* q_prev,
                              int32_t apply_bc);
/* Read the assembled system in CSR form.  Call with NULL arrays to get *n_rows and *nnz. */
PFG_API int pfg_get_csr(pfg_ctx* ctx, int32_t* n_rows, int64_t* nnz, int64_t* row_ptr, int32_t* col_idx,
                        double* values, double* rhs);
/* Element geometry of the current positions: detJ[E], invJ[E*9] (row-major 3x3). */
PFG_API int pfg_get_geometry(pfg_ctx* ctx, double* detJ, double* invJ);
/* Solve A x = b for the assembled system with the configured linear solver (x: initial guess
 * in, solution out, length R).  Returns iterations and the final ||A x - b|| in *res. */
PFG_API int pfg_linear_solve(pfg_ctx* ctx, double* x, int32_t* iterations, double* res);

/* ---- phase timers ----------------------------------------------------------------- */
/* GPU time per phase of the path, measured with CUDA events on the context's stream while
 * profiling is enabled.  Mirrors the reference's per-category timers (Solver::m_accumalatedTimes,
 * Solver.hpp:253, printed by Solver::displayTimeStats, Solver.cpp:79-91).  Phases:
 *   0 WC predict            1 WC continuity/element   2 WC continuity/node
 *   3 WC momentum/element   4 WC momentum/node        5 WC time step
 *   6 PSPG element prep     7 PSPG right-hand side    8 PSPG matrix (node pairs)
 *   9 Krylov iteration     10 Picard residual        11 position update
 *  12 Krylov SpMV (the two products of an iteration, also inside phase 9)
 *  13 Multigrid cycle (the preconditioner applies of an iteration, also inside phase 9)
 *  14 Multigrid setup (coarse values and block inverses after each assembly)
 *  15 Heat assembly        16 Heat CG SpMV (the product of each conjugate-gradient step) */
#define PFG_NUM_PHASES 17
PFG_API int pfg_set_profiling(pfg_ctx* ctx, int32_t enable);
/* Accumulated milliseconds and launch counts per phase since the last reset. */
PFG_API int pfg_get_phase_times(pfg_ctx* ctx, double* ms, int64_t* launches);
PFG_API int pfg_reset_phase_times(pfg_ctx* ctx);
/* ---- Heat equation and Boussinesq coupling (incompressible contexts) --------------------
 * The temperature is one value per node (the reference's state dim+1 of a Boussinesq problem,
 * state 0 of a Conduction problem), kept on the device next to the flow states.  Node
 * temperatures are reset to zero by pfg_upload_mesh. */
PFG_API int pfg_set_temperature(pfg_ctx* ctx, const double* T);   /* N values */
PFG_API int pfg_get_temperature(pfg_ctx* ctx, double* T);
/* Heat boundary conditions: flags[n] (pfg_heat_flag bits) and the Dirichlet temperature
 * t_dirichlet[n] of PFG_HEAT_T nodes (the "T" BC function evaluated by the caller at the
 * node position and time t + dt, HeatEquation.inl:384-389).  Needs the facets of the mesh
 * (pfg_upload_facets) when any node or heat_fs_flags has a flux flag.  Replaces the BC
 * evaluation of HeatEqIncompNewton::m_applyBC (:307-394). */
PFG_API int pfg_heat_set_bc(pfg_ctx* ctx, const uint8_t* flags, const double* t_dirichlet);
/* Prescribed heat flux vectors at the three Gauss points of every facet: q_gp[(f*3 + g)*dim
 * + d] (the "Q" BC function at Facet::getPosFromGP, time t + dt; MatricesBuilder.inl:
 * 246-272).  Read for the facets that take the Q term; NULL clears it. */
PFG_API int pfg_heat_set_flux(pfg_ctx* ctx, const double* q_gp);
/* One HeatEqIncompNewton::solve without phase change (one Picard pass, HeatEquation.inl:
 * 195-196, 216-224): assembles (cv rho M + dt k L) T = cv rho M T_prev + boundary terms at
 * the current positions, solves it (FP64 conjugate gradients, Jacobi preconditioner, to the
 * Krylov tolerances of the params) and replaces the node temperatures.  On failure the
 * temperatures are unchanged.  st->krylov_iterations and st->residual report the solve. */
PFG_API int pfg_heat_step(pfg_ctx* ctx, double dt, pfg_step_status* st);

/* ---- Launch tuning of the mixed incompressible form ---------------------------------------
 * Launch shapes of the kernels whose best shape depends on the mesh and the device: lanes per
 * node of the Krylov SpMV and of the multigrid's level-0 sweeps (node_lanes / 2, node_lanes or
 * 2 node_lanes, node_lanes = 4 in 2D and 8 in 3D); the pair assembly's form: 128 = row-staged (one thread per node
 * pair, 128 pairs per block, their rows' element records staged in shared memory; the 3D
 * default), 64 = pair-parallel reading the element records from global memory (the 2D
 * default), 256 = item-parallel (one
 * thread per pair element item, 256 items per block); threads
 * per block of the element prep (64, 128 or 256) and of the refinement residual's element
 * kernel (32 or 64).  A zero field keeps the current value.  The FP32 system depends on the
 * pair assembly's form through its FP32 rounding only, the solution (set by the double-float
 * refinement residual) on none of them.  pfem_gb300.tune sweeps these through a step from a
 * saved state and caches the choice per device, dimension and mesh size. */
typedef struct pfg_tuning {
    int32_t spmv_lanes;
    int32_t pair_block;
    int32_t elem_block;
    int32_t res_block;
    int32_t mg_lanes;          /* lanes per node of the multigrid's level-0 sweeps (as spmv_lanes) */
} pfg_tuning;
PFG_API int pfg_set_tuning(pfg_ctx* ctx, const pfg_tuning* t);
PFG_API int pfg_get_tuning(pfg_ctx* ctx, pfg_tuning* t);

/* Node pairs ((d+1)^2 blocks) read by the timed Krylov SpMV launches (phase 12) since the last
 * reset: the algorithmic work of those launches in a batch whose converged instances drop out
 * of the products (mixed precision; the plain FP64 form reports 0). */
PFG_API int pfg_get_spmv_pairs(pfg_ctx* ctx, int64_t* pairs);
PFG_API const char* pfg_phase_name(int32_t phase);

/* Library version string. */
PFG_API const char* pfg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PFEM_GPU_H */
