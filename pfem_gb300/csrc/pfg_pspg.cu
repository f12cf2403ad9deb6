// Incompressible PSPG P1-P1 assembly, boundary conditions and the Picard loop.
//
// Reference: MomContEqIncompNewton (srcs/simulation/physics/IncompNewton/MomContEquation*.inl)
// and PicardAlgo (srcs/simulation/nonLinearAlgo/PicardAlgo.cpp).
//
// Assembly is a gather over node pairs instead of an element scatter: thread t owns the
// (dim+1)x(dim+1) block of rows (n, *) and columns (m, *) for one pair (n, m) of the node
// adjacency.  It walks the elements of n in ascending element order, keeps the ones that also
// contain m, and adds their element-matrix entries in registers.  Each CSR value is therefore
// written exactly once, without atomics, and its element contributions are summed in the
// same order as Eigen's setFromTriplets sums the reference's triplets (element order).
//
// Element formulas: pfg_pspg_common.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "pfg_device.cuh"
#include "pfg_internal.cuh"
#include "pfg_pspg_common.cuh"

namespace pfg {

namespace {

// m_computeTauPSPG (MomContEquationPSPG.inl:237-259) and the geometry recompute of
// Mesh::updateNodesPositionFromSave (Mesh.cpp:1258-1264), one thread per element.
template <int DIM>
__global__ void k_elem_prep(int E, int N, const int* __restrict__ conn, const double* __restrict__ pos,
                            const double* __restrict__ q_iter, double rho, double mu, double dt, double refSize,
                            ViscArgs va, double* __restrict__ ed) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[DIM + 1];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    compute_geom<DIM>(pos, N, nd, g);
    double G[DIM][DIM + 1];
    grad_n<DIM>(g, G);
    const double h = sqrt(refSize * g.detJ / M_PI);
    double U = 0;
#pragma unroll
    for (int k = 0; k <= DIM; ++k) {
        double nodeU = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const double v = q_iter[(size_t)d * N + nd[k]];
            nodeU += v * v;
        }
        U += sqrt(nodeU);
    }
    U /= (DIM + 1);
    const double a = 2 / dt, b = 2 * U / h, c = 4 * mu / (h * h * rho);
    const double tau = 1 / sqrt(a * a + b * b + 9 * c * c);
    ed[e] = g.detJ;
    ed[(size_t)E + e] = tau;
#pragma unroll
    for (int f = 0; f < DIM; ++f)
#pragma unroll
        for (int i = 0; i <= DIM; ++i) ed[(size_t)(2 + f * (DIM + 1) + i) * E + e] = G[f][i];
    ed[(size_t)ed_ksum<DIM>() * E + e] = k_sum<DIM>(va, mu, G, q_iter, N, nd);
}

struct PspgConst {
    PspgCoef c;
    PspgTables t;
    BoussArgs bq;
};

// Matrix values, one thread per node pair (n, m).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_pspg_pairs(int P, int N, int E, const int* __restrict__ pair_node,
                                                      const int* __restrict__ nbr_ptr, const int* __restrict__ nbr,
                                                      const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                                                      const uint8_t* __restrict__ ne_loc,
                                                      const int* __restrict__ conn, const double* __restrict__ ed,
                                                      const uint8_t* __restrict__ flags,
                                                      const int* __restrict__ row_ptr, double* __restrict__ val,
                                                      const double* __restrict__ vbc, double* __restrict__ rhs,
                                                      int apply_bc, PspgConst k) {
    constexpr int NPE = DIM + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P) return;
    const int n = pair_node[t];
    const int b0 = nbr_ptr[n];
    const int deg = nbr_ptr[n + 1] - b0;
    const int rank = t - b0;
    const int m = nbr[t];
    const uint8_t fn = flags[n];
    if (fn & F_FREE) {  // identity rows (MomContEquationPSPG.inl:112-127)
#pragma unroll
        for (int f = 0; f <= DIM; ++f) val[row_ptr[n + f * N]] = 1.0;
        return;
    }
    double acc[NPE][NPE];
    pspg_pair_block<DIM>(n, m, E, ne_ptr, ne_elem, ne_loc, conn, ed, k.c, k.t, acc);
    pspg_write_block<DIM>(n, m, N, deg, rank, fn, flags[m], row_ptr, acc, apply_bc != 0, vbc, rhs, val, nullptr);
}

// Right-hand side and node boundary conditions, one thread per node (doublet scatter
// :93-97,:140-144 in element order, then m_applyBCPSPG :189-232).
template <int DIM>
__global__ void k_pspg_rhs(int N, int E, const int* __restrict__ ne_ptr, const int* __restrict__ ne_elem,
                           const uint8_t* __restrict__ ne_loc, const int* __restrict__ conn,
                           const double* __restrict__ ed, const uint8_t* __restrict__ flags,
                           const double* __restrict__ q_prev, const double* __restrict__ vbc,
                           double* __restrict__ rhs, int apply_bc, PspgConst k, const double* __restrict__ fst) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double bv[DIM], bp;
    pspg_node_rhs<DIM>(n, N, E, ne_ptr, ne_elem, ne_loc, conn, ed, flags[n], q_prev, vbc, apply_bc != 0, k.c, k.t, fst, k.bq,
                       bv, bp);
#pragma unroll
    for (int f = 0; f < DIM; ++f) rhs[(size_t)f * N + n] = bv[f];
    rhs[(size_t)DIM * N + n] = bp;
}

// x = x_save + dt * v for non-fixed nodes (Mesh::updateNodesPositionFromSave, Mesh.cpp:1246-1256)
template <int DIM>
__global__ void k_positions_from_save(int N, const uint8_t* __restrict__ flags, const double* __restrict__ save,
                                      const double* __restrict__ q, double dt, double* __restrict__ pos) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    if (flags[n] & F_FIXED) return;
#pragma unroll
    for (int d = 0; d < DIM; ++d) pos[(size_t)d * N + n] = save[(size_t)d * N + n] + q[(size_t)d * N + n] * dt;
}

template <int DIM>
__global__ void k_geometry_out(int E, int N, const int* __restrict__ conn, const double* __restrict__ pos,
                               double* __restrict__ detJ, double* __restrict__ invJ) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int nd[DIM + 1];
    load_nodes<DIM>(conn, E, e, nd);
    Geom<DIM> g;
    compute_geom<DIM>(pos, N, nd, g);
    detJ[e] = g.detJ;
    for (int r = 0; r < 3; ++r)
        for (int cc = 0; cc < 3; ++cc) invJ[(size_t)9 * e + 3 * r + cc] = (r < DIM && cc < DIM) ? g.invJ[r][cc] : 0.0;
}

template <int DIM>
__global__ void k_volume(int E, int N, const int* __restrict__ conn, const double* __restrict__ pos, double refSize,
                         double* partials, unsigned* ticket, double* out) {
    __shared__ double sh[32];
    double s = 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        int nd[DIM + 1];
        load_nodes<DIM>(conn, E, e, nd);
        Geom<DIM> g;
        compute_geom<DIM>(pos, N, nd, g);
        s += g.detJ * refSize;
    }
    grid_sum_last<BLOCK>(s, partials, ticket, sh, out);
}

// MinMaxExtractor::update (extractors/MinMaxExtractor.cpp:37-56); max starts at 0 like the
// reference, min at DBL_MAX.
__global__ void k_tip(int N, const uint8_t* __restrict__ flags, const double* __restrict__ x, int want_max,
                      double* out) {
    __shared__ double sh[32];
    double v = want_max ? 0.0 : 1.79769313486231570e308;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const uint8_t f = flags[n];
        if (!(f & F_BOUND) && !(f & F_FREE)) v = want_max ? fmax(v, x[n]) : fmin(v, x[n]);
    }
    v = want_max ? block_max<BLOCK>(v, sh) : block_min<BLOCK>(v, sh);
    if (threadIdx.x == 0) {
        // positive and negative doubles: order-preserving integer key
        long long bits = __double_as_longlong(v);
        long long key = bits >= 0 ? bits : (bits ^ 0x7fffffffffffffffLL);
        if (want_max)
            atomicMax(reinterpret_cast<long long*>(out), key);
        else
            atomicMin(reinterpret_cast<long long*>(out), key);
    }
}

PspgConst make_const(pfg_ctx* c, double dt) {
    const GaussConst g = gauss_const(c->dim);
    PspgConst k{};
    k.c.rho = c->prm.rho;
    k.c.dt = dt;
    k.c.refSize = g.refSize;
    k.c.mu_sum = 0;
    k.c.l_sum = 0;
    k.c.h_sum = 0;
    for (int q = 0; q < g.n; ++q) {
        k.c.mu_sum += c->prm.mu * g.w[q];
        k.c.l_sum += (1 / c->prm.rho) * g.w[q];
        k.c.h_sum += 1.0 * g.w[q];
    }
    for (int i = 0; i < 4; ++i) {
        k.t.s[i] = g.s[i];
        for (int j = 0; j < 4; ++j) k.t.MM[i][j] = g.MM[i][j];
    }
    for (int f = 0; f < 3; ++f) k.t.g[f] = c->prm.gravity[f];
    k.bq = boussinesq_args(c);
    return k;
}

template <int DIM>
int assemble_dim(pfg_ctx* c, double dt, const double* d_qiter, const double* d_qprev, bool apply_bc) {
    const int N = c->N, E = c->E;
    const GaussConst g = gauss_const(DIM);
    if (E > 0) {
        prof_begin(c, PH_PSPG_ELEM);
        k_elem_prep<DIM><<<div_up(E, BLOCK), BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos),
                                                                    d_qiter, c->prm.rho, c->prm.mu, dt, g.refSize,
                                                                    visc_args(c), ptr<double>(c->edata));
        prof_end(c, PH_PSPG_ELEM);
        PFG_CHECK_LAUNCH(c);
    }
    const PspgConst k = make_const(c, dt);
    prof_begin(c, PH_PSPG_RHS);
    const FstArgs fa = fst_args(c);
    if (fa.nodes && apply_bc)
        k_fst<DIM, double><<<div_up(fa.n_nodes, BLOCK), BLOCK, 0, c->stream>>>(
            fa, E, ptr<int>(c->conn), PosF64{ptr<double>(c->pos), N}, N, ptr<double>(c->fst_force));
    k_pspg_rhs<DIM><<<div_up(N, BLOCK), BLOCK, 0, c->stream>>>(
        N, E, ptr<int>(c->ne_ptr), ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn),
        ptr<double>(c->edata), ptr<uint8_t>(c->flags), d_qprev, ptr<double>(c->vbc), ptr<double>(c->rhs),
        apply_bc ? 1 : 0, k, fst_force<double>(c));
    prof_end(c, PH_PSPG_RHS);
    PFG_CHECK_LAUNCH(c);
    prof_begin(c, PH_PSPG_PAIRS);
    k_pspg_pairs<DIM><<<div_up(c->P, BLOCK), BLOCK, 0, c->stream>>>(
        c->P, N, E, ptr<int>(c->pair_node), ptr<int>(c->nbr_ptr), ptr<int>(c->nbr), ptr<int>(c->ne_ptr),
        ptr<int>(c->ne_elem), ptr<uint8_t>(c->ne_loc), ptr<int>(c->conn), ptr<double>(c->edata),
        ptr<uint8_t>(c->flags), ptr<int>(c->row_ptr), ptr<double>(c->val), ptr<double>(c->vbc),
        ptr<double>(c->rhs), apply_bc ? 1 : 0, k);
    prof_end(c, PH_PSPG_PAIRS);
    PFG_CHECK_LAUNCH(c);
    c->has_system = true;
    return PFG_OK;
}

}  // namespace

int pspg_alloc(pfg_ctx* c) {
    const size_t R = c->R, E = std::max(c->E, 1), N = c->N;
    const int ned = c->dim == 2 ? ed_count<2>() : ed_count<3>();
    int rc;
    if ((rc = ensure(c, c->val, sizeof(double) * (size_t)std::max<int64_t>(c->nnz, 1))) ||
        (rc = ensure(c, c->rhs, sizeof(double) * R)) || (rc = ensure(c, c->edata, sizeof(double) * ned * E)) ||
        (rc = ensure(c, c->q, sizeof(double) * R)) || (rc = ensure(c, c->q_prev, sizeof(double) * R)) ||
        (rc = ensure(c, c->q_iter_prev, sizeof(double) * R)))
        return rc;
    PFG_CUDA(c, cudaMemsetAsync(c->q.p, 0, sizeof(double) * R, c->stream));
    (void)N;
    return PFG_OK;
}

// Element data [detJ, tau, gradN, ksum] of the current positions into edata (the fractional
// step uses detJ, gradN and ksum).
int pspg_elem_prep(pfg_ctx* c, double dt, const double* d_qiter) {
    const int N = c->N, E = c->E;
    if (E == 0) return PFG_OK;
    const GaussConst g = gauss_const(c->dim);
    prof_begin(c, PH_PSPG_ELEM);
    if (c->dim == 2)
        k_elem_prep<2><<<div_up(E, BLOCK), BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), d_qiter,
                                                                  c->prm.rho, c->prm.mu, dt, g.refSize, visc_args(c),
                                                                  ptr<double>(c->edata));
    else
        k_elem_prep<3><<<div_up(E, BLOCK), BLOCK, 0, c->stream>>>(E, N, ptr<int>(c->conn), ptr<double>(c->pos), d_qiter,
                                                                  c->prm.rho, c->prm.mu, dt, g.refSize, visc_args(c),
                                                                  ptr<double>(c->edata));
    prof_end(c, PH_PSPG_ELEM);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

int pspg_assemble(pfg_ctx* c, double dt, const double* d_qiter, const double* d_qprev, bool apply_bc) {
    return c->dim == 2 ? assemble_dim<2>(c, dt, d_qiter, d_qprev, apply_bc)
                       : assemble_dim<3>(c, dt, d_qiter, d_qprev, apply_bc);
}

int pspg_update_positions(pfg_ctx* c, double dt, const double* d_q) {
    prof_begin(c, PH_POSITIONS);
    if (c->dim == 2)
        k_positions_from_save<2><<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(
            c->N, ptr<uint8_t>(c->flags), ptr<double>(c->pos_save), d_q, dt, ptr<double>(c->pos));
    else
        k_positions_from_save<3><<<div_up(c->N, BLOCK), BLOCK, 0, c->stream>>>(
            c->N, ptr<uint8_t>(c->flags), ptr<double>(c->pos_save), d_q, dt, ptr<double>(c->pos));
    prof_end(c, PH_POSITIONS);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

int compute_geometry(pfg_ctx* c, double* d_detJ, double* d_invJ) {
    if (c->E == 0) return PFG_OK;
    if (c->dim == 2)
        k_geometry_out<2><<<div_up(c->E, BLOCK), BLOCK, 0, c->stream>>>(c->E, c->N, ptr<int>(c->conn),
                                                                       ptr<double>(c->pos), d_detJ, d_invJ);
    else
        k_geometry_out<3><<<div_up(c->E, BLOCK), BLOCK, 0, c->stream>>>(c->E, c->N, ptr<int>(c->conn),
                                                                       ptr<double>(c->pos), d_detJ, d_invJ);
    PFG_CHECK_LAUNCH(c);
    return PFG_OK;
}

int volume(pfg_ctx* c, double* out) {
    double* red = ptr<double>(c->red);
    double* partials = red;
    double* res = red + c->max_grid * 4 + 8;
    unsigned* ticket = reinterpret_cast<unsigned*>(red + c->max_grid * 4 + 16);
    const GaussConst g = gauss_const(c->dim);
    const int grid = std::max(1, std::min(c->max_grid, div_up(std::max(c->E, 1), BLOCK)));
    if (c->dim == 2)
        k_volume<2><<<grid, BLOCK, 0, c->stream>>>(c->E, c->N, ptr<int>(c->conn), ptr<double>(c->pos), g.refSize,
                                                   partials, ticket, res);
    else
        k_volume<3><<<grid, BLOCK, 0, c->stream>>>(c->E, c->N, ptr<int>(c->conn), ptr<double>(c->pos), g.refSize,
                                                   partials, ticket, res);
    PFG_CHECK_LAUNCH(c);
    PFG_CUDA(c, cudaMemcpyAsync(c->h_scalars, res, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    *out = c->h_scalars[0];
    return PFG_OK;
}

int tip(pfg_ctx* c, int coord, int want_max, double* out) {
    double* red = ptr<double>(c->red);
    long long* key = reinterpret_cast<long long*>(red + c->max_grid * 4 + 24);
    const double init = want_max ? 0.0 : 1.79769313486231570e308;
    long long ib;
    std::memcpy(&ib, &init, sizeof(ib));  // both inits are non-negative doubles: key == bits
    PFG_CUDA(c, cudaMemcpyAsync(key, &ib, sizeof(ib), cudaMemcpyHostToDevice, c->stream));
    const int grid = std::max(1, std::min(c->max_grid, div_up(c->N, BLOCK)));
    k_tip<<<grid, BLOCK, 0, c->stream>>>(c->N, ptr<uint8_t>(c->flags), ptr<double>(c->pos) + (size_t)coord * c->N,
                                         want_max, reinterpret_cast<double*>(key));
    PFG_CHECK_LAUNCH(c);
    long long kb = 0;
    PFG_CUDA(c, cudaMemcpyAsync(&kb, key, sizeof(kb), cudaMemcpyDeviceToHost, c->stream));
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    long long bits = kb >= 0 ? kb : (kb ^ 0x7fffffffffffffffLL);
    std::memcpy(out, &bits, sizeof(double));
    return PFG_OK;
}

// PicardAlgo::solve (PicardAlgo.cpp:31-95) with the PSPG closures (MomContEquationPSPG.inl:261-373).
int picard_step(pfg_ctx* c, double dt, pfg_step_status* st) {
    const size_t R = c->R;
    std::memset(st, 0, sizeof(*st));
    st->dt = dt;
    double* q = ptr<double>(c->q);
    double* qprev = ptr<double>(c->q_prev);
    int rc;
    // prepare: save the node list, qPrev = states, build A and b at the current geometry
    PFG_CUDA(c, cudaMemcpyAsync(c->pos_save.p, c->pos.p, sizeof(double) * c->dim * c->N, cudaMemcpyDeviceToDevice,
                                c->stream));
    PFG_CUDA(c, cudaMemcpyAsync(qprev, q, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = pspg_assemble(c, dt, qprev, qprev, true))) return rc;
    // Picard iterate starts from qPrev for the Krylov initial guess (the reference's direct
    // solve needs none)
    double res = INFINITY;
    int it = 0;
    const int max_iter = c->prm.picard_max_iter;
    const double min_res = c->prm.picard_min_res;
    bool ok = true;
    while (res > min_res) {
        if (it > max_iter) {
            ok = false;
            break;
        }
        int kit = 0;
        double kres = 0;
        if (c->prm.linear_solver == PFG_LINSOLVE_LU) {
            // the reference's choice: a direct factorisation at every Picard iteration
            // (MomContEquationPSPG.inl:281-291); kit counts its refinement sweeps
            if ((rc = lu_solve(c, q, &kit))) return rc;
        } else if ((rc = bicgstab(c, q, &kit, &kres))) {
            return rc;
        }
        st->krylov_iterations += kit;
        if ((rc = pspg_update_positions(c, dt, q))) return rc;
        if (c->prm.residual != PFG_RES_AX_F) {
            // U / U_P residuals compare against the previous iterate (:319-364)
            PFG_CUDA(c, cudaMemcpyAsync(c->q_iter_prev.p, q, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
        }
        if ((rc = pspg_assemble(c, dt, q, qprev, true))) return rc;
        if ((rc = spmv_residual_norm(c, q, &res))) return rc;
        st->residual = res;
        ++it;
        if (std::isnan(res)) {
            ok = false;
            break;
        }
    }
    st->picard_iterations = it;
    if (!ok) {
        // Mesh::restoreNodesList: positions and states revert to the saved node list
        PFG_CUDA(c, cudaMemcpyAsync(c->pos.p, c->pos_save.p, sizeof(double) * c->dim * c->N,
                                    cudaMemcpyDeviceToDevice, c->stream));
        PFG_CUDA(c, cudaMemcpyAsync(q, qprev, sizeof(double) * R, cudaMemcpyDeviceToDevice, c->stream));
    }
    PFG_CUDA(c, cudaStreamSynchronize(c->stream));
    st->converged = ok ? 1 : 0;
    return PFG_OK;
}

}  // namespace pfg
